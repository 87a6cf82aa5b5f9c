"""FP64 CPU restatement of jax-fem's FE layer and weak-form engine (test infrastructure).

Follows jax_fem/fe.py and jax_fem/problem.py function by function; each
function names the reference lines it restates.  Kernels are evaluated with
torch.func on the CPU in float64 (vmap over cells, jacfwd for element
tangents and vjp for parameter gradients), which is the same AD structure the
reference builds with jax.vmap / value_and_jacfwd / jax.vjp.
"""
import numpy as np
import scipy.sparse as sp
import torch

from . import basis

torch.set_default_dtype(torch.float64)


def box_mesh(Nx, Ny, Nz, Lx, Ly, Lz):
    """Structured HEX8 mesh, restating jax_fem/generate_mesh.py:151-189 (meshio corner order)."""
    x = np.linspace(0, Lx, Nx + 1)
    y = np.linspace(0, Ly, Ny + 1)
    z = np.linspace(0, Lz, Nz + 1)
    xv, yv, zv = np.meshgrid(x, y, z, indexing="ij")
    points = np.stack((xv, yv, zv), axis=3).reshape(-1, 3)
    ind = np.arange(len(points)).reshape(Nx + 1, Ny + 1, Nz + 1)
    c = [ind[:-1, :-1, :-1], ind[1:, :-1, :-1], ind[1:, 1:, :-1], ind[:-1, 1:, :-1],
         ind[:-1, :-1, 1:], ind[1:, :-1, 1:], ind[1:, 1:, 1:], ind[:-1, 1:, 1:]]
    cells = np.stack(c, axis=3).reshape(-1, 8)
    return points, cells


def _call_location(fn, points):
    """Evaluate a location function per point, as jax.vmap(location_fn) does (fe.py:241-253)."""
    nargs = fn.__code__.co_argcount
    if nargs == 1:
        return np.array([bool(fn(p)) for p in points])
    if nargs == 2:
        return np.array([bool(fn(p, i)) for i, p in enumerate(points)])
    raise ValueError(f"Wrong number of arguments for location_fn: must be 1 or 2, get {nargs}")


class OracleFE:
    """Restates FiniteElement (fe.py:20-110) for one variable."""

    def __init__(self, points, cells, vec, ele_type="HEX8", quadrature_order=None, dirichlet_bc_info=None):
        self.points = np.asarray(points, dtype=np.float64)
        self.cells = np.asarray(cells, dtype=np.int64)
        self.vec = vec
        self.dim = 3
        self.ele_type = ele_type
        t = basis.element_tables(ele_type, quadrature_order)
        self.__dict__.update(t)
        self.num_cells = len(self.cells)
        self.num_total_nodes = len(self.points)
        self.num_total_dofs = self.num_total_nodes * vec
        self.num_quads = self.shape_vals.shape[0]
        self.num_nodes = self.shape_vals.shape[1]
        self.shape_grads, self.JxW = self.get_shape_grads()
        self.node_inds_list, self.vec_inds_list, self.vals_list = self.Dirichlet_boundary_conditions(dirichlet_bc_info)

    def get_shape_grads(self):
        """fe.py:112-141."""
        X = self.points[self.cells]  # (C, nn, dim)
        Jac = np.einsum("cnd,qne->cqde", X, self.shape_grads_ref)
        det = np.linalg.det(Jac)
        inv = np.linalg.inv(Jac)  # deta_dx
        grads = np.einsum("qne,cqed->cqnd", self.shape_grads_ref, inv)
        return grads, det * self.quad_weights[None, :]

    def get_face_shape_grads(self, boundary_inds):
        """fe.py:143-183: physical face shape grads and Nanson scale."""
        X = self.points[self.cells][boundary_inds[:, 0]]
        fg = self.face_shape_grads_ref[boundary_inds[:, 1]]  # (F, nfq, nn, dim)
        n = self.face_normals[boundary_inds[:, 1]]
        Jac = np.einsum("fnd,fqne->fqde", X, fg)
        det = np.linalg.det(Jac)
        inv = np.linalg.inv(Jac)
        grads = np.einsum("fqne,fqed->fqnd", fg, inv)
        nanson = np.linalg.norm(np.einsum("fe,fqed->fqd", n, inv), axis=-1)
        nanson = nanson * det * self.face_quad_weights[boundary_inds[:, 1]]
        return grads, nanson

    def get_physical_quad_points(self):
        """fe.py:185-197."""
        return np.einsum("qn,cnd->cqd", self.shape_vals, self.points[self.cells])

    def get_physical_surface_quad_points(self, boundary_inds):
        """fe.py:199-218."""
        X = self.points[self.cells][boundary_inds[:, 0]]
        return np.einsum("fqn,fnd->fqd", self.face_shape_vals[boundary_inds[:, 1]], X)

    def Dirichlet_boundary_conditions(self, dirichlet_bc_info):
        """fe.py:220-258."""
        node_inds_list, vec_inds_list, vals_list = [], [], []
        if dirichlet_bc_info is not None:
            location_fns, vecs, value_fns = dirichlet_bc_info
            assert len(location_fns) == len(value_fns) and len(value_fns) == len(vecs)
            for i in range(len(location_fns)):
                node_inds = np.argwhere(_call_location(location_fns[i], self.points)).reshape(-1)
                vec_inds = np.ones_like(node_inds, dtype=np.int32) * vecs[i]
                values = np.array([value_fns[i](p) for p in self.points[node_inds]], dtype=np.float64).reshape(-1)
                node_inds_list.append(node_inds)
                vec_inds_list.append(vec_inds)
                vals_list.append(values)
        return node_inds_list, vec_inds_list, vals_list

    def update_Dirichlet_boundary_conditions(self, dirichlet_bc_info):
        """fe.py:260-269."""
        self.node_inds_list, self.vec_inds_list, self.vals_list = self.Dirichlet_boundary_conditions(dirichlet_bc_info)

    def get_boundary_conditions_inds(self, location_fns):
        """fe.py:271-322: (cell, local face) pairs whose face vertices all satisfy location_fn."""
        out = []
        if location_fns is None:
            return out
        cell_face_nodes = self.cells[:, self.face_inds]  # (C, nf, nfv)
        for fn in location_fns:
            flags = _call_location(fn, self.points)
            # vmap over (cell, face, vertex) of the location function == per-node flag lookup
            # for 1-arg functions; 2-arg functions receive the global node index, as here.
            on = np.all(flags[cell_face_nodes], axis=2)
            out.append(np.argwhere(on))
        return out

    def sol_to_grad(self, sol):
        """fe.py:366-382."""
        return np.einsum("cnv,cqnd->cqvd", sol[self.cells], self.shape_grads)


class OracleProblem:
    """Single-variable restatement of Problem (problem.py:15-460).

    tensor_map(u_grad, *iv_q) -> (vec, dim); mass_map(u, x, *iv_q) -> (vec,);
    surface_maps[i](u, x, *iv_surf) -> (vec,).  All torch, one point at a time.
    universal_kernel(cell_sol_flat, x, cell_shape_grads, cell_JxW, cell_v_grads_JxW, *iv_cell) and
    universal_kernels_surface[i](cell_sol_flat, x, face_shape_vals, face_shape_grads, face_nanson_scale)
    as in problem.py:289-294 and :318-323 (cell_JxW (num_vars, nq), cell_v_grads_JxW (nq, nn, 1, dim),
    face_nanson_scale (num_vars, nfq)), torch, one cell / face at a time.
    """

    def __init__(self, points, cells, vec, ele_type="HEX8", quadrature_order=None, dirichlet_bc_info=None,
                 location_fns=None, tensor_map=None, mass_map=None, surface_maps=None, universal_kernel=None,
                 universal_kernels_surface=None):
        self.fe = OracleFE(points, cells, vec, ele_type, quadrature_order, dirichlet_bc_info)
        self.fes = [self.fe]
        self.vec = vec
        self.dim = 3
        self.num_cells = self.fe.num_cells
        self.num_total_dofs_all_vars = self.fe.num_total_dofs
        self.tensor_map = tensor_map
        self.mass_map = mass_map
        self.surface_maps = surface_maps or []
        self.universal_kernel = universal_kernel
        self.universal_kernels_surface = universal_kernels_surface or []
        self.boundary_inds_list = self.fe.get_boundary_conditions_inds(location_fns)
        if len(self.boundary_inds_list) and not (self.surface_maps or self.universal_kernels_surface):
            raise AssertionError("Missing definitions for surface integral")  # problem.py:340-346
        # COO indices (problem.py:86-107)
        fe = self.fe
        inds = (vec * fe.cells[:, :, None] + np.arange(vec)[None, None, :]).reshape(self.num_cells, -1)
        self.cell_inds = inds
        self.I = np.repeat(inds[:, :, None], inds.shape[1], axis=2).reshape(-1)
        self.J = np.repeat(inds[:, None, :], inds.shape[1], axis=1).reshape(-1)
        self.face_inds_list = []
        for b in self.boundary_inds_list:
            finds = inds[b[:, 0]]
            self.face_inds_list.append(finds)
            self.I = np.hstack((self.I, np.repeat(finds[:, :, None], finds.shape[1], axis=2).reshape(-1)))
            self.J = np.hstack((self.J, np.repeat(finds[:, None, :], finds.shape[1], axis=1).reshape(-1)))
        # geometry (problem.py:130-182)
        self.shape_grads = torch.from_numpy(fe.shape_grads)
        self.JxW = torch.from_numpy(fe.JxW)
        self.v_grads_JxW = self.shape_grads * self.JxW[:, :, None, None]
        self.physical_quad_points = torch.from_numpy(fe.get_physical_quad_points())
        self.shape_vals = torch.from_numpy(fe.shape_vals)
        self.face_data = []
        for b in self.boundary_inds_list:
            fgrads, nanson = fe.get_face_shape_grads(b)
            self.face_data.append(dict(
                vals=torch.from_numpy(fe.face_shape_vals[b[:, 1]]),
                grads=torch.from_numpy(fgrads),
                nanson=torch.from_numpy(nanson),
                x=torch.from_numpy(fe.get_physical_surface_quad_points(b)),
                cells=b[:, 0]))
        self.internal_vars = ()
        self.internal_vars_surfaces = [() for _ in self.boundary_inds_list]

    # ---- kernels (problem.py:189-303) -----------------------------------------
    def _cell_kernel(self, u_flat, grads, vgjxw, x, jxw, *iv):
        u = u_flat.reshape(self.fe.num_nodes, self.vec)
        val = torch.zeros_like(u)
        if self.tensor_map is not None:
            u_grads = torch.einsum("nv,qnd->qvd", u, grads)
            sig = torch.func.vmap(self.tensor_map)(u_grads, *iv)
            val = val + torch.einsum("qvd,qnd->nv", sig, vgjxw)
        if self.mass_map is not None:
            uq = torch.einsum("nv,qn->qv", u, self.shape_vals)
            m = torch.func.vmap(self.mass_map)(uq, x, *iv)
            val = val + torch.einsum("qv,qn,q->nv", m, self.shape_vals, jxw)
        if self.universal_kernel is not None:   # problem.py:289-294
            val = val + self.universal_kernel(u_flat, x, grads, jxw[None, :], vgjxw[:, :, None, :],
                                              *iv).reshape(u.shape)
        return val.reshape(-1)

    def _face_kernel(self, fn, ufn, u_flat, fvals, fgrads, nanson, x, *iv):
        u = u_flat.reshape(self.fe.num_nodes, self.vec)
        val = torch.zeros_like(u_flat)
        if fn is not None:
            uq = torch.einsum("nv,qn->qv", u, fvals)
            t = torch.func.vmap(fn)(uq, x, *iv)
            val = val + torch.einsum("qv,qn,q->nv", t, fvals, nanson).reshape(-1)
        if ufn is not None:                      # problem.py:318-323
            val = val + ufn(u_flat, x, fvals, fgrads, nanson[None, :]).reshape(-1)
        return val

    def _cells_sol(self, dofs):
        return dofs[torch.from_numpy(self.cell_inds)]

    def weak_form(self, dofs, internal_vars, internal_vars_surfaces, jac=False):
        """Per-cell values (and jacfwd tangents) -- problem.py:359-424."""
        cs = self._cells_sol(dofs)
        args = (cs, self.shape_grads, self.v_grads_JxW, self.physical_quad_points, self.JxW, *internal_vars)
        if jac:
            f = torch.func.vmap(torch.func.jacfwd(self._cell_kernel))
            cell_jac = f(*args)
        else:
            cell_jac = None
        cell_val = torch.func.vmap(self._cell_kernel)(*args)
        faces = []
        for i, fd in enumerate(self.face_data):
            fn = self.surface_maps[i] if i < len(self.surface_maps) else None
            ufn = self.universal_kernels_surface[i] if i < len(self.universal_kernels_surface) else None
            fargs = (cs[fd["cells"]], fd["vals"], fd["grads"], fd["nanson"], fd["x"], *internal_vars_surfaces[i])
            k = lambda *a, fn=fn, ufn=ufn: self._face_kernel(fn, ufn, *a)
            fval = torch.func.vmap(k)(*fargs)
            fjac = torch.func.vmap(torch.func.jacfwd(k))(*fargs) if jac else None
            faces.append((fval, fjac))
        return cell_val, cell_jac, faces

    def residual_from_weak(self, cell_val, faces):
        """compute_residual_vars_helper, problem.py:426-437 (scatter-add)."""
        res = torch.zeros(self.num_total_dofs_all_vars, dtype=cell_val.dtype)
        res = res.index_add(0, torch.from_numpy(self.cell_inds.reshape(-1)), cell_val.reshape(-1))
        for (fval, _), finds in zip(faces, self.face_inds_list):
            res = res.index_add(0, torch.from_numpy(finds.reshape(-1)), fval.reshape(-1))
        return res

    def compute_residual(self, dofs, internal_vars=None, internal_vars_surfaces=None):
        """problem.py:462-475 (flattened)."""
        iv = self.internal_vars if internal_vars is None else internal_vars
        ivs = self.internal_vars_surfaces if internal_vars_surfaces is None else internal_vars_surfaces
        cv, _, faces = self.weak_form(dofs, iv, ivs, jac=False)
        return self.residual_from_weak(cv, faces)

    def newton_update(self, dofs):
        """problem.py:447-460: residual and COO values V."""
        cv, cj, faces = self.weak_form(torch.as_tensor(dofs), self.internal_vars, self.internal_vars_surfaces, jac=True)
        V = [cj.reshape(-1)]
        for (_, fj) in faces:
            V.append(fj.reshape(-1))
        self.V = torch.cat(V).numpy()
        return self.residual_from_weak(cv, faces)

    # ---- BC helpers (solver.py:290-363) -----------------------------------------
    def bc_rows(self):
        fe = self.fe
        if not fe.node_inds_list:
            return np.zeros(0, dtype=np.int64), np.zeros(0)
        rows = np.concatenate([n * fe.vec + v for n, v in zip(fe.node_inds_list, fe.vec_inds_list)])
        vals = np.concatenate(fe.vals_list)
        return rows.astype(np.int64), vals


def coo_pattern(I, J, n):
    """PETSc COO preallocation pattern (solver.py:474-478): sorted unique (I,J) as CSR."""
    A = sp.coo_matrix((np.ones(len(I)), (I, J)), shape=(n, n)).tocsr()
    A.sum_duplicates()
    A.sort_indices()
    return A.indptr.astype(np.int64), A.indices.astype(np.int64)


def assemble_petsc(problem, V=None):
    """_PetscTangentCache.update (solver.py:522-529): setValuesCOO sums duplicates onto the
    COO-preallocated pattern, assemble, then zeroRows(bc rows) -- row := 0, diagonal := 1.0,
    pattern kept (KEEP_NONZERO_PATTERN, solver.py:477)."""
    n = problem.num_total_dofs_all_vars
    V = problem.V if V is None else V
    indptr, indices = coo_pattern(problem.I, problem.J, n)
    rows_p = np.repeat(np.arange(n, dtype=np.int64), np.diff(indptr))
    key_p = rows_p * n + indices
    key_v = problem.I.astype(np.int64) * n + problem.J.astype(np.int64)
    pos = np.searchsorted(key_p, key_v)
    data = np.bincount(pos, weights=V, minlength=len(indices))
    rows, _ = problem.bc_rows()
    for r in np.unique(rows):
        s, e = indptr[r], indptr[r + 1]
        data[s:e] = 0.0
        data[s + np.searchsorted(indices[s:e], r)] = 1.0
    return sp.csr_matrix((data, indices, indptr), shape=(n, n))


def apply_bc_vec(res, dofs, problem, scale=1.0):
    """solver.py:290-304: res[bc] = dofs[bc] - vals*scale."""
    res = np.array(res, dtype=np.float64, copy=True)
    fe = problem.fe
    for n, v, val in zip(fe.node_inds_list, fe.vec_inds_list, fe.vals_list):
        r = n * fe.vec + v
        res[r] = np.asarray(dofs)[r]
        res[r] -= val * scale
    return res


def assign_bc(dofs, problem):
    """solver.py:316-324."""
    dofs = np.array(dofs, dtype=np.float64, copy=True)
    fe = problem.fe
    for n, v, val in zip(fe.node_inds_list, fe.vec_inds_list, fe.vals_list):
        dofs[n * fe.vec + v] = val
    return dofs


def copy_bc(dofs, problem):
    """solver.py:349-363."""
    out = np.zeros_like(np.asarray(dofs, dtype=np.float64))
    fe = problem.fe
    for n, v in zip(fe.node_inds_list, fe.vec_inds_list):
        r = n * fe.vec + v
        out[r] = np.asarray(dofs)[r]
    return out
