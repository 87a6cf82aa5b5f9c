"""Device-side state of a Problem and thin wrappers over the C ABI.

One Engine per Problem owns every device buffer of the hot path: mesh,
node-block sparsity pattern, per-cell slot table, external load vector,
Dirichlet arrays, matrix values (FP64 and/or FP32), preconditioners and the
Krylov workspaces.  All work is enqueued on torch's current CUDA stream via
the C ABI; torch is used only for memory and a few O(#dofs) bookkeeping ops.
"""
import ctypes as C
import time

import numpy as np
import torch

from . import _lib
from ._lib import call, ptr
from .logger import logger


def structured_grid(points, rtol=1e-9):
    """(nx, ny, nz) node counts when node n sits at grid point (i, j, k) of a tensor-product grid
    with n = (i*ny + j)*nz + k -- x slowest, z fastest, the numbering of box_mesh
    (jax_fem/generate_mesh.py:151-189) -- else None.  Coordinates are compared to the grid lines
    within rtol of the box size; the converter to the structured storage then checks every node
    row's pattern against the grid's stencil."""
    P = np.asarray(points, dtype=np.float64)
    N = len(P)
    if N < 2 or P.shape[1] != 3:
        return None
    tol = rtol * max(float(np.ptp(P, axis=0).max()), 1e-300)
    moved_xy = np.nonzero((np.abs(P[:, 0] - P[0, 0]) > tol) | (np.abs(P[:, 1] - P[0, 1]) > tol))[0]
    nz = int(moved_xy[0]) if len(moved_xy) else N
    moved_x = np.nonzero(np.abs(P[:, 0] - P[0, 0]) > tol)[0]
    nyz = int(moved_x[0]) if len(moved_x) else N
    if nz < 1 or nyz % nz or N % nyz:
        return None
    ny, nx = nyz // nz, N // nyz
    G = P.reshape(nx, ny, nz, 3)
    if not (np.all(np.abs(G[:, :, :, 0] - G[:, :1, :1, 0]) <= tol) and
            np.all(np.abs(G[:, :, :, 1] - G[:1, :, :1, 1]) <= tol) and
            np.all(np.abs(G[:, :, :, 2] - G[:1, :1, :, 2]) <= tol)):
        return None
    for ax, n in ((0, nx), (1, ny), (2, nz)):
        line = G[:, 0, 0, 0] if ax == 0 else G[0, :, 0, 1] if ax == 1 else G[0, 0, :, 2]
        if n > 1 and not np.all(np.diff(line) > tol):
            return None
    return nx, ny, nz


def _stream():
    return _lib.stream_handle()


class DeviceCSR:
    """Assembled global matrix on the device (scalar CSR values, node-block column indices).

    Stands where the reference passes a PETSc Mat (jax_fem/solver.py:540-553)."""

    def __init__(self, eng, precision, vals, bc_mode, source=None):
        self.eng = eng
        self.precision = precision
        self.data = vals
        self.bc_mode = bc_mode
        self.source = source          # FP64 matrix a DF48 matrix was split from
        self.ref64 = None             # the same FP64 values, sliced (DF48 copies: reliable updates)
        n = eng.num_dofs
        self.shape = (n, n)
        self.nnz = eng.nnz
        self.pc = {}

    @property
    def dtype(self):
        return self.data.dtype

    @property
    def indptr(self):
        return self.eng.indptr

    @property
    def indices(self):
        return self.eng.scalar_indices()

    def matvec(self, x):
        if self.precision in (_lib.FEM_SYM_DF48, _lib.FEM_SSYM_DF48):
            return self._matvec_dfx(x)
        if self.precision in (_lib.FEM_DF48, _lib.FEM_SLICED_DF48):
            x = x.to(torch.float64).contiguous()
            xs = torch.empty(2 * x.numel(), dtype=torch.float32, device=x.device)
            call("fem_vector_split", ptr(x), x.numel(), ptr(xs), _stream())
            y = torch.empty_like(x)
            call("fem_spmv", C.byref(self.eng.pattern), self.eng.num_nodes, self.eng.vec, self.precision,
                 ptr(self.data), ptr(xs), ptr(y), _stream())
            return y
        x = x.to(self.vector_dtype).contiguous()
        y = torch.empty_like(x)
        call("fem_spmv", C.byref(self.eng.pattern), self.eng.num_nodes, self.eng.vec, self.precision,
             ptr(self.data), ptr(x), ptr(y), _stream())
        return y

    def _matvec_dfx(self, x):
        """fem_spmv_dfx on a node-interleaved double-float copy of x (FP64 result)."""
        eng = self.eng
        x = x.to(torch.float64).reshape(-1)
        pad = 4 if eng.vec == 3 else 1
        hi = x.float()
        xp = torch.zeros(eng.num_nodes, pad, 2, dtype=torch.float32, device=x.device)
        xp[:, :eng.vec, 0] = hi.view(-1, eng.vec)
        xp[:, :eng.vec, 1] = (x - hi.double()).float().view(-1, eng.vec)
        yh = torch.empty(eng.num_dofs, dtype=torch.float32, device=x.device)
        yl = torch.empty_like(yh)
        ws = eng.workspace(_lib.FEM_SLICED_DF48)
        call("fem_spmv_dfx", C.byref(eng.pattern), eng.num_nodes, eng.vec, self.precision, ptr(self.data), ptr(xp),
             ptr(yh), ptr(yl), None, ptr(ws), ws.numel(), _stream())
        return yh.double() + yl.double()

    __matmul__ = matvec

    def transpose(self):
        """A^T in the same CSR pattern (FP32 / FP64 CSR order), as the reference's PETSc
        A.transpose() before the adjoint solve (solver.py:1405-1409)."""
        if self.precision not in (_lib.FEM_F32, _lib.FEM_F64):
            raise ValueError("transpose() works on FP32 / FP64 CSR matrices")
        out = torch.empty_like(self.data)
        ws = self.eng.workspace(_lib.FEM_F64)
        call("fem_matrix_transpose", C.byref(self.eng.pattern), self.eng.num_nodes, self.eng.vec, self.precision,
             ptr(self.data), ptr(out), ptr(ws), ws.numel(), _stream())
        return DeviceCSR(self.eng, self.precision, out, self.bc_mode)

    @property
    def vector_dtype(self):
        return torch.float32 if self.precision in (_lib.FEM_F32, _lib.FEM_SLICED_F32) else torch.float64

    def diagonal(self):
        if self.source is not None:
            return self.source.diagonal()
        return self.data[self.eng.diag]

    def preconditioner(self, kind):
        if kind == _lib.FEM_PC_NONE:
            return None
        if self.source is not None:
            # preconditioner of a derived (sliced / DF48) matrix, set up from its FP64 CSR source;
            # FP64 for FP64 solver copies, FP32 otherwise
            if kind not in self.pc:
                pc64 = self.source.preconditioner(kind)
                if self.precision == _lib.FEM_SLICED_F64:
                    self.pc[kind] = pc64
                    return pc64
                pc = torch.empty(pc64.numel(), dtype=torch.float32, device=pc64.device)
                call("fem_cast_f64_f32", ptr(pc64), ptr(pc), pc64.numel(), None, _stream())
                self.pc[kind] = pc
            return self.pc[kind]
        if kind not in self.pc:
            n = self.eng.num_dofs if kind == _lib.FEM_PC_JACOBI else self.eng.num_nodes * self.eng.vec ** 2
            buf = torch.empty(n, dtype=self.data.dtype, device=self.data.device)
            call("fem_precond_setup", C.byref(self.eng.pattern), self.eng.num_nodes, self.eng.vec, self.precision,
                 ptr(self.data), kind, ptr(buf), _stream())
            self.pc[kind] = buf
        return self.pc[kind]

    def to_torch(self):
        """torch sparse CSR view (debugging / custom solvers)."""
        return torch.sparse_csr_tensor(self.indptr, self.indices.to(torch.int64), self.data, size=self.shape)

    # PETSc Mat methods used by the reference's custom_solver plug-ins (solver.py:278-280; the
    # documented example converts with A.getValuesCSR() / A.getSize())
    def getValuesCSR(self):
        """(indptr, indices, data) host arrays of the FP64 values (int32 indices as PETSc)."""
        src = self if self.source is None else self.source
        return (src.indptr.cpu().numpy().astype(np.int32), src.indices.cpu().numpy().astype(np.int32),
                src.data.double().cpu().numpy())

    def getSize(self):
        return self.shape

    def to_scipy(self):
        """Host copy as scipy CSR (for user code and tests only)."""
        import scipy.sparse as sp
        return sp.csr_matrix((self.data.double().cpu().numpy(), self.indices.cpu().numpy(),
                              self.indptr.cpu().numpy()), shape=self.shape)


class Engine:
    def __init__(self, problem, device="cuda"):
        if not torch.cuda.is_available():
            raise RuntimeError("jax_fem_gb300 runs on a CUDA GPU (sm_103a); no GPU is visible")
        _lib.load()
        self.problem = problem
        fe = problem.fes[0]
        self.fe = fe
        self.device = torch.device(device)
        self.vec = fe.vec
        self.num_nodes = fe.num_total_nodes
        self.num_cells = fe.num_cells
        self.num_quads = fe.num_quads
        self.nn = fe.num_nodes
        self.num_dofs = self.num_nodes * self.vec
        self.timing = {"local_assembly": 0.0, "global_matrix": 0.0, "linear": 0.0, "adjoint": 0.0}
        self.solve_log = []
        self.sync_timing = True
        dev = self.device
        self.coords = torch.as_tensor(fe.points, dtype=torch.float64, device=dev).contiguous()
        self.conn = torch.as_tensor(fe.cells, dtype=torch.int32, device=dev).contiguous()
        self.mesh = _lib.FemMesh(fe.elem_id, self.vec, self.num_nodes, self.num_cells,
                                 self.coords.data_ptr(), self.conn.data_ptr(), None, None)
        self._build_geometry()
        self._build_pattern()
        self._bc_seen = None
        self.bc_value_terms = []
        self._mat = None
        self._mat_key = None
        self._qp = None
        self._hist = None
        self._tangent_cache = {}
        self._ws = {}
        self.f_ext = torch.zeros(self.num_dofs, dtype=torch.float64, device=dev)
        self._loads_done = False
        self._robin = []            # (face_cells, face_ids, degree, coeffs) of u-dependent surface maps
        self._uk = None             # compiled universal kernels (get_universal_kernel[s_surface])
        self._uk_key = None

    def _build_geometry(self):
        """Physical shape gradients and JxW of every cell and quadrature point, computed once on the
        device and kept, as the reference keeps fe.shape_grads / fe.JxW (problem.py:130-147); the
        cell kernels then read them instead of recomputing the Jacobians on the FP64 pipe.  Kept
        only while it takes at most a quarter of the free device memory (1.6 GB per 1M HEX8 cells);
        otherwise the kernels recompute the geometry."""
        self.shape_grads = self.jxw = None
        n = self.num_cells * self.num_quads
        need = n * (self.nn * 3 + 1) * 8
        if n == 0 or need > torch.cuda.mem_get_info(self.device)[0] // 4:
            return
        self.shape_grads = torch.empty(n * self.nn * 3, dtype=torch.float64, device=self.device)
        self.jxw = torch.empty(n, dtype=torch.float64, device=self.device)
        call("fem_cell_geometry", C.byref(self.mesh), ptr(self.shape_grads), ptr(self.jxw), _stream())
        self.mesh.shape_grads = self.shape_grads.data_ptr()
        self.mesh.jxw = self.jxw.data_ptr()

    def add_robin(self, boundary_inds, coeffs):
        """Register the u-dependent polynomial part of a surface map on the faces boundary_inds."""
        bi = np.asarray(boundary_inds)
        fc = torch.as_tensor(bi[:, 0].astype(np.int32), device=self.device)
        fi = torch.as_tensor(bi[:, 1].astype(np.int32), device=self.device)
        co = np.ascontiguousarray(np.asarray(coeffs, dtype=np.float64))
        self._robin.append((fc, fi, co.shape[1] - 1, co))
        self._tangent_cache.clear()

    @property
    def robin_linear(self):
        return all(deg <= 1 for _, _, deg, _ in self._robin)

    def _robin_call(self, outputs, precision, dofs, w=None, bc_mode=_lib.FEM_BC_NONE, bc=None, res=None, vals=None,
                    apply_out=None):
        for fc, fi, deg, co in self._robin:
            call("fem_surface_robin", C.byref(self.mesh), C.byref(self.pattern), ptr(fc), ptr(fi), fc.numel(), deg,
                 co.ctypes.data_as(C.POINTER(C.c_double)), outputs, precision, ptr(dofs), ptr(w), ptr(bc), bc_mode,
                 ptr(res), ptr(vals), ptr(apply_out), _stream())

    # ---- pattern -------------------------------------------------------------------
    def _build_pattern(self):
        dev, s = self.device, _stream()
        elem = self.fe.elem_id
        nb = C.c_size_t()
        call("fem_pattern_workspace", self.num_cells, self.nn, self.num_nodes, C.byref(nb))
        ws = torch.empty(nb.value, dtype=torch.uint8, device=dev)
        self.block_ptr = torch.empty(self.num_nodes + 1, dtype=torch.int64, device=dev)
        nnzb = C.c_int64()
        call("fem_pattern_count", elem, ptr(self.conn), self.num_cells, self.num_nodes, ptr(ws), nb.value,
             ptr(self.block_ptr), C.byref(nnzb), s)
        self.nnzb = nnzb.value
        self.block_cols = torch.empty(self.nnzb, dtype=torch.int32, device=dev)
        call("fem_pattern_fill", elem, ptr(self.conn), self.num_cells, self.num_nodes, ptr(ws), nb.value,
             ptr(self.block_ptr), ptr(self.block_cols), s)
        del ws
        self.slots = torch.empty(self.num_cells * self.nn * self.nn, dtype=torch.uint8, device=dev)
        call("fem_pattern_slots", elem, ptr(self.conn), self.num_cells, ptr(self.block_ptr), ptr(self.block_cols),
             ptr(self.slots), s)
        self.indptr = torch.empty(self.num_dofs + 1, dtype=torch.int64, device=dev)
        self.diag = torch.empty(self.num_dofs, dtype=torch.int64, device=dev)
        call("fem_pattern_scalar", self.num_nodes, self.vec, ptr(self.block_ptr), ptr(self.block_cols),
             ptr(self.indptr), ptr(self.diag), None, s)
        self.nnz = self.nnzb * self.vec * self.vec
        # node grid of a structured box numbering (the grid layout below and the FEM_SSYM_DF48
        # solver copy), vec 3 and elements whose nodes couple only grid neighbours
        self.grid = structured_grid(self.fe.points) if self.vec == 3 and self.fe.ele_type in ("HEX8", "TET4") \
            else None
        # sliced layout (32 node rows per slice) of the solver copies of the matrix: on the node grid
        # 27 stencil slots per slice whose columns follow from the grid, else each row's blocks in order
        self.n_slices = (self.num_nodes + 31) // 32
        self.slice_ptr = torch.empty(self.n_slices + 1, dtype=torch.int64, device=dev)
        self.slices_grid = False
        if self.grid is not None:
            self.n_slots = 27 * self.n_slices
            self.slice_cols = torch.empty(self.n_slots * 32, dtype=torch.int32, device=dev)
            try:
                call("fem_pattern_slices_grid", self.num_nodes, ptr(self.block_ptr), ptr(self.block_cols),
                     *self.grid, ptr(self.slice_ptr), ptr(self.slice_cols), s)
                self.slices_grid = True
            except _lib.FemError as exc:
                logger.info("grid slice layout refused (%s); general sliced layout", exc)
        if not self.slices_grid:
            n_slots = C.c_int64()
            call("fem_pattern_slices", self.num_nodes, ptr(self.block_ptr), ptr(self.block_cols), ptr(self.slice_ptr),
                 None, C.byref(n_slots), s)
            self.n_slots = n_slots.value
            self.slice_cols = torch.empty(self.n_slots * 32, dtype=torch.int32, device=dev)
            call("fem_pattern_slices", self.num_nodes, ptr(self.block_ptr), ptr(self.block_cols), ptr(self.slice_ptr),
                 ptr(self.slice_cols), None, s)
        # upper node blocks only: the symmetric DF48 solver copy (FEM_SYM_DF48)
        self.slice_ptr_u = torch.empty(self.n_slices + 1, dtype=torch.int64, device=dev)
        n_slots_u = C.c_int64()
        call("fem_pattern_slices_upper", self.num_nodes, ptr(self.block_ptr), ptr(self.block_cols),
             ptr(self.slice_ptr_u), None, C.byref(n_slots_u), s)
        self.n_slots_u = n_slots_u.value
        self.slice_cols_u = torch.empty(self.n_slots_u * 32, dtype=torch.int32, device=dev)
        call("fem_pattern_slices_upper", self.num_nodes, ptr(self.block_ptr), ptr(self.block_cols),
             ptr(self.slice_ptr_u), ptr(self.slice_cols_u), None, s)
        gx, gy, gz = self.grid if self.grid is not None else (0, 0, 0)
        self.pattern = _lib.FemPattern(self.nnzb, self.block_ptr.data_ptr(), self.block_cols.data_ptr(),
                                       self.indptr.data_ptr(), self.diag.data_ptr(), self.slots.data_ptr(),
                                       self.n_slices, self.n_slots, self.slice_ptr.data_ptr(),
                                       self.slice_cols.data_ptr(), self.n_slots_u, self.slice_ptr_u.data_ptr(),
                                       self.slice_cols_u.data_ptr(), gx, gy, gz, int(self.slices_grid))
        self._indices = None

    def scalar_indices(self):
        if self._indices is None:
            self._indices = torch.empty(self.nnz, dtype=torch.int32, device=self.device)
            call("fem_pattern_scalar", self.num_nodes, self.vec, ptr(self.block_ptr), ptr(self.block_cols),
                 None, None, ptr(self._indices), _stream())
        return self._indices

    # ---- Dirichlet arrays ---------------------------------------------------------
    def refresh_bc(self):
        fe = self.fe
        key = (fe.bc_version, id(fe.node_inds_list), id(fe.vals_list))
        if key == self._bc_seen:
            return
        rows, vals, graph = [], [], []
        for n, v, val in zip(fe.node_inds_list, fe.vec_inds_list, fe.vals_list):
            rows.append(np.asarray(n, dtype=np.int64) * fe.vec + np.asarray(v, dtype=np.int64))
            if torch.is_tensor(val):
                if val.requires_grad:
                    graph.append((len(vals), val))
                val = val.detach().cpu().numpy()
            vals.append(np.asarray(val, dtype=np.float64))
        # Dirichlet values that carry a torch graph (differentiable set_params): (positions in
        # the final bc_rows, tensor entries) -- the adjoint sends lam_b to them
        self.bc_value_terms = []
        if rows:
            offs = np.concatenate([[0], np.cumsum([len(r) for r in rows])])
            rows = np.concatenate(rows)
            vals = np.concatenate(vals)
            # later lists overwrite earlier ones on shared rows (solver.py:297-300): keep the last
            _, last = np.unique(rows[::-1], return_index=True)
            keep = np.sort(len(rows) - 1 - last)
            rows, vals = rows[keep], vals[keep]
            for li, t in graph:
                c = np.arange(offs[li], offs[li + 1])
                kept = np.isin(c, keep)
                if kept.any():
                    pos = np.searchsorted(keep, c[kept])
                    self.bc_value_terms.append((torch.as_tensor(pos, device=self.device),
                                                t[torch.as_tensor(np.nonzero(kept)[0], device=t.device)]))
        else:
            rows, vals = np.zeros(0, dtype=np.int64), np.zeros(0)
        dev = self.device
        self.bc_rows = torch.as_tensor(rows.astype(np.int32), device=dev)
        self.bc_rows_long = self.bc_rows.to(torch.int64)
        self.bc_vals = torch.as_tensor(vals, device=dev)
        mask = torch.zeros(self.num_dofs, dtype=torch.uint8, device=dev)
        if len(rows):
            mask[self.bc_rows_long] = 1
        self.bc_mask = mask
        self.n_bc = len(rows)
        self._bc_seen = key
        self._tangent_cache.clear()

    @property
    def tangent_symmetric(self):
        """Whether K(u) is symmetric: the material's tangent (Robin parts are symmetric)."""
        m, _ = self.material()
        return bool(m.symmetric) and not self.has_universal   # a compiled user kernel may be non-symmetric

    # ---- external loads (mass / surface maps independent of u) -----------------------
    def refresh_loads(self):
        if self._loads_done:
            return
        p = self.problem
        f = torch.zeros(self.num_dofs, dtype=torch.float64, device=self.device)
        s = _stream()
        if p._body_force is not None:
            fq = torch.as_tensor(p._body_force, dtype=torch.float64, device=self.device).contiguous()
            call("fem_body_load", C.byref(self.mesh), ptr(fq), ptr(f), s)
        for bi, t in zip(p.boundary_inds_list, p._surface_tractions):
            if t is None or len(bi) == 0:
                continue
            fc = torch.as_tensor(bi[:, 0].astype(np.int32), device=self.device)
            fid = torch.as_tensor(bi[:, 1].astype(np.int32), device=self.device)
            tq = torch.as_tensor(t, dtype=torch.float64, device=self.device).contiguous()
            call("fem_surface_load", C.byref(self.mesh), ptr(fc), ptr(fid), len(bi), ptr(tq), ptr(f), s)
        self.f_ext = f
        self._loads_done = True

    def quad_points(self):
        x = torch.empty(self.num_cells * self.num_quads * 3, dtype=torch.float64, device=self.device)
        jxw = torch.empty(self.num_cells * self.num_quads, dtype=torch.float64, device=self.device)
        call("fem_quad_points", C.byref(self.mesh), ptr(x), ptr(jxw), _stream())
        return x.reshape(self.num_cells, self.num_quads, 3), jxw.reshape(self.num_cells, self.num_quads)

    def face_quad_points(self, boundary_inds):
        bi = np.asarray(boundary_inds)
        nfq = self.fe.num_face_quads
        x = torch.empty(len(bi) * nfq * 3, dtype=torch.float64, device=self.device)
        nan = torch.empty(len(bi) * nfq, dtype=torch.float64, device=self.device)
        if len(bi):
            fc = torch.as_tensor(bi[:, 0].astype(np.int32), device=self.device)
            fid = torch.as_tensor(bi[:, 1].astype(np.int32), device=self.device)
            call("fem_face_quad_points", C.byref(self.mesh), ptr(fc), ptr(fid), len(bi), ptr(x), ptr(nan), _stream())
        return x.reshape(len(bi), nfq, 3), nan.reshape(len(bi), nfq)

    # ---- material ------------------------------------------------------------------
    def material(self):
        p = self.problem
        if self._mat is None:
            self._mat = p._resolve_material()
        m = self._mat
        key = (p._params_version,)
        if key != self._mat_key:
            qp, hist = m.bind(p.internal_vars, self.num_cells, self.num_quads, self.device)
            same = (self._mat_key is not None and hist is None and getattr(self, "_hist", None) is None and
                    ((qp is None and self._qp is None) or
                     (qp is not None and self._qp is not None and torch.equal(qp, self._qp))))
            consts = m.consts()
            self._consts = (C.c_double * max(1, len(consts)))(*consts)
            self._qp, self._hist = qp, hist
            self._mat_struct = _lib.FemMaterial(m.kind, len(consts), self._consts, m.n_qp_params,
                                                None if qp is None else qp.data_ptr(),
                                                None if hist is None else hist.data_ptr())
            self._mat_key = key
            if not same:
                self._tangent_cache.clear()
        return m, self._mat_struct

    # ---- kernels -------------------------------------------------------------------
    def residual(self, dofs, apply_bc=True, out=None):
        """R(u) = R_int(u) + f_ext, BC rows replaced by u_b - g (apply_bc_vec, solver.py:290-304)."""
        self.refresh_loads()
        _, ms = self.material()
        res = out if out is not None else torch.empty(self.num_dofs, dtype=torch.float64, device=self.device)
        res.copy_(self.f_ext)
        dofs = dofs.contiguous()
        call("fem_assemble", C.byref(self.mesh), C.byref(ms), C.byref(self.pattern), _lib.FEM_OUT_RESIDUAL,
             _lib.FEM_F64, ptr(dofs), None, None, _lib.FEM_BC_NONE, ptr(res), None, None, _stream())
        if self._robin:
            self._robin_call(_lib.FEM_OUT_RESIDUAL, _lib.FEM_F64, dofs, res=res)
        if self.has_universal:
            self._universal_call(_lib.FEM_OUT_RESIDUAL, dofs, res=res)
        if apply_bc:
            self.refresh_bc()
            if self.n_bc:
                call("fem_apply_bc_vec", ptr(res), ptr(dofs), ptr(self.bc_rows), ptr(self.bc_vals), self.n_bc, 1.0,
                     _stream())
        return res

    def tangent(self, dofs, precision, bc_mode, cache=True, df_source=False):
        """Assemble K(u) in `precision` with Dirichlet handling `bc_mode` and unit BC diagonal.
        The DF48 solver copies are split from an FP64 CSR tangent that the isotropic laws assemble
        in double-float arithmetic (fem_assemble with FEM_DF48: FP64 values accurate to ~2^-46,
        beyond what the 40-bit copy keeps); df_source asks for that FP64 CSR itself.  The FP64
        path's own tangent (precision FEM_F64) is always assembled in FP64."""
        self.refresh_bc()
        m, ms = self.material()
        if precision == _lib.FEM_SSYM_DF48 and (self.grid is None or bc_mode != _lib.FEM_BC_SYMMETRIC):
            precision = _lib.FEM_SLICED_DF48      # no structured copy for this mesh / elimination
        df_source = df_source and precision == _lib.FEM_F64
        key = (precision, bc_mode, "df") if df_source else (precision, bc_mode)
        if cache and m.linear and self.robin_linear and not self.has_universal and key in self._tangent_cache:
            return self._tangent_cache[key]
        if precision not in (_lib.FEM_F32, _lib.FEM_F64):
            # solver copies (DF48, sliced FP32 / FP64 / DF48) are converted from the FP64 CSR tangent
            df_copy = precision in (_lib.FEM_DF48, _lib.FEM_SLICED_DF48, _lib.FEM_SYM_DF48, _lib.FEM_SSYM_DF48)
            A64 = self.tangent(dofs, _lib.FEM_F64, bc_mode, cache=cache, df_source=df_copy)
            nb = C.c_size_t()
            call("fem_matrix_bytes", C.byref(self.pattern), self.vec, precision, C.byref(nb))
            name = f"valsx{precision}_{bc_mode}"
            buf = getattr(self, name, None)
            if buf is None or buf.numel() != nb.value:
                buf = torch.empty(nb.value, dtype=torch.uint8, device=self.device)
                setattr(self, name, buf)
            try:
                call("fem_matrix_convert", C.byref(self.pattern), self.num_nodes, self.vec, ptr(A64.data), precision,
                     ptr(buf), _stream())
            except _lib.FemError as exc:
                if precision != _lib.FEM_SSYM_DF48:
                    raise
                # the node pattern is not the grid's stencil (the converter checked every row):
                # no structured copy for this mesh, the general sliced layout instead
                logger.info("structured symmetric storage refused (%s); sliced DF48 instead", exc)
                self.grid = None
                if not self.slices_grid:     # the grid sliced layout still reads the node grid
                    self.pattern.grid_nx = self.pattern.grid_ny = self.pattern.grid_nz = 0
                return self.tangent(dofs, _lib.FEM_SLICED_DF48, bc_mode, cache=cache)
            view = buf.view(torch.float64) if precision == _lib.FEM_SLICED_F64 else \
                buf.view(torch.float32) if precision == _lib.FEM_SLICED_F32 else buf
            A = DeviceCSR(self, precision, view, bc_mode, source=A64)
            if df_copy and bc_mode == _lib.FEM_BC_SYMMETRIC and self.pattern.n_slices > 0:
                A.ref64 = self._sliced_reference(A64, bc_mode)
            self._tangent_cache[key] = A
            return A
        dtype = torch.float32 if precision == _lib.FEM_F32 else torch.float64
        buf_name = f"vals{precision}_{bc_mode}" + ("df" if df_source else "")
        vals = getattr(self, buf_name, None)
        if vals is None:
            vals = torch.empty(self.nnz, dtype=dtype, device=self.device)
            setattr(self, buf_name, vals)
        vals.zero_()
        dofs = dofs.contiguous()
        call("fem_assemble", C.byref(self.mesh), C.byref(ms), C.byref(self.pattern), _lib.FEM_OUT_MATRIX,
             _lib.FEM_DF48 if df_source else precision, ptr(dofs), None, ptr(self.bc_mask), bc_mode, None,
             ptr(vals), None, _stream())
        if self._robin:
            self._robin_call(_lib.FEM_OUT_MATRIX, precision, dofs, bc_mode=bc_mode, bc=self.bc_mask, vals=vals)
        if self.has_universal:
            if precision != _lib.FEM_F64:
                raise NotImplementedError("universal kernels assemble FP64 tangents (the solver copies are "
                                          "converted from them)")
            self._universal_call(_lib.FEM_OUT_MATRIX, dofs, bc=self.bc_mask if bc_mode != _lib.FEM_BC_NONE else None,
                                 bc_mode=bc_mode, vals=vals)
        if bc_mode != _lib.FEM_BC_NONE and self.n_bc:
            call("fem_zero_rows", C.byref(self.pattern), self.vec, precision, ptr(vals), ptr(self.bc_rows), self.n_bc,
                 1.0, _stream())
        A = DeviceCSR(self, precision, vals, bc_mode)
        self._tangent_cache[key] = A
        return A

    def _sliced_reference(self, A64, bc_mode):
        """Sliced FP64 copy of A64 (the FP64 CSR a DF48 copy was split from): the operator of the
        mixed solver's FP64 reliable updates (fem_pcg_refined takes FEM_SLICED_F64), whose SpMV
        runs ~2.3x faster than the CSR one on the same values."""
        nb = C.c_size_t()
        call("fem_matrix_bytes", C.byref(self.pattern), self.vec, _lib.FEM_SLICED_F64, C.byref(nb))
        name = f"valsref_{bc_mode}"
        buf = getattr(self, name, None)
        if buf is None or buf.numel() != nb.value:
            buf = torch.empty(nb.value, dtype=torch.uint8, device=self.device)
            setattr(self, name, buf)
        call("fem_matrix_convert", C.byref(self.pattern), self.num_nodes, self.vec, ptr(A64.data),
             _lib.FEM_SLICED_F64, ptr(buf), _stream())
        return DeviceCSR(self, _lib.FEM_SLICED_F64, buf.view(torch.float64), bc_mode, source=A64)

    def apply(self, dofs, w, skip_bc_rows=True):
        """K(u) w in FP64, matrix-free (tangent action kernel)."""
        self.refresh_bc()
        _, ms = self.material()
        out = torch.zeros(self.num_dofs, dtype=torch.float64, device=self.device)
        call("fem_assemble", C.byref(self.mesh), C.byref(ms), C.byref(self.pattern), _lib.FEM_OUT_APPLY,
             _lib.FEM_F64, ptr(dofs.contiguous()), ptr(w.contiguous()), ptr(self.bc_mask) if skip_bc_rows else None,
             _lib.FEM_BC_NONE, None, None, ptr(out), _stream())
        if self._robin:
            self._robin_call(_lib.FEM_OUT_APPLY, _lib.FEM_F64, dofs.contiguous(), w=w.contiguous(),
                             bc=self.bc_mask if skip_bc_rows else None, apply_out=out)
        if self.has_universal:
            self._universal_call(_lib.FEM_OUT_APPLY, dofs.contiguous(), w=w.contiguous(),
                                 bc=self.bc_mask if skip_bc_rows else None, apply_out=out)
        return out

    # ---- compiled universal kernels (get_universal_kernel / get_universal_kernels_surface) ----
    @property
    def has_universal(self):
        p = self.problem
        return hasattr(p, "get_universal_kernel") or hasattr(p, "get_universal_kernels_surface")

    def _universal_ivs(self):
        """The internal variables as the universal cell kernel sees them: per cell (nq, ...) arrays,
        concatenated per cell into one FP64 buffer (num_cells, iv_stride)."""
        p = self.problem
        ivs = [torch.as_tensor(t, dtype=torch.float64, device=self.device) for t in p.internal_vars]
        for t in ivs:
            if t.dim() < 1 or t.shape[0] != self.num_cells:
                raise ValueError(f"internal variable of shape {tuple(t.shape)}: the universal kernel needs "
                                 f"(num_cells, num_quads, ...) arrays")
        shapes = tuple(tuple(t.shape[1:]) for t in ivs)
        buf = torch.cat([t.reshape(self.num_cells, -1) for t in ivs], dim=1).contiguous() if ivs else None
        return ivs, shapes, buf

    def universal(self):
        """Compiled kernels of the problem's universal kernels, traced again whenever the shapes of
        the internal variables change."""
        from . import jit
        p = self.problem
        _, shapes, _ = self._universal_ivs()
        key = shapes
        if self._uk is not None and self._uk_key == key:
            return self._uk
        fe = self.fe
        t = {k: getattr(fe, k) for k in ("shape_vals", "shape_grads_ref", "quad_weights", "face_shape_vals",
                                         "face_shape_grads_ref", "face_quad_weights", "face_normals")}
        cell = face = None
        if hasattr(p, "get_universal_kernel"):
            fn_src, ivs = jit.trace_cell(p.get_universal_kernel(), self.nn, self.num_quads, self.vec, shapes)
            cell = (jit.CompiledKernels(jit.cell_source(fn_src, t, self.nn, self.num_quads, self.vec, ivs), ivs, 0),
                    ivs)
        if hasattr(p, "get_universal_kernels_surface"):
            kernels = p.get_universal_kernels_surface()
            if len(kernels) != len(p.boundary_inds_list):
                raise AssertionError("get_universal_kernels_surface must give one kernel per location_fns entry")
            if any(len(v) for v in p.internal_vars_surfaces):
                raise NotImplementedError("internal_vars_surfaces are not passed to compiled surface kernels")
            srcs = [jit.trace_face(fn, self.nn, fe.num_face_quads, self.vec, k) for k, fn in enumerate(kernels)]
            faces = []
            for bi in p.boundary_inds_list:
                bi = np.asarray(bi)
                faces.append((torch.as_tensor(bi[:, 0].astype(np.int32), device=self.device),
                              torch.as_tensor(bi[:, 1].astype(np.int32), device=self.device)) if len(bi) else None)
            face = (jit.CompiledKernels(jit.face_source(srcs, t, self.nn, self.vec, 0), 0, len(srcs)), faces)
        self._uk, self._uk_key = (cell, face), key
        return self._uk

    def _universal_call(self, outputs, dofs, w=None, lam=None, bc=None, bc_mode=_lib.FEM_BC_NONE, res=None,
                        vals=None, apply_out=None, vjp_out=None):
        from . import jit
        (cell, face) = self.universal()
        s = _stream()
        common = dict(coords=self.coords.data_ptr(), conn=self.conn.data_ptr(), u=dofs.data_ptr(),
                      w=None if w is None else w.data_ptr(), lam=None if lam is None else lam.data_ptr(),
                      indptr=self.indptr.data_ptr(), slots=self.slots.data_ptr(),
                      bc=None if bc is None else bc.data_ptr(), bc_mode=bc_mode, outputs=outputs,
                      res=None if res is None else res.data_ptr(), vals=None if vals is None else vals.data_ptr(),
                      apply_out=None if apply_out is None else apply_out.data_ptr())
        if cell is not None:
            ck, ivs = cell
            _, _, buf = self._universal_ivs()
            self._uk_ivbuf = buf      # alive until the stream has used it
            P = jit.params(n_items=self.num_cells, iv=None if buf is None else buf.data_ptr(), iv_stride=ivs,
                           vjp_out=None if vjp_out is None else vjp_out.data_ptr(), **common)
            ck.launch("fem_ucell", P, self.num_cells, s)
        if face is not None and not (outputs & _lib.FEM_OUT_PARAM_VJP):
            fk, faces = face
            for k, fc in enumerate(faces):
                if fc is None:
                    continue
                P = jit.params(n_items=fc[0].numel(), face_cells=fc[0].data_ptr(), face_ids=fc[1].data_ptr(),
                               iv=None, iv_stride=0, vjp_out=None, **common)
                fk.launch(f"fem_uface_{k}", P, fc[0].numel(), s)

    def universal_param_vjp(self, dofs, lam):
        """-lam^T dR_universal/d(internal vars): a list shaped like problem.internal_vars (lam masked
        to 0 on Dirichlet dofs), or None without a universal cell kernel."""
        (cell, _) = self.universal()
        if cell is None or cell[1] == 0:
            return None
        self.refresh_bc()
        ivs, shapes, _ = self._universal_ivs()
        out = torch.empty(self.num_cells, cell[1], dtype=torch.float64, device=self.device)
        self._universal_call(_lib.FEM_OUT_PARAM_VJP, dofs.contiguous(), lam=lam.contiguous(), bc=self.bc_mask,
                             vjp_out=out)
        res, o = [], 0
        for t, sh in zip(ivs, shapes):
            k = int(np.prod(sh))
            res.append(out[:, o:o + k].reshape(t.shape))
            o += k
        return res

    def param_vjp(self, dofs, lam):
        """-lam^T dR/dp per quadrature point (lam masked to 0 on Dirichlet dofs)."""
        self.refresh_bc()
        m, ms = self.material()
        if m.param_index is None:
            raise NotImplementedError(f"{type(m).__name__} has no differentiable per-point parameter")
        g = torch.empty(self.num_cells * self.num_quads, dtype=torch.float64, device=self.device)
        call("fem_param_vjp", C.byref(self.mesh), C.byref(ms), ptr(dofs.contiguous()), ptr(lam.contiguous()),
             ptr(self.bc_mask), ptr(g), _stream())
        return g

    def j2_history_vjp(self, dofs, lam=None, hist_bar=None, want_scale=False, want_u=False):
        """fem_j2_history_vjp: cotangents of the J2 history (cells, nq, 18) and of the modulus scale
        (cells*nq, or None); in update mode (hist_bar) also that of u (n_dofs, or None)."""
        self.refresh_bc()
        m, ms = self.material()
        nq = self.num_cells * self.num_quads
        hg = torch.empty(nq * 18, dtype=torch.float64, device=self.device)
        sg = torch.empty(nq, dtype=torch.float64, device=self.device) if want_scale else None
        ug = torch.zeros(self.num_dofs, dtype=torch.float64, device=self.device) if want_u else None
        hb = None if hist_bar is None else hist_bar.to(torch.float64).reshape(-1).contiguous()
        call("fem_j2_history_vjp", C.byref(self.mesh), C.byref(ms), ptr(dofs.contiguous()),
             None if lam is None else ptr(lam.contiguous()), ptr(self.bc_mask), None if hb is None else ptr(hb),
             ptr(hg), ptr(sg), ptr(ug), _stream())
        return hg.reshape(self.num_cells, self.num_quads, 18), sg, ug

    def j2_update(self, dofs):
        m, ms = self.material()
        out = torch.empty(self.num_cells * self.num_quads * 18, dtype=torch.float64, device=self.device)
        call("fem_j2_update", C.byref(self.mesh), C.byref(ms), ptr(dofs.contiguous()), ptr(out), _stream())
        out = out.reshape(self.num_cells, self.num_quads, 18)
        return out[:, :, :9].reshape(self.num_cells, self.num_quads, 3, 3), \
            out[:, :, 9:].reshape(self.num_cells, self.num_quads, 3, 3)

    # ---- Krylov --------------------------------------------------------------------
    def workspace(self, precision):
        if precision not in self._ws:
            nb = C.c_size_t()
            call("fem_krylov_workspace", self.num_dofs, precision, C.byref(nb))
            self._ws[precision] = torch.empty(nb.value, dtype=torch.uint8, device=self.device)
        return self._ws[precision]

    def krylov(self, method, A, b, x, pc_kind, rtol, atol, maxiter):
        """Run fem_pcg / fem_bicgstab; x is updated in place. Returns (iterations, residual norm, status)."""
        ws = self.workspace(_lib.FEM_F32 if A.vector_dtype == torch.float32 else _lib.FEM_F64)
        pc = A.preconditioner(pc_kind)
        it, rn, st = C.c_int64(), C.c_double(), C.c_int32()
        t0 = time.perf_counter()
        call("fem_pcg" if method == "cg" else "fem_bicgstab", C.byref(self.pattern), self.num_nodes, self.vec,
             A.precision, ptr(A.data), pc_kind, ptr(pc), ptr(b), ptr(x), float(rtol), float(atol), int(maxiter),
             ptr(ws), ws.numel(), C.byref(it), C.byref(rn), C.byref(st), _stream())
        rec = dict(method=method, precision={0: "fp32", 1: "fp64", 3: "sliced-fp32", 4: "sliced-fp64"}.get(A.precision),
                   iterations=it.value, res_norm=rn.value, status=_lib.SOLVE_STATUS.get(st.value, "?"),
                   seconds=time.perf_counter() - t0)
        self.solve_log.append(rec)
        logger.debug("krylov %s", rec)
        return it.value, rn.value, st.value

    def pcg_refined(self, A32, b, x, u_lin, pc_kind, rtol, atol, delta, maxiter):
        """PCG with FP64 reliable updates on the Dirichlet-eliminated tangent at u_lin; A32 is a
        FEM_F32 or FEM_DF48 matrix.  x (FP64) is updated in place.
        Returns (iterations, residual replacements, residual, status)."""
        self.refresh_bc()
        _, ms = self.material()
        ws = self.workspace(_lib.FEM_F64)
        pc = A32.preconditioner(pc_kind)
        it, up, rn, st = C.c_int64(), C.c_int64(), C.c_double(), C.c_int32()
        t0 = time.perf_counter()
        ref = A32.source if A32.source is not None and A32.source.bc_mode == _lib.FEM_BC_SYMMETRIC else None
        if ref is not None and getattr(A32, "ref64", None) is not None:
            ref = A32.ref64      # the same values in the sliced FP64 layout
        call("fem_pcg_refined", C.byref(self.pattern), self.num_nodes, self.vec, A32.precision, ptr(A32.data),
             pc_kind, ptr(pc),
             C.byref(self.mesh), C.byref(ms), ptr(u_lin.contiguous()), None if ref is None else ptr(ref.data),
             _lib.FEM_F64 if ref is None else ref.precision, ptr(self.bc_mask), ptr(b.contiguous()), ptr(x),
             float(rtol), float(atol), float(delta), int(maxiter), ptr(ws), ws.numel(), C.byref(it), C.byref(up),
             C.byref(rn), C.byref(st), _stream())
        rec = dict(method="cg-refined",
                   precision={_lib.FEM_DF48: "df48+fp64", _lib.FEM_SLICED_DF48: "df48+fp64",
                              _lib.FEM_SYM_DF48: "sym-df48+fp64",
                              _lib.FEM_SSYM_DF48: "ssym-df48+fp64"}.get(A32.precision, "fp32+fp64"),
                   iterations=it.value, updates=up.value,
                   res_norm=rn.value, status=_lib.SOLVE_STATUS.get(st.value, "?"), seconds=time.perf_counter() - t0)
        self.solve_log.append(rec)
        logger.debug("krylov %s", rec)
        return it.value, up.value, rn.value, st.value

    def cast32(self, x64, mask=None):
        out = torch.empty(x64.numel(), dtype=torch.float32, device=self.device)
        call("fem_cast_f64_f32", ptr(x64.contiguous()), ptr(out), x64.numel(), ptr(mask), _stream())
        return out

    def axpy32(self, alpha, x32, y64):
        call("fem_axpy_f32_f64", float(alpha), ptr(x32), ptr(y64), y64.numel(), _stream())
        return y64
