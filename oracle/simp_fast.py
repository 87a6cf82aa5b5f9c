"""Vectorised FP64 CPU restatement of one SIMP topology-optimisation iteration
(test infrastructure and CPU baseline -- never shipped or measured as the product).

Same algorithm as the reference's path for a SIMP linear-elastic problem:
  element tangents   K_e = sum_q JxW (lam g_a g_b^T + mu g_b g_a^T + mu (g_a.g_b) I)
                     (what jacfwd of the laplace kernel yields, jax_fem/problem.py:189-214, 262-301)
  global assembly    COO sum onto the PETSc pattern (jax_fem/solver.py:469-529)
  Dirichlet rows     symmetric elimination (same solution as zeroRows + BC-consistent x0,
                     jax_fem/solver.py:390-421)
  solve              Jacobi or 3x3 block-Jacobi PCG (PETSc KSPCG + PCJACOBI / PCBJACOBI,
                     jax_fem/solver.py:109-134)
  adjoint            K_ff lam_f = v_f, grad = -E'(theta) lam_e^T K0_e u_e
                     (implicit_vjp, jax_fem/solver.py:1362-1418)
"""
import numpy as np
import scipy.sparse as sp

from . import basis


def hex8_geometry(points, cells):
    t = basis.element_tables("HEX8")
    X = points[cells]
    J = np.einsum("cnd,qne->cqde", X, t["shape_grads_ref"])
    inv = np.linalg.inv(J)
    G = np.einsum("qne,cqed->cqnd", t["shape_grads_ref"], inv)
    jxw = np.linalg.det(J) * t["quad_weights"]
    return G, jxw


def unit_element_stiffness(G, jxw, nu):
    """K0_e for E = 1: (C, 24, 24).

    K[(a,i),(b,k)] = sum_q jxw (lam g_ai g_bk + mu g_ak g_bi + mu d_ik g_a.g_b).  All three terms
    come from S[(a,i),(b,k)] = sum_q jxw g_ai g_bk, one batched matrix product of the scaled
    24-vectors of shape gradients: the second term is S with i and k swapped, the third the
    trace of S over i = k."""
    lam = nu / ((1 + nu) * (1 - 2 * nu))
    mu = 1.0 / (2 * (1 + nu))
    C, nq, nn, _ = G.shape
    V = (G * np.sqrt(jxw)[:, :, None, None]).reshape(C, nq, 3 * nn)
    S = np.matmul(V.transpose(0, 2, 1), V).reshape(C, nn, 3, nn, 3)
    dots = np.einsum("caibi->cab", S)
    K = lam * S + mu * S.transpose(0, 1, 4, 3, 2)
    K += mu * dots[:, :, None, :, None] * np.eye(3)[None, None, :, None, :]
    return K.reshape(C, 3 * nn, 3 * nn)


def element_stiffness(points, cells, nu, chunk=131072):
    """K0_e of every cell, computed in chunks of cells to bound the temporaries."""
    out = np.empty((len(cells), 24, 24))
    for s in range(0, len(cells), chunk):
        G, jxw = hex8_geometry(points, cells[s:s + chunk])
        out[s:s + chunk] = unit_element_stiffness(G, jxw, nu)
    return out


def traction_load(points, cells, on_face, t):
    """Consistent nodal load of a constant traction-type surface map t (vec 3) on the faces whose
    four vertices all satisfy the node flags on_face: f_a += sum_q t N_a(q) nanson(q)
    (get_boundary_conditions_inds + the surface kernel, jax_fem/fe.py:271-322,
    problem.py:238-259), computed on the selected faces only."""
    tb = basis.element_tables("HEX8")
    face_nodes = cells[:, tb["face_inds"]]                    # (C, nf, 4)
    sel = np.argwhere(np.all(on_face[face_nodes], axis=2))     # (F, 2): cell, local face
    X = points[cells[sel[:, 0]]]
    fg = tb["face_shape_grads_ref"][sel[:, 1]]
    n = tb["face_normals"][sel[:, 1]]
    Jac = np.einsum("fnd,fqne->fqde", X, fg)
    inv = np.linalg.inv(Jac)
    nanson = np.linalg.norm(np.einsum("fe,fqed->fqd", n, inv), axis=-1) * np.linalg.det(Jac)
    nanson = nanson * tb["face_quad_weights"][sel[:, 1]]
    w = np.einsum("fqn,fq->fn", tb["face_shape_vals"][sel[:, 1]], nanson)   # (F, nn)
    f = np.zeros((points.shape[0], 3))
    np.add.at(f, cells[sel[:, 0]].reshape(-1), (w.reshape(-1)[:, None] * np.asarray(t)[None, :]))
    return f.reshape(-1)


class CsrMap:
    """The global CSR pattern and the position of every element-matrix entry in it -- what
    PETSc's COO preallocation (setPreallocationCOO, jax_fem/solver.py:469-478) builds once, so
    that each assembly is one summation of the element values into fixed slots (setValuesCOO,
    solver.py:522-526).  Built from the sorted unique node pairs of the cells (vec x vec blocks):
    scalar row vec*n + i holds vec*nb_n values, and entry (cell c, node a, comp i, node b,
    comp k) sits at vec^2 bp[n_a] + i vec nb_{n_a} + vec (slot of n_b in row n_a) + k.
    Dirichlet rows and columns are eliminated symmetrically with a unit diagonal."""

    def __init__(self, cells, n_nodes, bc, vec=3):
        C, nn = cells.shape
        self.vec, self.n_nodes = vec, n_nodes
        na = np.repeat(cells, nn, axis=1).reshape(-1).astype(np.int64)     # (C*nn*nn) in (c, a, b) order
        nb = np.tile(cells, (1, nn)).reshape(-1).astype(np.int64)
        keys = na * n_nodes + nb
        uk = np.unique(keys)
        brow = uk // n_nodes
        bcol = (uk % n_nodes).astype(np.int64)
        cnt = np.bincount(brow, minlength=n_nodes)
        bp = np.zeros(n_nodes + 1, dtype=np.int64)
        np.cumsum(cnt, out=bp[1:])
        kb = np.searchsorted(uk, keys)
        del keys
        vv = vec * vec
        base = vv * bp[na] + vec * (kb - bp[na])
        width = vec * cnt[na]
        del kb, nb
        ar = np.arange(vec, dtype=np.int64)
        slot = (base.reshape(C, nn, 1, nn, 1) + (ar[None, None, :, None, None] * width.reshape(C, nn, 1, nn, 1))
                + ar[None, None, None, None, :])
        self.slot = slot.reshape(-1)          # matches K (C, nn*vec, nn*vec) row-major
        del base, width, na
        self.nnz = int(vv * len(uk))
        N = vec * n_nodes
        indptr = np.empty(N + 1, dtype=np.int64)
        rs = (vv * bp[:-1])[:, None] + ar[None, :] * (vec * cnt)[:, None]
        indptr[:-1] = rs.reshape(-1)
        indptr[-1] = self.nnz
        # scalar column of every slot: block column * vec + k, laid out row by row
        pos = ((vv * bp[brow])[:, None, None] + ar[None, :, None] * (vec * cnt[brow])[:, None, None]
               + (vec * (np.arange(len(uk)) - bp[brow]))[:, None, None] + ar[None, None, :])
        indices = np.empty(self.nnz, dtype=np.int32)
        indices[pos.reshape(-1)] = np.broadcast_to((vec * bcol)[:, None, None] + ar[None, None, :],
                                                   pos.shape).reshape(-1).astype(np.int32)
        del pos
        self.indptr, self.indices = indptr, indices
        row_of = np.repeat(np.arange(N, dtype=np.int32), np.diff(indptr))
        self.elim = bc[row_of] | bc[indices]
        del row_of
        diag_slot = np.searchsorted(uk, np.arange(n_nodes, dtype=np.int64) * n_nodes + np.arange(n_nodes))
        self.diag = ((vv * bp[:-1])[:, None] + ar[None, :] * (vec * cnt)[:, None]
                     + (vec * (diag_slot - bp[:-1]))[:, None] + ar[None, :]).reshape(-1)
        self.bc_rows = np.nonzero(bc)[0]
        self.block_diag = ((vv * bp[:-1])[:, None, None] + ar[None, :, None] * (vec * cnt)[:, None, None]
                           + (vec * (diag_slot - bp[:-1]))[:, None, None] + ar[None, None, :])

    def assemble(self, V):
        """CSR values from the element values V (C, nn*vec, nn*vec): sum into the slots, then
        the symmetric Dirichlet elimination with a unit diagonal."""
        vals = np.bincount(self.slot, weights=V.reshape(-1), minlength=self.nnz)
        vals[self.elim] = 0.0
        vals[self.diag[self.bc_rows]] = 1.0
        N = self.vec * self.n_nodes
        return sp.csr_matrix((vals, self.indices, self.indptr), shape=(N, N))

    def block_jacobi(self, A):
        """Inverse vec x vec diagonal blocks of A, applied as a preconditioner (component-wise
        products of contiguous arrays: z_i = sum_j Dinv_ij r_j)."""
        vec = self.vec
        D = np.linalg.inv(A.data[self.block_diag])
        Dc = [[np.ascontiguousarray(D[:, i, j]) for j in range(vec)] for i in range(vec)]

        def apply(r):
            rr = r.reshape(-1, vec)
            rc = [np.ascontiguousarray(rr[:, j]) for j in range(vec)]
            z = np.empty_like(rr)
            for i in range(vec):
                acc = Dc[i][0] * rc[0]
                for j in range(1, vec):
                    acc += Dc[i][j] * rc[j]
                z[:, i] = acc
            return z.reshape(-1)
        return apply


class ThreadedCSR:
    """y = A x with the rows split into `threads` contiguous blocks run in a thread pool."""

    def __init__(self, A, threads):
        from concurrent.futures import ThreadPoolExecutor
        self.A = A
        n = A.shape[0]
        self.bounds = np.linspace(0, n, threads + 1).astype(np.int64)
        self.blocks = [A[self.bounds[i]:self.bounds[i + 1]] for i in range(threads)]
        self.pool = ThreadPoolExecutor(threads)

    def diagonal(self):
        return self.A.diagonal()

    def __matmul__(self, x):
        y = np.empty(self.A.shape[0])

        def part(i):
            y[self.bounds[i]:self.bounds[i + 1]] = self.blocks[i] @ x
        list(self.pool.map(part, range(len(self.blocks))))
        return y


class SimpCantilever:
    def __init__(self, points, cells, bc_rows, f_ext, Emax=1.0, Emin=1e-3, nu=0.3, penal=3.0):
        self.points, self.cells = points, cells
        self.N = points.shape[0] * 3
        self.Emax, self.Emin, self.nu, self.penal = Emax, Emin, nu, penal
        self.K0 = element_stiffness(points, cells, nu)
        self.dofs = (3 * cells[:, :, None] + np.arange(3)[None, None, :]).reshape(len(cells), 24)
        self.bc = np.zeros(self.N, dtype=bool)
        self.bc[bc_rows] = True
        self.f = f_ext.copy()
        self.f[self.bc] = 0.0
        self._csr_map = None

    @property
    def I(self):
        return np.repeat(self.dofs[:, :, None], 24, axis=2).reshape(-1)

    @property
    def J(self):
        return np.repeat(self.dofs[:, None, :], 24, axis=1).reshape(-1)

    def modulus(self, th):
        return self.Emin + (self.Emax - self.Emin) * th ** self.penal

    @property
    def csr_map(self):
        if self._csr_map is None:
            self._csr_map = CsrMap(self.cells, self.points.shape[0], self.bc)
        return self._csr_map

    def assemble_csr(self, theta):
        """Assembly through the precomputed COO -> CSR slot map (the PETSc COO path): element
        values E(theta_e) K0_e summed into their fixed CSR slots, Dirichlet eliminated."""
        E = self.modulus(theta.reshape(-1))
        return self.csr_map.assemble(E[:, None, None] * self.K0)

    def assemble(self, theta):
        E = self.modulus(theta.reshape(-1))
        V = (E[:, None, None] * self.K0)
        I, J = self.I, self.J
        keep = ~(self.bc[I] | self.bc[J])
        A = sp.csr_matrix((V.reshape(-1)[keep], (I[keep], J[keep])), shape=(self.N, self.N))
        A = A + sp.diags(self.bc.astype(np.float64))
        A.sum_duplicates()
        return A.tocsr()

    @staticmethod
    def pcg(A, b, rtol, maxiter=100000, iters=None, threads=1, precond=None):
        """Jacobi PCG (or the preconditioner `precond`, a function r -> z); with threads > 1 the
        SpMV runs on row blocks in a thread pool (scipy's CSR kernel releases the GIL), the way a
        multi-core host would run it."""
        if threads > 1 and not isinstance(A, ThreadedCSR):
            A = ThreadedCSR(A, threads)
        if precond is None:
            d = A.diagonal()
            precond = lambda v: v / d
        from scipy.linalg.blas import daxpy, ddot, dscal
        x = np.zeros_like(b)
        r = b.copy()
        z = precond(r)
        p = z.copy()
        rz = ddot(r, z)
        thresh2 = (rtol * np.linalg.norm(b)) ** 2
        rr = ddot(r, r)
        it = 0
        # vector updates in place through BLAS level 1 (no temporaries)
        while rr > thresh2 and it < maxiter and (iters is None or it < iters):
            q = A @ p
            alpha = rz / ddot(p, q)
            daxpy(p, x, a=alpha)
            daxpy(q, r, a=-alpha)
            z = precond(r)
            rz_new = ddot(r, z)
            rr = ddot(r, r)
            dscal(rz_new / rz, p)
            daxpy(z, p)
            rz = rz_new
            it += 1
        return x, it

    def iteration(self, theta, rtol=1e-8, pcg_iters=None):
        """Compliance, gradient and PCG iteration counts (forward, adjoint)."""
        A = self.assemble(theta)
        u, it_f = self.pcg(A, self.f, rtol, iters=pcg_iters)
        J = self.f @ u
        lam, it_a = self.pcg(A, self.f, rtol, iters=pcg_iters)    # v = dJ/du = f
        th = theta.reshape(-1)
        dE = (self.Emax - self.Emin) * self.penal * th ** (self.penal - 1)
        ue, le = u[self.dofs], lam[self.dofs]
        g = -dE * np.einsum("ci,cij,cj->c", le, self.K0, ue)
        return J, g.reshape(theta.shape), it_f, it_a
