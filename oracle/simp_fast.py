"""Vectorised FP64 CPU restatement of one SIMP topology-optimisation iteration
(test infrastructure and CPU baseline -- never shipped or measured as the product).

Same algorithm as the reference's path for a SIMP linear-elastic problem:
  element tangents   K_e = sum_q JxW (lam g_a g_b^T + mu g_b g_a^T + mu (g_a.g_b) I)
                     (what jacfwd of the laplace kernel yields, jax_fem/problem.py:189-214, 262-301)
  global assembly    COO sum onto the PETSc pattern (jax_fem/solver.py:469-529)
  Dirichlet rows     symmetric elimination (same solution as zeroRows + BC-consistent x0,
                     jax_fem/solver.py:390-421)
  solve              Jacobi PCG (PETSc KSPCG + PCJACOBI, jax_fem/solver.py:109-134)
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
    """K0_e for E = 1: (C, 24, 24)."""
    lam = nu / ((1 + nu) * (1 - 2 * nu))
    mu = 1.0 / (2 * (1 + nu))
    C = G.shape[0]
    eye = np.eye(3)
    # K[(a,i),(b,k)] = sum_q jxw (lam g_ai g_bk + mu g_ak g_bi + mu d_ik g_a.g_b)
    t1 = lam * np.einsum("cq,cqai,cqbk->caibk", jxw, G, G)
    t2 = mu * np.einsum("cq,cqak,cqbi->caibk", jxw, G, G)
    dots = np.einsum("cq,cqad,cqbd->cab", jxw, G, G)
    t3 = mu * np.einsum("cab,ik->caibk", dots, eye)
    return (t1 + t2 + t3).reshape(C, 24, 24)


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
        G, jxw = hex8_geometry(points, cells)
        self.K0 = unit_element_stiffness(G, jxw, nu)
        self.dofs = (3 * cells[:, :, None] + np.arange(3)[None, None, :]).reshape(len(cells), 24)
        self.I = np.repeat(self.dofs[:, :, None], 24, axis=2).reshape(-1)
        self.J = np.repeat(self.dofs[:, None, :], 24, axis=1).reshape(-1)
        self.bc = np.zeros(self.N, dtype=bool)
        self.bc[bc_rows] = True
        self.f = f_ext.copy()
        self.f[self.bc] = 0.0

    def modulus(self, th):
        return self.Emin + (self.Emax - self.Emin) * th ** self.penal

    def assemble(self, theta):
        E = self.modulus(theta.reshape(-1))
        V = (E[:, None, None] * self.K0)
        keep = ~(self.bc[self.I] | self.bc[self.J])
        A = sp.csr_matrix((V.reshape(-1)[keep], (self.I[keep], self.J[keep])), shape=(self.N, self.N))
        A = A + sp.diags(self.bc.astype(np.float64))
        A.sum_duplicates()
        return A.tocsr()

    @staticmethod
    def pcg(A, b, rtol, maxiter=100000, iters=None, threads=1):
        """Jacobi PCG; with threads > 1 the SpMV runs on row blocks in a thread pool (scipy's
        CSR kernel releases the GIL), the way a multi-core host would run it."""
        if threads > 1:
            A = ThreadedCSR(A, threads)
        d = A.diagonal()
        x = np.zeros_like(b)
        r = b.copy()
        z = r / d
        p = z.copy()
        rz = r @ z
        thresh = rtol * np.linalg.norm(b)
        it = 0
        while np.linalg.norm(r) > thresh and it < maxiter and (iters is None or it < iters):
            q = A @ p
            alpha = rz / (p @ q)
            x += alpha * p
            r -= alpha * q
            z = r / d
            rz_new = r @ z
            p = z + (rz_new / rz) * p
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
