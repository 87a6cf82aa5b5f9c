"""The vectorised SIMP oracle (oracle/simp_fast.py) against the general restatement
(oracle/fem.py), on the CPU: its COO -> CSR slot map reproduces the PETSc-semantics pattern and
values, its end-face traction load equals the general surface kernel's, its block-Jacobi PCG
solves the system and its batched element stiffness equals the per-point einsum form."""
import numpy as np
import torch

from oracle import basis, fem as ofem, simp_fast


def _case(n=(6, 3, 2), L=(2.0, 1.0, 0.5), jitter=0.0):
    pts, cells = ofem.box_mesh(*n, *L)
    if jitter:
        pts = pts + np.random.default_rng(5).uniform(-jitter, jitter, pts.shape)
    left = np.isclose(pts[:, 0], 0.0, atol=1e-5)
    rows = (3 * np.argwhere(left).reshape(-1)[:, None] + np.arange(3)[None, :]).reshape(-1)
    return pts, cells, rows


def test_element_stiffness_matches_einsum_form():
    pts, cells, _ = _case(jitter=0.02)
    G, jxw = simp_fast.hex8_geometry(pts, cells)
    K = simp_fast.unit_element_stiffness(G, jxw, 0.3)
    lam, mu = 0.3 / (1.3 * 0.4), 1.0 / 2.6
    t1 = lam * np.einsum("cq,cqai,cqbk->caibk", jxw, G, G)
    t2 = mu * np.einsum("cq,cqak,cqbi->caibk", jxw, G, G)
    t3 = mu * np.einsum("cab,ik->caibk", np.einsum("cq,cqad,cqbd->cab", jxw, G, G), np.eye(3))
    ref = (t1 + t2 + t3).reshape(-1, 24, 24)
    assert np.abs(K - ref).max() <= 1e-14 * np.abs(ref).max()


def test_csr_map_pattern_values_and_load():
    pts, cells, rows = _case()
    right = np.isclose(pts[:, 0], 2.0, atol=1e-5)
    f = simp_fast.traction_load(pts, cells, right, [0.0, 0.0, 1.0])
    op = ofem.OracleProblem(pts, cells, 3, location_fns=[lambda p: np.isclose(p[0], 2.0, atol=1e-5)],
                            tensor_map=None, surface_maps=[lambda u, x: torch.tensor([0.0, 0.0, 1.0])])
    f_or = op.compute_residual(torch.zeros(3 * len(pts))).numpy()
    assert np.abs(f - f_or).max() <= 1e-14
    assert abs(f.reshape(-1, 3)[:, 2].sum() - 0.5) <= 1e-14            # traction 1 on a 1 x 0.5 face
    sc = simp_fast.SimpCantilever(pts, cells, rows, f)
    th = 0.5 + np.random.default_rng(1).uniform(-0.05, 0.05, (len(cells), 1))
    M = sc.csr_map
    ip, ix = ofem.coo_pattern(sc.I, sc.J, sc.N)
    np.testing.assert_array_equal(M.indptr, ip)
    np.testing.assert_array_equal(M.indices, ix)
    A = sc.assemble_csr(th)
    B = sc.assemble(th)
    assert abs(A - B).max() <= 1e-15 * abs(B).max()
    P = M.block_jacobi(A)
    u, it = sc.pcg(A, sc.f, 1e-12, precond=P)
    assert np.linalg.norm(sc.f - A @ u) <= 1e-11 * np.linalg.norm(sc.f)   # rtol 1e-12 on the recursive residual
    blocks = A.toarray().reshape(len(pts), 3, len(pts), 3)[np.arange(len(pts)), :, np.arange(len(pts)), :]
    r = np.random.default_rng(2).standard_normal(sc.N)
    z = np.einsum("nij,nj->ni", np.linalg.inv(blocks), r.reshape(-1, 3)).reshape(-1)
    assert np.abs(P(r) - z).max() <= 1e-12 * np.abs(z).max()
