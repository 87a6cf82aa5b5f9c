"""GPU parity of the TO update (jax_fem/mma.py): the filter built by fem_filter_build against the
oracle's scipy k-d tree filter, the filter products, fem_mma_update against the oracle's
mmasub/subsolv over successive iterations, and the optimize loop against the same loop driven
by the oracle."""
import importlib

import numpy as np
import pytest
import torch

from oracle import mma as omma

pytestmark = pytest.mark.gpu


def _mma_mod():
    return importlib.import_module("jax_fem_gb300.mma")


def _dense(F, n):
    cols = F.cols.cpu().numpy()
    vals = F.vals.cpu().numpy()
    H = np.zeros((n, n))
    for i in range(n):
        for k in range(cols.shape[1]):
            if cols[i, k] >= 0:
                H[i, cols[i, k]] += vals[i, k]
    return H


def _jittered_box(nx, ny, nz, amp, seed):
    import jax_fem_gb300 as jf
    m = jf.box_mesh(nx, ny, nz, 1.0, 0.8, 0.6)
    pts = np.array(m.points)
    rng = np.random.default_rng(seed)
    h = 1.0 / nx
    pts += rng.uniform(-amp, amp, pts.shape) * h
    return jf.Mesh(pts, m.cells_dict["hexahedron"])


@pytest.mark.parametrize("amp", [0.0, 0.15])
def test_filter_matches_kd_tree(cuda, amp):
    """compute_filter_kd_tree on a uniform and on a jittered HEX8 mesh (9x7x5): the domain volume
    (JxW summed on the device) equals the oracle's to 1e-14, and the GPU filter's weights and row
    sums equal the oracle's k-d tree filter to 1e-14."""
    import jax_fem_gb300 as jf

    class P(jf.Problem):
        def get_tensor_map(self):
            return jf.LinearElastic(1.0, 0.3)

    mesh = _jittered_box(9, 7, 5, amp, 1)
    prob = P(mesh, vec=3, dim=3)
    fe = prob.fes[0]
    M = _mma_mod()
    H, Hs = M.compute_filter_kd_tree(fe)
    cent = np.mean(fe.points[fe.cells], axis=1)
    V = omma.cell_volume(fe.points, fe.cells, fe.shape_grads_ref, fe.quad_weights)
    assert abs(M._cell_volume(fe) - V) <= 1e-14 * V
    Ho, Hso, rmin = omma.filter_kd_tree(cent, V)
    assert abs(H.rmin - rmin) <= 1e-14 * rmin
    np.testing.assert_allclose(_dense(H, fe.num_cells), Ho.toarray(), rtol=0, atol=1e-14)
    np.testing.assert_allclose(Hs.cpu().numpy(), Hso, rtol=1e-14, atol=0)


def test_filter_truncates_to_twenty_nearest(cuda):
    """A random cloud with ~45 points inside rmin: fem_filter_build keeps the 20 nearest, as the
    k-d tree query does (random distances, no ties)."""
    import ctypes as C
    import jax_fem_gb300 as jf
    L = jf._lib
    rng = np.random.default_rng(4)
    n = 3000
    pts = rng.uniform(0, 1, (n, 3))
    rmin = 0.155
    c = torch.tensor(pts, device=cuda)
    cols = torch.empty(n, 20, dtype=torch.int32, device=cuda)
    vals = torch.empty(n, 20, dtype=torch.float64, device=cuda)
    hs = torch.empty(n, dtype=torch.float64, device=cuda)
    nb = C.c_size_t()
    L.call("fem_filter_workspace", n, C.byref(nb))
    ws = torch.empty(nb.value, dtype=torch.uint8, device=cuda)
    L.call("fem_filter_build", n, L.ptr(c), rmin, 20, L.ptr(cols), L.ptr(vals), L.ptr(hs), L.ptr(ws), nb.value,
           L.stream_handle())
    import scipy.spatial
    dd, ii = scipy.spatial.KDTree(pts).query(pts, 20)
    w = np.where(rmin - dd > 0, rmin - dd, 0.0)
    got = _dense(_mma_mod().Filter(cols, vals, hs, rmin), n)
    ref = np.zeros((n, n))
    np.add.at(ref, (np.repeat(np.arange(n), 20), ii.reshape(-1)), w.reshape(-1))
    assert (ref > 0).sum(1).max() == 20          # the cut is exercised
    np.testing.assert_allclose(got, ref, rtol=0, atol=1e-15)


def test_filter_products_match_oracle(cuda):
    """applySensitivityFilter / applyDensityFilter against the oracle's products (1e-13)."""
    import jax_fem_gb300 as jf

    class P(jf.Problem):
        def get_tensor_map(self):
            return jf.LinearElastic(1.0, 0.3)

    prob = P(_jittered_box(8, 6, 4, 0.1, 2), vec=3, dim=3)
    fe = prob.fes[0]
    M = _mma_mod()
    H, Hs = M.compute_filter_kd_tree(fe)
    Ho, Hso, _ = omma.filter_kd_tree(np.mean(fe.points[fe.cells], axis=1),
                                   omma.cell_volume(fe.points, fe.cells, fe.shape_grads_ref, fe.quad_weights))
    rng = np.random.default_rng(5)
    n = fe.num_cells
    rho = rng.uniform(0.0005, 1.0, (n, 1))
    dJ = rng.standard_normal((n, 1))
    dvc = rng.standard_normal((2, n, 1))
    ft = {"H": H, "Hs": Hs}
    dJf, dvcf = M.applySensitivityFilter(ft, torch.tensor(rho, device=cuda), torch.tensor(dJ, device=cuda),
                                         torch.tensor(dvc, device=cuda))
    rJ, rv = omma.sensitivity_filter(Ho, Hso, rho.reshape(-1), dJ.reshape(-1), dvc.reshape(2, -1))
    np.testing.assert_allclose(dJf.cpu().numpy().reshape(-1), rJ, rtol=1e-13, atol=1e-13 * np.abs(rJ).max())
    np.testing.assert_allclose(dvcf.cpu().numpy().reshape(2, -1), rv, rtol=1e-13, atol=1e-13 * np.abs(rv).max())
    dens = M.applyDensityFilter(ft, torch.tensor(rho, device=cuda)).cpu().numpy().reshape(-1)
    np.testing.assert_allclose(dens, (Ho @ rho.reshape(-1)) / Hso, rtol=1e-13)


@pytest.mark.parametrize("m", [1, 2])
def test_mma_update_matches_oracle(cuda, m):
    """Four successive fem_mma_update calls (epochs 1-4: initial and adapted asymptotes) on
    n = 5000 variables against the oracle's mmasub; each step starts both sides from the same
    inputs.  xmma, low and upp agree to 1e-9."""
    M = _mma_mod()
    rng = np.random.default_rng(10 + m)
    n = 5000
    x = rng.uniform(0.2, 0.8, n)
    xold1, xold2 = x.copy(), x.copy()
    low, upp = np.ones(n), np.ones(n)
    xmin, xmax = np.zeros(n), np.ones(n)
    for epoch in range(1, 5):
        df0 = rng.standard_normal(n)
        fval = rng.uniform(-0.2, 0.2, m)
        dfdx = rng.uniform(-1, 1, (m, n)) / n
        mm = M.MMA()
        mm.setNumConstraints(m)
        mm.setNumDesignVariables(n)
        mm.setMinandMaxBoundsForDesignVariables(torch.tensor(xmin, device=cuda), torch.tensor(xmax, device=cuda))
        mm.epoch = epoch
        mm.xold1, mm.xold2 = torch.tensor(xold1, device=cuda), torch.tensor(xold2, device=cuda)
        mm.setLowerAndUpperAsymptotes(torch.tensor(low, device=cuda), torch.tensor(upp, device=cuda))
        mm.setScalingParams(1.0, np.zeros(m), 1e4 * np.ones(m), np.zeros(m))
        mm.setMoveLimit(0.2)
        mm.setObjectiveWithGradient(0.0, torch.tensor(df0, device=cuda))
        mm.setConstraintWithGradient(fval, torch.tensor(dfdx, device=cuda))
        mm.mmasub(torch.tensor(x, device=cuda))
        xg = mm.xmma.cpu().numpy().reshape(-1)
        lg, ug = (t.cpu().numpy().reshape(-1) for t in mm.getAsymptoteValues())
        xr, lr, ur = omma.mmasub(epoch, x, xold1, xold2, low, upp, xmin, xmax, 0.2, 0.0, df0, fval, dfdx,
                                 1.0, np.zeros(m), 1e4 * np.ones(m), np.zeros(m))
        np.testing.assert_allclose(lg, lr, rtol=0, atol=1e-13)
        np.testing.assert_allclose(ug, ur, rtol=0, atol=1e-13)
        assert np.abs(xg - xr).max() <= 1e-9, (epoch, np.abs(xg - xr).max())
        assert mm.newton_steps > 0
        xold2, xold1, x = xold1, x, xr
        low, upp = lr, ur


def test_optimize_three_iterations_matches_oracle_loop(cuda):
    """optimize() (filter + MMA on the GPU) for three iterations of the SIMP cantilever 12x6x3
    (vf 0.5, move limit 0.1) against the reference's loop run with the oracle's filter and mmasub
    on the same objective: the designs agree to 1e-7 after every iteration."""
    import cases
    import jax_fem_gb300 as jf
    M = _mma_mod()
    prob, _, _ = cases.simp_box(12, 6, 3)
    fe = prob.fes[0]
    opts = {"petsc_solver": {"ksp_type": "cg", "pc_type": "bjacobi", "rtol": 1e-12}, "rel_tol": 1e-10, "tol": 0.0}
    fwd = jf.ad_wrapper(prob, opts, opts)
    vf = 0.5
    n = fe.num_cells

    def objective(rho):
        th = torch.as_tensor(rho, dtype=torch.float64, device=cuda).reshape(n, 1).detach().requires_grad_(True)
        u = fwd(th)[0]
        J = torch.dot(prob._engine.f_ext, u.reshape(-1))
        J.backward()
        return J.item(), th.grad.detach()

    def cons(rho, it):
        r = torch.as_tensor(rho, dtype=torch.float64, device=cuda).reshape(-1)
        return np.array([r.mean().item() / vf - 1.0]), torch.full((1, n, 1), 1.0 / (n * vf), dtype=torch.float64,
                                                                  device=cuda)

    designs = []

    def objective_logged(rho):
        designs.append(torch.as_tensor(rho).detach().cpu().numpy().reshape(-1).copy())
        return objective(rho)

    rho_ini = vf * np.ones((n, 1))
    rho = M.optimize(fe, rho_ini, {"maxIters": 3, "movelimit": 0.1}, objective_logged, cons, 1)
    designs.append(rho.cpu().numpy().reshape(-1))

    # the same loop with the oracle's filter and MMA
    Ho, Hso, _ = omma.filter_kd_tree(np.mean(fe.points[fe.cells], axis=1),
                                   omma.cell_volume(fe.points, fe.cells, fe.shape_grads_ref, fe.quad_weights))
    x = rho_ini.reshape(-1).copy()
    xold1, xold2 = x.copy(), x.copy()
    low, upp = np.ones(n), np.ones(n)
    for it in range(1, 4):
        np.testing.assert_allclose(designs[it - 1], x, rtol=0, atol=1e-7)
        J, dJ = objective(x)
        vc, dvc = cons(x, it)
        dJf, dvcf = omma.sensitivity_filter(Ho, Hso, x, dJ.cpu().numpy().reshape(-1), dvc.cpu().numpy().reshape(1, -1))
        xn, low, upp = omma.mmasub(it, x, xold1, xold2, low, upp, np.zeros(n), np.ones(n), 0.1, J, dJf, vc, dvcf,
                                   1.0, np.zeros(1), 1e4 * np.ones(1), np.zeros(1))
        xold2, xold1, x = xold1, x, xn
    np.testing.assert_allclose(designs[3], x, rtol=0, atol=1e-7)
