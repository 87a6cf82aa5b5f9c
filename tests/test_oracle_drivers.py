"""CPU checks that pin the oracle's restatement of the nonlinear drivers (oracle/drivers.py:
arc_length_solver_disp_driven / _force_driven and dynamic_relax_solve, jax_fem/solver.py:559-1049)
independently of the GPU: properties the reference's algorithms guarantee, on small problems."""
import numpy as np
import pytest
import torch

from oracle import drivers as odr, fem as ofem, materials as omat, solve as osolve


def _box(n, tensor_map, stretch=None, traction=None):
    pts, cells = ofem.box_mesh(n, n, n, 1.0, 1.0, 1.0)
    left = lambda p: np.isclose(p[0], 0.0, atol=1e-5)
    right = lambda p: np.isclose(p[0], 1.0, atol=1e-5)
    zero = lambda p: 0.0
    if stretch is not None:
        bc = [[left] * 3 + [right] * 3, [0, 1, 2, 0, 1, 2], [zero] * 3 + [lambda p: stretch, zero, zero]]
    else:
        bc = [[left] * 3, [0, 1, 2], [zero] * 3]
    locs = [right] if traction is not None else None
    surf = None if traction is None else [lambda u, x: torch.tensor(traction, dtype=torch.float64)]
    return ofem.OracleProblem(pts, cells, 3, dirichlet_bc_info=bc, location_fns=locs, tensor_map=tensor_map,
                              surface_maps=surf)


def test_arc_length_linear_path_meets_constraint_and_direct_solve():
    """Displacement control on linear elasticity: every converged step satisfies the Crisfield
    constraint ||du||^2 + psi^2 dlam^2 ||q||^2 = Delta_l^2 (q the prescribed-displacement load
    vector, solver.py:559-640), the path is u = lam u_1 (linear problem), and at lam = 1 the
    solution equals the direct solve."""
    prob = _box(2, omat.linear_elastic(10.0, 0.3), stretch=0.3)
    delta_l, psi = 0.05, 1.0
    n = prob.num_total_dofs_all_vars
    ref = ofem.assign_bc(np.zeros(n), prob)
    ref2 = float(np.sum(ref ** 2))
    u, lam, du_dir, dlam_dir = np.zeros(n), 0.0, np.zeros(n), 0.0
    u1 = np.asarray(osolve.newton_solve(prob, {"spsolve_solver": {}})).reshape(-1)
    steps = 0
    while lam < 1.0 and steps < 200:
        u_new, lam_new, du_dir, dlam_dir = odr.arc_length_step(prob, u, lam, du_dir, dlam_dir, delta_l, psi)
        c = np.sum((u_new - u) ** 2) + psi ** 2 * (lam_new - lam) ** 2 * ref2
        assert abs(c - delta_l ** 2) <= 1e-8 * delta_l ** 2
        assert lam_new > lam                                            # the forward root is taken
        np.testing.assert_allclose(u_new, lam_new * u1, rtol=0, atol=1e-9 * np.abs(u1).max())
        u, lam = u_new, lam_new
        steps += 1
    assert lam >= 1.0 and steps > 1


def test_arc_length_driver_reaches_full_load():
    """The outer loop stops at the first lam >= 1 and records every step's lam, increasing."""
    prob = _box(2, omat.linear_elastic(10.0, 0.3), stretch=0.3)
    u, lam, lams = odr.arc_length(prob, "displacement", delta_l=0.1, psi=1.0)
    assert lam >= 1.0 and lams[-1] == lam and all(b > a for a, b in zip(lams, lams[1:]))
    assert all(x < 1.0 for x in lams[:-1])


@pytest.mark.parametrize("traction", [[0.0, 0.0, -0.2]])
def test_dynamic_relaxation_reaches_newton_solution(traction):
    """Dynamic relaxation (solver.py:918-1049) of a Neo-Hookean cube under an end traction stops
    at max|R| <= tol and lands on the oracle's Newton solution (1e-5 of max|u|)."""
    prob = _box(2, omat.neo_hookean(10.0, 0.3), traction=traction)
    q, it = odr.dynamic_relax(prob, tol=1e-7, nKMat=50, max_iters=50000)
    rows, _ = prob.bc_rows()
    r = prob.compute_residual(torch.from_numpy(q)).numpy().copy()
    r[rows] = 0.0
    assert np.abs(r).max() <= 1e-7 and it > 0
    newton = np.asarray(osolve.newton_solve(prob, {"spsolve_solver": {}, "rel_tol": 1e-12, "tol": 0.0})).reshape(-1)
    assert np.abs(q - newton).max() <= 1e-5 * np.abs(newton).max()
