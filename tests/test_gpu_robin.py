"""GPU parity of u-dependent (Robin) surface maps (problem.py:238-259; the pattern of
applications/robin_bc/example.py:64-80, there 5 u^2 on two faces) against the oracle, whose face
kernel differentiates the same map with torch.func.jacfwd."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _box(n):
    import jax_fem_gb300 as jf
    m = jf.box_mesh(n, n, n, 1.0, 1.0, 1.0)
    return m.points, m.cells_dict["hexahedron"]


def test_nonlinear_robin_poisson_vs_oracle(cuda):
    """Laplace on HEX8 5^3, u = 1 on x=0, source 10 sin(pi y), Robin map 5 u^2 on x=1 and y=1:
    the residual and tangent at a random state (1e-12) and the Newton solution (1e-10) match
    the oracle; the tangent is not cached across states (it depends on u)."""
    import jax_fem_gb300 as jf
    from oracle import fem as ofem, materials as omat, solve as osolve
    pts, cells = _box(5)
    left = lambda p: np.isclose(p[0], 0.0, atol=1e-5)
    right = lambda p: np.isclose(p[0], 1.0, atol=1e-5)
    top = lambda p: np.isclose(p[1], 1.0, atol=1e-5)
    bc = [[left], [0], [lambda p: 1.0]]

    class P(jf.Problem):
        def get_tensor_map(self):
            return jf.Laplace()

        def get_mass_map(self):
            return lambda u, x: np.array([-10.0 * np.sin(np.pi * x[1])])

        def get_surface_maps(self):
            return [lambda u, x: 5.0 * u ** 2, lambda u, x: 5.0 * u ** 2]

    prob = P(jf.Mesh(pts, cells), vec=1, dim=3, dirichlet_bc_info=bc, location_fns=[right, top])
    oprob = ofem.OracleProblem(pts, cells, 1, dirichlet_bc_info=bc, location_fns=[right, top],
                               tensor_map=omat.laplace(),
                               mass_map=lambda u, x: torch.stack([-10.0 * torch.sin(np.pi * x[1])]),
                               surface_maps=[lambda u, x: 5.0 * u ** 2, lambda u, x: 5.0 * u ** 2])
    eng = prob._engine
    u = np.random.default_rng(3).uniform(0.2, 1.0, eng.num_dofs)
    res = eng.residual(torch.tensor(u, device=cuda), apply_bc=False).cpu().numpy()
    ores = oprob.compute_residual(torch.tensor(u)).numpy()
    assert np.abs(res - ores).max() <= 1e-12 * np.abs(ores).max()
    prob.newton_update([torch.tensor(u, device=cuda).reshape(-1, 1)])
    A = jf.get_A(prob)
    oprob.newton_update(torch.tensor(u))
    Ao = ofem.assemble_petsc(oprob)
    assert np.abs(A.data.cpu().numpy() - Ao.data).max() <= 1e-12 * np.abs(Ao.data).max()
    opts = {"petsc_solver": {"ksp_type": "cg", "pc_type": "jacobi", "rtol": 1e-13}, "rel_tol": 1e-12, "tol": 0.0}
    sol = jf.solver(prob, opts)[0].reshape(-1).cpu().numpy()
    ref = np.asarray(osolve.newton_solve(oprob, {"spsolve_solver": {}, "rel_tol": 1e-13, "tol": 0.0})).reshape(-1)
    assert np.abs(sol - ref).max() <= 1e-10 * np.abs(ref).max()


def test_spring_support_elasticity_mixed_and_fp64(cuda):
    """Linear elasticity on HEX8 6^3 clamped at x=0 with a spring support and load on x=1:
    t(u, x) = 50 u + (0, 0, -x_1) (u-dependent surface map of degree 1, so the tangent is cached).
    FP64 and mixed solutions match the oracle's direct solve to 1e-9."""
    import jax_fem_gb300 as jf
    from oracle import fem as ofem, materials as omat, solve as osolve
    pts, cells = _box(6)
    left = lambda p: np.isclose(p[0], 0.0, atol=1e-5)
    right = lambda p: np.isclose(p[0], 1.0, atol=1e-5)
    zero = lambda p: 0.0
    bc = [[left] * 3, [0, 1, 2], [zero] * 3]

    class P(jf.Problem):
        def get_tensor_map(self):
            return jf.LinearElastic(100.0, 0.3)

        def get_surface_maps(self):
            return [lambda u, x: 50.0 * u + np.array([0.0, 0.0, -x[1]])]

    prob = P(jf.Mesh(pts, cells), vec=3, dim=3, dirichlet_bc_info=bc, location_fns=[right])
    oprob = ofem.OracleProblem(pts, cells, 3, dirichlet_bc_info=bc, location_fns=[right],
                               tensor_map=omat.linear_elastic(100.0, 0.3),
                               surface_maps=[lambda u, x: 50.0 * u + torch.stack([0.0 * x[1], 0.0 * x[1], -x[1]])])
    ref = np.asarray(osolve.newton_solve(oprob, {"spsolve_solver": {}, "rel_tol": 1e-13, "tol": 0.0})).reshape(-1)
    for precision in ("fp64", "mixed"):
        opts = {"petsc_solver": {"ksp_type": "cg", "pc_type": "bjacobi", "rtol": 1e-12}, "rel_tol": 1e-11,
                "tol": 0.0, "precision": precision}
        sol = jf.solver(prob, opts)[0].reshape(-1).cpu().numpy()
        assert np.abs(sol - ref).max() <= 1e-9 * np.abs(ref).max(), precision
