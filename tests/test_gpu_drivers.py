"""GPU parity of the arc-length (displacement and force control) and dynamic-relaxation drivers
(solver.py:559-1049) against the oracle's restatement of the same loops (scipy direct solves of
the row-eliminated systems)."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _neo(n, traction=None, stretch=False):
    import jax_fem_gb300 as jf
    from oracle import fem as ofem, materials as omat
    m = jf.box_mesh(n, n, n, 1.0, 1.0, 1.0)
    pts, cells = m.points, m.cells_dict["hexahedron"]
    left = lambda p: np.isclose(p[0], 0.0, atol=1e-5)
    right = lambda p: np.isclose(p[0], 1.0, atol=1e-5)
    zero = lambda p: 0.0
    if stretch:
        bc = [[left] * 3 + [right] * 3, [0, 1, 2, 0, 1, 2], [zero] * 3 + [lambda p: 0.3, zero, zero]]
    else:
        bc = [[left] * 3, [0, 1, 2], [zero] * 3]
    locs = [right] if traction is not None else None

    class P(jf.Problem):
        def get_tensor_map(self):
            return jf.NeoHookean(10.0, 0.3)

        if traction is not None:
            def get_surface_maps(self):
                return [lambda u, x: np.array(traction)]

    prob = P(jf.Mesh(pts, cells), vec=3, dim=3, dirichlet_bc_info=bc, location_fns=locs)
    oprob = ofem.OracleProblem(pts, cells, 3, dirichlet_bc_info=bc, location_fns=locs,
                               tensor_map=omat.neo_hookean(10.0, 0.3),
                               surface_maps=None if traction is None else
                               [lambda u, x: torch.tensor(traction, dtype=torch.float64)])
    return prob, oprob


def test_arc_length_displacement_vs_oracle(cuda):
    """Displacement-controlled arc length (Delta_l 0.1, psi 1) on Neo-Hookean 3^3 with x=1 u_x = 0.3
    at full load: the lambda path matches the oracle's step for step (1e-8) and the polished
    full-load solution matches the oracle's Newton polish (1e-9)."""
    import jax_fem_gb300 as jf
    from oracle import drivers as odr, solve as osolve
    prob, oprob = _neo(3, stretch=True)
    sol, info = jf.solver(prob, {"arc_length": {"control": "displacement", "Delta_l": 0.1, "psi": 1.0,
                                                "return_info": True, "newton": {"rel_tol": 1e-12, "tol": 1e-11},
                                                "linear": {"petsc_solver": {"ksp_type": "cg", "pc_type": "bjacobi",
                                                                            "rtol": 1e-13}}}})
    u_o, lam_o, lams_o = odr.arc_length(oprob, "displacement", delta_l=0.1, psi=1.0)
    lams = [h["lam"] for h in info["history"]]
    assert len(lams) == len(lams_o) and info["polished"]
    np.testing.assert_allclose(lams, lams_o, rtol=0, atol=1e-8)
    ref = np.asarray(osolve.newton_solve(oprob, {"spsolve_solver": {}, "rel_tol": 1e-12, "tol": 0.0,
                                                 "initial_guess": u_o})).reshape(-1)
    got = sol[0].reshape(-1).cpu().numpy()
    assert np.abs(got - ref).max() <= 1e-9 * np.abs(ref).max()


def test_arc_length_force_vs_oracle(cuda):
    """Force-controlled arc length (counter-load q_aux = -get_q_vec, Delta_l 0.1, psi 0.5) on
    Neo-Hookean 3^3 under an end traction: lambda path (1e-8) and polished solution (1e-9)."""
    import jax_fem_gb300 as jf
    from oracle import drivers as odr, solve as osolve
    prob, oprob = _neo(3, traction=[0.0, 0.0, -0.4])
    q_aux = -jf.get_q_vec(prob)
    sol, info = jf.solver(prob, {"arc_length": {"control": "force", "q_vec_aux": q_aux, "Delta_l": 0.1,
                                                "psi": 0.5, "return_info": True,
                                                "newton": {"rel_tol": 1e-12, "tol": 1e-11},
                                                "linear": {"petsc_solver": {"ksp_type": "cg", "pc_type": "bjacobi",
                                                                            "rtol": 1e-13}}}})
    u_o, lam_o, lams_o = odr.arc_length(oprob, "force", delta_l=0.1, psi=0.5, q_aux=q_aux.cpu().numpy())
    lams = [h["lam"] for h in info["history"]]
    assert len(lams) == len(lams_o) and info["polished"]
    np.testing.assert_allclose(lams, lams_o, rtol=0, atol=1e-8)
    ref = np.asarray(osolve.newton_solve(oprob, {"spsolve_solver": {}, "rel_tol": 1e-12, "tol": 0.0,
                                                 "initial_guess": u_o})).reshape(-1)
    got = sol[0].reshape(-1).cpu().numpy()
    assert np.abs(got - ref).max() <= 1e-9 * np.abs(ref).max()


def test_dynamic_relaxation_vs_oracle(cuda):
    """Dynamic relaxation (tol 1e-6 on max |R|) of Neo-Hookean 3^3 under an end traction: the
    GPU loop (fused kernels) and the oracle's loop take the same number of iterations (+-2) and
    end within 1e-6 of each other and of the Newton solution (relative to max|u|)."""
    import jax_fem_gb300 as jf
    from oracle import drivers as odr
    prob, oprob = _neo(3, traction=[0.0, 0.0, -0.2])
    sol = jf.solver(prob, {"dynamic_relax": {"tol": 1e-6, "nKMat": 50, "info": False, "info_force": False,
                                             "max_iters": 20000}})[0].reshape(-1).cpu().numpy()
    it = prob.dr_info["iterations"]
    q_o, it_o = odr.dynamic_relax(oprob, tol=1e-6, nKMat=50, max_iters=20000)
    assert prob.dr_info["error"] <= 1e-6 and abs(it - it_o) <= 2, (it, it_o)
    scale = np.abs(q_o).max()
    assert np.abs(sol - q_o).max() <= 1e-6 * scale
    newton = jf.solver(prob, {"petsc_solver": {"ksp_type": "cg", "pc_type": "bjacobi", "rtol": 1e-12},
                              "rel_tol": 1e-11, "tol": 0.0})[0].reshape(-1).cpu().numpy()
    assert np.abs(sol - newton).max() <= 1e-4 * scale
