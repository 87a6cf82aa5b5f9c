"""Degenerate inputs through the public API on the GPU: every dof constrained (no free unknowns),
a single cell, and a zero right-hand side, in FP64 and mixed precision.  The reference's
solver() handles the same cases through its row-eliminated systems (solver.py:290-363,
402-409)."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _elastic(n, bc, surface=None, loc=None):
    import jax_fem_gb300 as jf
    m = jf.box_mesh(*n, 1.0, 1.0, 1.0)

    class P(jf.Problem):
        def get_tensor_map(self):
            return jf.LinearElastic(70e3, 0.3)

        def get_surface_maps(self):
            return [surface] if surface else []

    kw = {"location_fns": [loc]} if loc else {}
    return P(jf.Mesh(m.points, m.cells_dict["hexahedron"]), vec=3, dim=3, dirichlet_bc_info=bc, **kw)


def _opts(prec):
    return {"petsc_solver": {"ksp_type": "cg", "pc_type": "bjacobi", "rtol": 1e-12}, "rel_tol": 1e-12, "tol": 0.0,
            "precision": prec}


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_every_dof_constrained(cuda, prec):
    """All nodes carry Dirichlet values on all three components: the solution is the prescribed
    field, whatever the solver (no free unknowns)."""
    import jax_fem_gb300 as jf
    every = lambda p: True
    bc = [[every] * 3, [0, 1, 2], [lambda p: 0.01 * p[0], lambda p: -0.02 * p[1], lambda p: 0.0]]
    prob = _elastic((2, 2, 2), bc)
    sol = jf.solver(prob, _opts(prec))[0].cpu().numpy()
    pts = np.asarray(prob.mesh[0].points if isinstance(prob.mesh, list) else prob.mesh.points)
    want = np.stack([0.01 * pts[:, 0], -0.02 * pts[:, 1], 0.0 * pts[:, 2]], axis=1)
    assert np.abs(sol - want).max() <= 1e-15


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_single_cell(cuda, prec):
    """One HEX8 cell clamped on x = 0 and pulled on x = 1: mixed and FP64 agree (1e-9), and the
    solution matches the oracle's direct solve (1e-10)."""
    import jax_fem_gb300 as jf
    from oracle import fem as ofem, materials as omat, solve as osolve
    x0 = lambda p: np.isclose(p[0], 0.0, atol=1e-5)
    x1 = lambda p: np.isclose(p[0], 1.0, atol=1e-5)
    bc = [[x0] * 3, [0, 1, 2], [lambda p: 0.0] * 3]
    prob = _elastic((1, 1, 1), bc, surface=lambda u, x: np.array([10.0, 0.0, -5.0]), loc=x1)
    sol = jf.solver(prob, _opts(prec))[0].reshape(-1).cpu().numpy()
    m = jf.box_mesh(1, 1, 1, 1.0, 1.0, 1.0)
    oprob = ofem.OracleProblem(m.points, m.cells_dict["hexahedron"], 3, dirichlet_bc_info=bc, location_fns=[x1],
                               tensor_map=omat.linear_elastic(70e3, 0.3),
                               surface_maps=[lambda u, x: torch.tensor([10.0, 0.0, -5.0])])
    ref = np.asarray(osolve.newton_solve(oprob, {"spsolve_solver": {}, "rel_tol": 1e-12, "tol": 0.0})).reshape(-1)
    assert np.abs(sol - ref).max() <= 1e-10 * np.abs(ref).max()


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_zero_load_gives_zero_solution(cuda, prec):
    """No load and homogeneous Dirichlet values: the solver returns exactly zero (a zero right-hand
    side must not divide by its norm)."""
    import jax_fem_gb300 as jf
    x0 = lambda p: np.isclose(p[0], 0.0, atol=1e-5)
    bc = [[x0] * 3, [0, 1, 2], [lambda p: 0.0] * 3]
    prob = _elastic((3, 2, 2), bc)
    sol = jf.solver(prob, _opts(prec))[0]
    assert torch.isfinite(sol).all() and sol.abs().max().item() == 0.0
