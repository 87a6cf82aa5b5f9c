"""GPU parity tests: the CUDA path (through the C ABI) against the CPU oracle and the
reference's FEniCSx gold fixtures.  Tolerances are stated per test."""
import importlib

import numpy as np
import pytest
import torch

from conftest import golden

pytestmark = pytest.mark.gpu


def _cube(cuda):
    import cases
    return cases.cube_elasticity(golden("linear_elasticity_cube"))


def test_pattern_bit_exact(cuda):
    """CSR pattern (indptr/indices after coalescing) equals the PETSc COO pattern of I/J."""
    from oracle import fem as ofem
    prob, oprob = _cube(cuda)
    eng = prob._engine
    ip, ix = ofem.coo_pattern(oprob.I, oprob.J, oprob.num_total_dofs_all_vars)
    assert eng.nnz == len(ix) == 268119
    np.testing.assert_array_equal(eng.indptr.cpu().numpy(), ip)
    np.testing.assert_array_equal(eng.scalar_indices().cpu().numpy(), ix)


def test_assembled_values_fp64(cuda):
    """get_A after newton_update: PETSc zeroRows semantics, values within 1e-12 relative."""
    import jax_fem_gb300 as jf
    from oracle import fem as ofem
    prob, oprob = _cube(cuda)
    rng = np.random.default_rng(3)
    u = rng.standard_normal(oprob.num_total_dofs_all_vars) * 1e-3
    prob.newton_update([torch.tensor(u, device=cuda).reshape(-1, 3)])
    A = jf.get_A(prob)
    oprob.newton_update(torch.tensor(u))
    Ao = ofem.assemble_petsc(oprob)
    a = A.data.cpu().numpy()
    scale = np.abs(Ao.data).max()
    assert np.abs(a - Ao.data).max() <= 1e-12 * scale
    np.testing.assert_array_equal(A.indices.cpu().numpy(), Ao.indices)


def test_assembled_values_fp32(cuda):
    import jax_fem_gb300 as jf
    from oracle import fem as ofem
    prob, oprob = _cube(cuda)
    eng = prob._engine
    A32 = eng.tangent(torch.zeros(eng.num_dofs, dtype=torch.float64, device=cuda), jf._lib.FEM_F32,
                      jf._lib.FEM_BC_ROWS, cache=False)
    oprob.newton_update(torch.zeros(oprob.num_total_dofs_all_vars))
    Ao = ofem.assemble_petsc(oprob)
    scale = np.abs(Ao.data).max()
    assert np.abs(A32.data.double().cpu().numpy() - Ao.data).max() <= 2e-6 * scale


def test_residual_matches_oracle(cuda):
    prob, oprob = _cube(cuda)
    rng = np.random.default_rng(5)
    u = rng.standard_normal(oprob.num_total_dofs_all_vars) * 1e-3
    r = prob.compute_residual([torch.tensor(u, device=cuda).reshape(-1, 3)])[0].reshape(-1).cpu().numpy()
    ro = oprob.compute_residual(torch.tensor(u)).numpy()
    assert np.abs(r - ro).max() <= 1e-12 * np.abs(ro).max()


def test_spmv_matches_scipy(cuda):
    import jax_fem_gb300 as jf
    from oracle import fem as ofem
    prob, oprob = _cube(cuda)
    eng = prob._engine
    A = eng.tangent(torch.zeros(eng.num_dofs, dtype=torch.float64, device=cuda), jf._lib.FEM_F64,
                    jf._lib.FEM_BC_ROWS, cache=False)
    oprob.newton_update(torch.zeros(oprob.num_total_dofs_all_vars))
    Ao = ofem.assemble_petsc(oprob)
    x = np.random.default_rng(1).standard_normal(Ao.shape[0])
    y = A.matvec(torch.tensor(x, device=cuda)).cpu().numpy()
    yo = Ao @ x
    assert np.abs(y - yo).max() <= 1e-12 * np.abs(yo).max()
    A32 = eng.tangent(torch.zeros(eng.num_dofs, dtype=torch.float64, device=cuda), jf._lib.FEM_F32,
                      jf._lib.FEM_BC_ROWS, cache=False)
    y32 = A32.matvec(torch.tensor(x, device=cuda)).double().cpu().numpy()
    assert np.abs(y32 - yo).max() <= 1e-5 * np.abs(yo).max()


def test_cube_solution_gold_and_oracle(cuda):
    """test_linear_elasticity_cube.py:73-83 (decimal 5) and the oracle's direct solve (1e-10)."""
    import jax_fem_gb300 as jf
    from oracle import solve as osolve
    g = golden("linear_elasticity_cube")
    prob, oprob = _cube(cuda)
    sol = jf.solver(prob)[0].cpu().numpy()                       # default: jax_solver (BiCGStab + Jacobi)
    np.testing.assert_array_almost_equal(g["sol"], sol, decimal=5)
    osol = osolve.newton_solve(oprob, {"spsolve_solver": {}})
    sol_cg = jf.solver(prob, {"petsc_solver": {"ksp_type": "cg", "pc_type": "bjacobi", "rtol": 1e-13}})[0]
    assert np.abs(sol_cg.cpu().numpy() - osol).max() <= 1e-10 * np.abs(osol).max()
    assert np.abs(sol - osol).max() <= 1e-7 * np.abs(osol).max()


def test_mixed_bicgstab_newton_refinement(cuda):
    """precision='mixed' with the reference's default jax_solver (BiCGStab + Jacobi): the
    BiCGStab runs in FP32 on the sliced FP32 copy and Newton's FP64 residual refines it; at
    rel_tol 1e-11 (the FP64 residual of this cube bottoms out near 2.5e-12) the solution matches
    the oracle's direct solve to 1e-8 relative."""
    import jax_fem_gb300 as jf
    from oracle import solve as osolve
    prob, oprob = _cube(cuda)
    sol = jf.solver(prob, {"jax_solver": {}, "precision": "mixed", "rel_tol": 1e-11, "tol": 0.0})[0].cpu().numpy()
    osol = osolve.newton_solve(oprob, {"spsolve_solver": {}})
    assert np.abs(sol - osol).max() <= 1e-8 * np.abs(osol).max()


def test_bicgstab_matches_jax_iteration(cuda):
    """fem_bicgstab follows jax.scipy's BiCGStab: same iteration count and iterate as the restated loop."""
    import jax_fem_gb300 as jf
    from oracle import fem as ofem, solve as osolve
    prob, oprob = _cube(cuda)
    eng = prob._engine
    z = torch.zeros(eng.num_dofs, dtype=torch.float64, device=cuda)
    res = eng.residual(z, apply_bc=True)
    A = eng.tangent(z, jf._lib.FEM_F64, jf._lib.FEM_BC_ROWS, cache=False)
    b = -res
    oprob.newton_update(torch.zeros(oprob.num_total_dofs_all_vars))
    Ao = ofem.assemble_petsc(oprob)
    bo = b.cpu().numpy()
    d = Ao.diagonal()
    # Same iterate after a fixed number of steps.  With the Jacobi preconditioner this
    # recurrence amplifies rounding ~100x per step (on the CPU alone, v/d versus v*(1/d)
    # already differs by 3e-5 after 10 steps), so preconditioned iterates are compared
    # over the first steps and the unpreconditioned iteration over 10 steps.
    for k, pc, tol in ((1, True, 1e-13), (2, True, 1e-11), (3, True, 1e-8), (10, False, 1e-12)):
        x = torch.zeros_like(b)
        it, rn, st = eng.krylov("bicgstab", A, b, x, jf._lib.FEM_PC_JACOBI if pc else jf._lib.FEM_PC_NONE,
                                1e-10, 1e-10, k)
        xo, ito = osolve.bicgstab_jax(Ao, bo, None, (lambda v: v / d) if pc else None, 1e-10, 1e-10, k)
        assert it == ito == k and st == jf._lib.FEM_SOLVE_MAXITER
        assert np.abs(x.cpu().numpy() - xo).max() <= tol * np.abs(xo).max()
    # full solve: same stopping rule, iteration counts within rounding drift
    x = torch.zeros_like(b)
    it, rn, st = eng.krylov("bicgstab", A, b, x, jf._lib.FEM_PC_JACOBI, 1e-10, 1e-10, 10000)
    xo, ito = osolve.bicgstab_jax(Ao, bo, None, lambda v: v / d, 1e-10, 1e-10, 10000)
    assert st == 0 and abs(it - ito) <= max(3, 0.1 * ito)
    assert rn <= 1e-10 * np.linalg.norm(bo) * (1 + 1e-12)
    assert np.abs(x.cpu().numpy() - xo).max() <= 1e-6 * np.abs(xo).max()


def test_poisson_gold(cuda):
    import cases
    import jax_fem_gb300 as jf
    g = golden("linear_poisson")
    prob, _ = cases.poisson(g)
    sol = jf.solver(prob)[0].cpu().numpy()
    np.testing.assert_array_almost_equal(g["sol"], sol, decimal=5)


@pytest.mark.parametrize("pc", ["jacobi", "bjacobi", "none"])
def test_poisson_mixed_vec1(cuda, pc):
    """The mixed CG on a scalar problem (vec 1: the generic double-float update and direction
    kernels, not the 32-node tiles): the Poisson gold fixture (decimal 5), the oracle's direct
    solve (1e-9 relative) and the FP64 CG (1e-10), for each preconditioner."""
    import cases
    import jax_fem_gb300 as jf
    from oracle import solve as osolve
    g = golden("linear_poisson")
    prob, oprob = cases.poisson(g)
    lin = {"petsc_solver": {"ksp_type": "cg", "pc_type": pc, "rtol": 1e-12}, "rel_tol": 1e-12, "tol": 0.0}
    s64 = jf.solver(prob, lin)[0].cpu().numpy()
    smx = jf.solver(prob, dict(lin, precision="mixed"))[0].cpu().numpy()
    np.testing.assert_array_almost_equal(g["sol"], smx, decimal=5)
    osol = np.asarray(osolve.newton_solve(oprob, {"spsolve_solver": {}})).reshape(smx.shape)
    assert np.abs(smx - osol).max() <= 1e-9 * np.abs(osol).max()
    assert np.abs(smx - s64).max() <= 1e-10 * np.abs(s64).max()


def test_cylinder_gold_and_area(cuda):
    """test_linear_elasticity_cylinder.py:113-132: decimal 3 solution, decimal 4 area."""
    import cases
    import jax_fem_gb300 as jf
    g = golden("linear_elasticity_cylinder")
    prob, _ = cases.cylinder_elasticity(g)
    sol = jf.solver(prob, {"petsc_solver": {"ksp_type": "cg", "pc_type": "bjacobi", "rtol": 1e-12}})[0]
    np.testing.assert_array_almost_equal(g["sol"], sol.cpu().numpy(), decimal=3)
    _, nanson = prob._engine.face_quad_points(prob.boundary_inds_list[0])
    np.testing.assert_almost_equal(g["surface_area"][0], nanson.sum().item(), decimal=4)


def test_hyperelastic_gold_and_traction(cuda):
    """test_hyper_elasticity.py:109-127: decimal 5 solution and top traction."""
    import cases
    import jax_fem_gb300 as jf
    g = golden("hyperelasticity")
    prob, _, _ = cases.hyperelastic(g)
    sol = jf.solver(prob, {"petsc_solver": {"ksp_type": "cg", "pc_type": "bjacobi", "rtol": 1e-12}})[0]
    np.testing.assert_array_almost_equal(g["sol"], sol.cpu().numpy(), decimal=5)
    fe = prob.fes[0]
    top = fe.get_boundary_conditions_inds([cases._top])[0]
    fg, nanson = fe.get_face_shape_grads(top)
    cells = torch.as_tensor(fe.cells, device=cuda)[torch.as_tensor(top[:, 0], device=cuda)]
    ug = torch.einsum("fnv,fqnd->fqvd", sol[cells], fg)
    F = ug + torch.eye(3, dtype=torch.float64, device=cuda)
    E, nu = 1e3, 0.3
    mu, kappa = E / (2 * (1 + nu)), E / (3 * (1 - 2 * nu))
    J = torch.linalg.det(F)
    H = torch.linalg.inv(F).transpose(-1, -2)
    I1 = (F * F).sum((-1, -2))
    P = mu * J[..., None, None] ** (-2 / 3) * (F - I1[..., None, None] / 3 * H) + kappa * (J * (J - 1))[..., None, None] * H
    trac = (P[..., :, 2] * nanson[..., None]).sum((0, 1))
    np.testing.assert_almost_equal(g["traction"][0], trac[2].item(), decimal=5)


def test_plasticity_gold(cuda):
    """test_plasticity.py:129-161: 5 load steps, decimal 5 solution and decimal 3 averaged stress."""
    import cases
    import jax_fem_gb300 as jf
    g = golden("plasticity")
    prob, bc, disps = cases.plasticity(g)
    avg = []
    sol = None
    for d in disps:
        bc[2][-1] = (lambda p, d=d: d)
        prob.fes[0].update_Dirichlet_boundary_conditions(bc)
        sol = jf.solver(prob, {"petsc_solver": {"ksp_type": "cg", "pc_type": "bjacobi", "rtol": 1e-12}})[0]
        prob.update_stress_strain(sol)
        avg.append(prob.compute_avg_stress()[2, 2].item())
    np.testing.assert_array_almost_equal(g["sol"], sol.cpu().numpy(), decimal=5)
    np.testing.assert_array_almost_equal(g["avg_stresses"], np.array(avg), decimal=3)


def _simp_grad(prob, theta_np, cuda, opts, adj):
    import jax_fem_gb300 as jf
    theta = torch.tensor(theta_np, device=cuda, requires_grad=True)
    fwd = jf.ad_wrapper(prob, opts, adj)
    sol = fwd(theta)[0]
    J = torch.dot(prob._engine.f_ext, sol.reshape(-1))
    J.backward()
    return sol.detach(), J.item(), theta.grad.detach().cpu().numpy()


def test_simp_adjoint_vs_oracle_and_fd(cuda):
    """ad_wrapper gradient vs the oracle's implicit_vjp (torch AD through the restated residual)
    within 1e-9 relative, and vs central finite differences (h=1e-6) within 1e-5 relative."""
    import cases
    from oracle import solve as osolve
    prob, oprob, theta_np = cases.simp_box(6, 3, 2)
    opts = {"petsc_solver": {"ksp_type": "cg", "pc_type": "jacobi", "rtol": 1e-13}}
    sol, J, g = _simp_grad(prob, theta_np, cuda, opts, opts)
    oprob.internal_vars = cases.oracle_set_params(oprob, torch.tensor(theta_np))
    osol = osolve.newton_solve(oprob, {"spsolve_solver": {}})
    f = prob._engine.f_ext.cpu().numpy()
    assert np.abs(sol.cpu().numpy() - osol).max() <= 1e-10 * np.abs(osol).max()
    fo = f.copy()
    fo[oprob.bc_rows()[0]] = 0.0
    g_or, _ = osolve.implicit_vjp(oprob, osol, theta_np, cases.oracle_set_params, fo)
    assert np.abs(g - g_or).max() <= 1e-9 * np.abs(g_or).max()
    import jax_fem_gb300 as jf
    rng = np.random.default_rng(0)
    h = 1e-6
    for c in rng.choice(len(theta_np), size=5, replace=False):
        vals = []
        for s in (+1, -1):
            tp = theta_np.copy()
            tp[c, 0] += s * h
            prob.set_params(torch.tensor(tp, device=cuda))
            u = jf.solver(prob, opts)[0]
            vals.append(torch.dot(prob._engine.f_ext, u.reshape(-1)).item())
        fd = (vals[0] - vals[1]) / (2 * h)
        assert abs(fd - g[c, 0]) <= 1e-5 * np.abs(g).max()


@pytest.mark.parametrize("mode", ["mixed", "mixed_ssym", "mixed_sym"])
def test_mixed_precision_matches_fp64(cuda, mode):
    """Mixed (DF48 matrix, double-float CG, FP64 reliable updates) vs FP64: solution, objective,
    gradient.  'mixed' runs on the general sliced storage, 'mixed_ssym' on this machine mesh's
    structured symmetric storage, 'mixed_sym' on the upper-block storage of the general pattern."""
    import cases
    prob, _, theta_np = cases.simp_box(12, 6, 3)
    o64 = {"petsc_solver": {"ksp_type": "cg", "pc_type": "bjacobi", "rtol": 1e-12}, "rel_tol": 1e-12, "tol": 0.0}
    omx = dict(o64, precision=mode)
    a64 = {"petsc_solver": {"ksp_type": "cg", "pc_type": "bjacobi", "rtol": 1e-12}}
    amx = dict(a64, precision=mode)
    s64, J64, g64 = _simp_grad(prob, theta_np, cuda, o64, a64)
    eng = prob._engine
    eng.solve_log.clear()
    smx, Jmx, gmx = _simp_grad(prob, theta_np, cuda, omx, amx)
    want = {"mixed": "df48+fp64", "mixed_ssym": "ssym-df48+fp64", "mixed_sym": "sym-df48+fp64"}[mode]
    assert all(r["precision"] == want for r in eng.solve_log if r["method"] == "cg-refined"), eng.solve_log
    assert (smx - s64).abs().max().item() <= 1e-9 * s64.abs().max().item()
    assert abs(Jmx - J64) <= 1e-10 * abs(J64)
    assert np.abs(gmx - g64).max() <= 1e-8 * np.abs(g64).max()


def test_mixed_refine_delta_large_converges(cuda):
    """refine_delta = 0.9: each reliable update then cuts the squared true residual by only about
    0.81, which must count as progress (no FEM_SOLVE_STAGNATED on a converging solve); forward and
    adjoint solves converge and match FP64 like the default delta."""
    import cases
    prob, _, theta_np = cases.simp_box(12, 6, 3)
    o64 = {"petsc_solver": {"ksp_type": "cg", "pc_type": "bjacobi", "rtol": 1e-12}, "rel_tol": 1e-12, "tol": 0.0}
    a64 = {"petsc_solver": {"ksp_type": "cg", "pc_type": "bjacobi", "rtol": 1e-12}}
    s64, J64, g64 = _simp_grad(prob, theta_np, cuda, o64, a64)
    eng = prob._engine
    eng.solve_log.clear()
    smx, Jmx, gmx = _simp_grad(prob, theta_np, cuda, dict(o64, precision="mixed", refine_delta=0.9),
                               dict(a64, precision="mixed", refine_delta=0.9))
    refined = [r for r in eng.solve_log if r["method"] == "cg-refined"]
    assert len(refined) >= 2 and all(r["status"] == "converged" for r in refined), refined
    assert all(r["updates"] > 5 for r in refined)   # delta 0.9: many small replacements
    assert (smx - s64).abs().max().item() <= 1e-9 * s64.abs().max().item()
    assert np.abs(gmx - g64).max() <= 1e-8 * np.abs(g64).max()


@pytest.mark.parametrize("n", [(1, 1, 1), (3, 1, 1), (4, 2, 1), (3, 3, 3), (5, 3, 2)])
def test_small_and_ragged_meshes(cuda, n):
    """Meshes of 8, 16, 30, 64 and 72 nodes: below one 32-node tile (the update kernels' partial
    tile only), exactly two tiles (no partial tile) and a ragged last tile.  FP64 and mixed
    solutions and the mixed gradient against the oracle's direct solve and implicit_vjp (1e-10 /
    1e-9 / 1e-8 relative)."""
    import cases
    from oracle import solve as osolve
    prob, oprob, theta_np = cases.simp_box(*n)
    oprob.internal_vars = cases.oracle_set_params(oprob, torch.tensor(theta_np))
    osol = osolve.newton_solve(oprob, {"spsolve_solver": {}})
    fo = prob._engine.f_ext.cpu().numpy().copy()
    fo[oprob.bc_rows()[0]] = 0.0
    g_or, _ = osolve.implicit_vjp(oprob, osol, theta_np, cases.oracle_set_params, fo)
    scale = np.abs(osol).max()
    for mode, tol in (("fp64", 1e-10), ("mixed", 1e-9)):
        lin = {"petsc_solver": {"ksp_type": "cg", "pc_type": "bjacobi", "rtol": 1e-12}}
        if mode == "mixed":
            lin["precision"] = "mixed"
        sol, _, g = _simp_grad(prob, theta_np, cuda, dict(lin, rel_tol=1e-12, tol=0.0), lin)
        assert np.abs(sol.cpu().numpy() - osol).max() <= tol * scale, mode
        assert np.abs(g - g_or).max() <= 1e-8 * np.abs(g_or).max(), mode


@pytest.mark.parametrize("mode", ["mixed", "mixed32"])
@pytest.mark.parametrize("load", [1e-30, 1e25])
def test_mixed_precision_extreme_scaling(cuda, load, mode):
    """Loads of 1e-30 and 1e25: the FP32-based CG's residual products would fall below FP32's
    normal range (or above its maximum) without the solvers' power-of-two vector scaling.  Mixed
    (double-float) and mixed32 (FP32) solution and gradient against FP64 (1e-9 / 1e-8 relative);
    Newton's absolute tolerance off."""
    import cases
    prob, _, theta_np = cases.simp_box(6, 3, 2, load=load)
    lin = {"petsc_solver": {"ksp_type": "cg", "pc_type": "bjacobi", "rtol": 1e-12}}
    s64, _, g64 = _simp_grad(prob, theta_np, cuda, dict(lin, rel_tol=1e-12, tol=0.0), lin)
    lmx = dict(lin, precision=mode)
    smx, _, gmx = _simp_grad(prob, theta_np, cuda, dict(lmx, rel_tol=1e-12, tol=0.0), lmx)
    assert np.isfinite(smx.cpu().numpy()).all() and np.isfinite(gmx).all()
    assert (smx - s64).abs().max().item() <= 1e-9 * s64.abs().max().item()
    assert np.abs(gmx - g64).max() <= 1e-8 * np.abs(g64).max()


def test_tet10_pattern_and_values(cuda):
    """TET10 (Kuhn split) pattern bit-exact and FP64 tangent within 1e-12 of the oracle."""
    import jax_fem_gb300 as jf
    from oracle import fem as ofem, materials as omat
    m = jf.box_mesh_tet10(3, 2, 2, 1.0, 1.0, 1.0)
    pts, cells = m.points, m.cells_dict["tetra10"]
    left = lambda p: np.isclose(p[0], 0.0, atol=1e-5)
    bc = [[left] * 3, [0, 1, 2], [lambda p: 0.0] * 3]

    class P(jf.Problem):
        def get_tensor_map(self):
            return jf.LinearElastic(1.0, 0.3)

    prob = P(jf.Mesh(pts, cells), vec=3, dim=3, ele_type="TET10", dirichlet_bc_info=bc)
    oprob = ofem.OracleProblem(pts, cells, 3, ele_type="TET10", dirichlet_bc_info=bc,
                               tensor_map=omat.linear_elastic(1.0, 0.3))
    eng = prob._engine
    ip, ix = ofem.coo_pattern(oprob.I, oprob.J, oprob.num_total_dofs_all_vars)
    np.testing.assert_array_equal(eng.indptr.cpu().numpy(), ip)
    np.testing.assert_array_equal(eng.scalar_indices().cpu().numpy(), ix)
    u = np.random.default_rng(2).standard_normal(oprob.num_total_dofs_all_vars) * 1e-2
    prob.newton_update([torch.tensor(u, device=cuda).reshape(-1, 3)])
    A = jf.get_A(prob)
    oprob.newton_update(torch.tensor(u))
    Ao = ofem.assemble_petsc(oprob)
    assert np.abs(A.data.cpu().numpy() - Ao.data).max() <= 1e-12 * np.abs(Ao.data).max()


def test_neo_hookean_tangent_matches_ad(cuda):
    """Hand-derived Neo-Hookean tangent vs the oracle's jacfwd(grad psi) at a deformed state (1e-11)."""
    import cases
    import jax_fem_gb300 as jf
    from oracle import fem as ofem
    g = golden("hyperelasticity")
    prob, oprob, _ = cases.hyperelastic(g)
    u = np.random.default_rng(4).standard_normal(oprob.num_total_dofs_all_vars) * 5e-2
    prob.newton_update([torch.tensor(u, device=cuda).reshape(-1, 3)])
    A = jf.get_A(prob)
    oprob.newton_update(torch.tensor(u))
    Ao = ofem.assemble_petsc(oprob)
    assert np.abs(A.data.cpu().numpy() - Ao.data).max() <= 1e-11 * np.abs(Ao.data).max()


def test_j2_tangent_matches_ad(cuda):
    """J2 consistent tangent (plastic branch active) vs the oracle's jacfwd of the return map."""
    import cases
    import jax_fem_gb300 as jf
    from oracle import fem as ofem, materials as omat
    g = golden("plasticity")
    prob, bc, disps = cases.plasticity(g)
    rng = np.random.default_rng(6)
    C, nq = prob.num_cells, prob.fes[0].num_quads
    sig = rng.standard_normal((C, nq, 3, 3)) * 100.0
    sig = 0.5 * (sig + np.swapaxes(sig, -1, -2))
    eps = rng.standard_normal((C, nq, 3, 3)) * 1e-3
    eps = 0.5 * (eps + np.swapaxes(eps, -1, -2))
    prob.internal_vars = [torch.tensor(sig, device=cuda), torch.tensor(eps, device=cuda)]
    u = rng.standard_normal(prob.num_total_dofs_all_vars) * 1e-2
    prob.newton_update([torch.tensor(u, device=cuda).reshape(-1, 3)])
    A = jf.get_A(prob)
    _, rmap = omat.j2_maps(70e3, 0.3, 250.0)
    oprob = ofem.OracleProblem(g["points"], g["cells"], 3, dirichlet_bc_info=bc, tensor_map=rmap)
    oprob.internal_vars = [torch.tensor(sig), torch.tensor(eps)]
    oprob.newton_update(torch.tensor(u))
    Ao = ofem.assemble_petsc(oprob)
    assert np.abs(A.data.cpu().numpy() - Ao.data).max() <= 1e-10 * np.abs(Ao.data).max()


def test_nan_input_is_reported(cuda):
    """A NaN design variable (host-made fault) ends the solve with an error, not a hang."""
    import cases
    import jax_fem_gb300 as jf
    prob, _, theta_np = cases.simp_box(4, 2, 2)
    theta_np = theta_np.copy()
    theta_np[3, 0] = np.nan
    prob.set_params(torch.tensor(theta_np, device=cuda))
    with pytest.raises((FloatingPointError, AssertionError, RuntimeError)):
        jf.solver(prob, {"petsc_solver": {"ksp_type": "cg", "pc_type": "jacobi", "rtol": 1e-10}})


def test_bounded_wait_reports_and_context_survives(cuda):
    """The bulk-copy kernels' bounded mbarrier wait, made to run out on a phase that nothing
    completes (fem_selftest_bounded_wait): the call returns FEM_ERR_DEVICE with the fault message
    after ~2 s instead of hanging, and the context still runs a mixed solve to the oracle's answer."""
    import ctypes
    import time
    import cases
    import jax_fem_gb300 as jf
    from oracle import solve as osolve
    L = jf._lib
    nb = ctypes.c_size_t()
    L.call("fem_krylov_workspace", 0, L.FEM_F64, ctypes.byref(nb))
    ws = torch.empty(nb.value, dtype=torch.uint8, device=cuda)
    t0 = time.perf_counter()
    rc = L.load().fem_selftest_bounded_wait(L.ptr(ws), nb.value, L.stream_handle())
    waited = time.perf_counter() - t0
    assert rc == L.FEM_ERR_DEVICE and "bounded device wait" in L.last_error()
    assert 0.2 < waited < 30.0
    prob, oprob, theta_np = cases.simp_box(4, 2, 2)
    lin = {"petsc_solver": {"ksp_type": "cg", "pc_type": "bjacobi", "rtol": 1e-12}, "precision": "mixed"}
    sol, _, _ = _simp_grad(prob, theta_np, cuda, dict(lin, rel_tol=1e-12, tol=0.0), lin)
    oprob.internal_vars = cases.oracle_set_params(oprob, torch.tensor(theta_np))
    osol = osolve.newton_solve(oprob, {"spsolve_solver": {}})
    assert np.abs(sol.cpu().numpy() - osol).max() <= 1e-9 * np.abs(osol).max()


def test_spmv_timing_inside_mixed_solve(cuda):
    """fem_spmv_timing_start/stop around a mixed solve: one timed SpMV per 16-iteration chunk,
    each between 0 and 10 ms on this small case; nothing is timed once stopped."""
    import ctypes
    import cases
    import jax_fem_gb300 as jf
    lib = jf._lib.load()
    prob, _, theta_np = cases.simp_box(12, 6, 3)
    prob.set_params(torch.tensor(theta_np, device=cuda))
    lin = {"petsc_solver": {"ksp_type": "cg", "pc_type": "bjacobi", "rtol": 1e-10}, "precision": "mixed"}
    sec, cnt = ctypes.c_double(), ctypes.c_int64()
    assert lib.fem_spmv_timing_start() == jf._lib.FEM_OK
    jf.solver(prob, lin)
    assert lib.fem_spmv_timing_stop(ctypes.byref(sec), ctypes.byref(cnt)) == jf._lib.FEM_OK
    its = sum(r["iterations"] for r in prob._engine.solve_log if r.get("iterations"))
    assert cnt.value >= 1 and cnt.value <= its // 16 + 64
    assert 0.0 < sec.value / cnt.value < 1e-2
    first = (sec.value, cnt.value)
    prob.set_params(torch.tensor(theta_np * 1.01, device=cuda))
    jf.solver(prob, lin)
    assert lib.fem_spmv_timing_stop(ctypes.byref(sec), ctypes.byref(cnt)) == jf._lib.FEM_OK
    assert (sec.value, cnt.value) == first


def test_maxiter_status(cuda):
    import cases
    import jax_fem_gb300 as jf
    prob, _, theta_np = cases.simp_box(8, 4, 2)
    prob.set_params(torch.tensor(theta_np, device=cuda))
    eng = prob._engine
    z = torch.zeros(eng.num_dofs, dtype=torch.float64, device=cuda)
    A = eng.tangent(z, jf._lib.FEM_F64, jf._lib.FEM_BC_SYMMETRIC)
    b = -eng.residual(z)
    x = torch.zeros_like(b)
    it, rn, st = eng.krylov("cg", A, b, x, jf._lib.FEM_PC_JACOBI, 1e-14, 0.0, 3)
    assert it == 3 and st == jf._lib.FEM_SOLVE_MAXITER


def test_df48_spmv_matches_fp64(cuda):
    """DF48 (FP32 hi + int16 correction, double-float SpMV) reproduces the FP64 SpMV to ~1e-11."""
    import jax_fem_gb300 as jf
    import cases
    prob, _, theta_np = cases.simp_box(10, 5, 3)
    prob.set_params(torch.tensor(theta_np, device=cuda))
    eng = prob._engine
    z = torch.zeros(eng.num_dofs, dtype=torch.float64, device=cuda)
    A64 = eng.tangent(z, jf._lib.FEM_F64, jf._lib.FEM_BC_SYMMETRIC, cache=False)
    x = torch.randn(eng.num_dofs, dtype=torch.float64, device=cuda)
    y64 = A64.matvec(x)
    L = jf._lib
    for fmt, tol in ((L.FEM_DF48, 1e-11), (L.FEM_SLICED_DF48, 1e-11), (L.FEM_SYM_DF48, 1e-11),
                     (L.FEM_SSYM_DF48, 1e-11), (L.FEM_SLICED_F64, 1e-14),
                     (L.FEM_SLICED_F32, 1e-6)):
        A = eng.tangent(z, fmt, jf._lib.FEM_BC_SYMMETRIC, cache=False)
        y = A.matvec(x).double()
        assert (y - y64).abs().max().item() <= tol * y64.abs().max().item(), fmt


def test_mixed32_variant_converges(cuda):
    """The all-FP32 variant (FP32 matrix and vectors, FP64 reliable updates) meets the same tolerance."""
    import cases
    prob, _, theta_np = cases.simp_box(12, 6, 3)
    o = {"petsc_solver": {"ksp_type": "cg", "pc_type": "bjacobi", "rtol": 1e-10}, "rel_tol": 1e-10, "tol": 0.0}
    s64, J64, g64 = _simp_grad(prob, theta_np, cuda, o, o)
    s32, J32, g32 = _simp_grad(prob, theta_np, cuda, dict(o, precision="mixed32"), dict(o, precision="mixed32"))
    assert (s32 - s64).abs().max().item() <= 1e-8 * s64.abs().max().item()
    assert np.abs(g32 - g64).max() <= 1e-7 * np.abs(g64).max()


def _df_nodes(x, vec):
    """Node-interleaved double-float copy of an FP64 vector (the fem_spmv_dfx input layout)."""
    pad = 4 if vec == 3 else 1
    hi = x.float()
    lo = (x - hi.double()).float()
    xp = torch.zeros(x.numel() // vec, pad, 2, dtype=torch.float32, device=x.device)
    xp[:, :vec, 0] = hi.view(-1, vec)
    xp[:, :vec, 1] = lo.view(-1, vec)
    return xp


@pytest.mark.parametrize("kind", ["sliced", "sym", "ssym"])
@pytest.mark.parametrize("n", [(10, 5, 3), (64, 40, 40), (1, 1, 1), (3, 40, 2), (2, 2, 60), (100, 50, 25)])
def test_spmv_dfx_matches_fp64(cuda, n, kind):
    """The mixed CG's SpMV (bulk-copy staged, double-float in and out) against the FP64 SpMV:
    y to 1e-11 of max|y|, the fused dot x.y to 1e-11 relative.  (64, 40, 40) has more slices
    than resident warps, so warps stream several slices through their shared-memory ring.  With
    sym the matrix is FEM_SYM_DF48 (upper node blocks; the transposed half through FP64 atomics,
    the dot through x.Ax = 2 x.(upper part) - x.diag); with ssym FEM_SSYM_DF48 (structured grid
    stencil, transposed half in registers and shuffles, plane i+1 and warp edges by atomics).
    The grids cover one group of lines with a partial warp (1,1,1), more lines per plane than a
    warp (3,40,2: 41 lines of a plane span two warps), one k step per work item (2,2,60: every row
    next to a chunk boundary) and items of several steps (64,40,40 and 100,50,25)."""
    import ctypes as C
    import jax_fem_gb300 as jf
    import cases
    L = jf._lib
    prob, _, theta_np = cases.simp_box(*n)
    prob.set_params(torch.tensor(theta_np, device=cuda))
    eng = prob._engine
    z = torch.zeros(eng.num_dofs, dtype=torch.float64, device=cuda)
    A64 = eng.tangent(z, L.FEM_F64, L.FEM_BC_SYMMETRIC, cache=False)
    fmt = {"sliced": L.FEM_SLICED_DF48, "sym": L.FEM_SYM_DF48, "ssym": L.FEM_SSYM_DF48}[kind]
    Adf = eng.tangent(z, fmt, L.FEM_BC_SYMMETRIC, cache=False)
    assert Adf.precision == fmt
    g = torch.Generator(device=cuda).manual_seed(3)
    x = torch.randn(eng.num_dofs, dtype=torch.float64, device=cuda, generator=g)
    y64 = A64.matvec(x)
    xp = _df_nodes(x, 3)
    yh = torch.empty(eng.num_dofs, dtype=torch.float32, device=cuda)
    yl = torch.empty_like(yh)
    dot = torch.zeros(1, dtype=torch.float64, device=cuda)
    nb = C.c_size_t()
    L.call("fem_krylov_workspace", eng.num_dofs, L.FEM_SLICED_DF48, C.byref(nb))
    ws = torch.empty(nb.value, dtype=torch.uint8, device=cuda)
    for _ in range(2):  # a second call reuses the workspace and its control block
        L.call("fem_spmv_dfx", C.byref(eng.pattern), eng.num_nodes, 3, fmt, L.ptr(Adf.data), L.ptr(xp),
               L.ptr(yh), L.ptr(yl), L.ptr(dot), L.ptr(ws), nb.value, L.stream_handle())
        y = yh.double() + yl.double()
        assert (y - y64).abs().max().item() <= 1e-11 * y64.abs().max().item()
        ref = torch.dot(x, y64).item()
        assert abs(dot.item() - ref) <= 1e-11 * abs(ref)


@pytest.mark.parametrize("n", [(1, 1, 1), (3, 40, 2), (2, 2, 60), (10, 5, 3), (64, 40, 40)])
def test_grid_slices_match_general_layout(cuda, n):
    """On a box mesh the sliced solver copies use the grid layout (fem_pattern_slices_grid: 27
    stencil slots per slice, the columns implied by the grid; (1,1,1) is a 2x2x2 node grid, where
    two slots of a row share a column offset and only the in-grid one may hold the block).  The
    same FP64 matrix converted into the general layout (fem_pattern_slices) gives the same FP64
    sliced SpMV (equal: the grid layout only adds zero blocks to the same accumulation order) and
    the mixed CG's SpMV within 1e-13 of |A| |x| per row and the dot within 1e-13 of |x|.|A| |x|
    (double-float rounding, ~2^-46 of each row's sum of |a x|, differs because the layouts pair
    different slots on the paired FP32 instructions)."""
    import ctypes as C
    import jax_fem_gb300 as jf
    import cases
    L = jf._lib
    prob, _, theta_np = cases.simp_box(*n)
    prob.set_params(torch.tensor(theta_np, device=cuda))
    eng = prob._engine
    assert eng.slices_grid and eng.pattern.slices_grid == 1 and eng.n_slots == 27 * eng.n_slices
    z = torch.zeros(eng.num_dofs, dtype=torch.float64, device=cuda)
    A64 = eng.tangent(z, L.FEM_F64, L.FEM_BC_SYMMETRIC, cache=False)
    st = L.stream_handle()
    gen = L.FemPattern.from_buffer_copy(eng.pattern)
    sp = torch.empty(eng.n_slices + 1, dtype=torch.int64, device=cuda)
    n_slots = C.c_int64()
    L.call("fem_pattern_slices", eng.num_nodes, L.ptr(eng.block_ptr), L.ptr(eng.block_cols), L.ptr(sp), None,
           C.byref(n_slots), st)
    sc = torch.empty(n_slots.value * 32, dtype=torch.int32, device=cuda)
    L.call("fem_pattern_slices", eng.num_nodes, L.ptr(eng.block_ptr), L.ptr(eng.block_cols), L.ptr(sp), L.ptr(sc),
           None, st)
    gen.slice_ptr, gen.slice_cols, gen.n_slots, gen.slices_grid = sp.data_ptr(), sc.data_ptr(), n_slots.value, 0

    def convert(pat, fmt):
        nb = C.c_size_t()
        L.call("fem_matrix_bytes", C.byref(pat), 3, fmt, C.byref(nb))
        buf = torch.empty(nb.value, dtype=torch.uint8, device=cuda)
        L.call("fem_matrix_convert", C.byref(pat), eng.num_nodes, 3, L.ptr(A64.data), fmt, L.ptr(buf), st)
        return buf

    g = torch.Generator(device=cuda).manual_seed(5)
    x = torch.randn(eng.num_dofs, dtype=torch.float64, device=cuda, generator=g)

    def spmv64(pat):
        vals = convert(pat, L.FEM_SLICED_F64)
        y = torch.empty(eng.num_dofs, dtype=torch.float64, device=cuda)
        L.call("fem_spmv", C.byref(pat), eng.num_nodes, 3, L.FEM_SLICED_F64, L.ptr(vals), L.ptr(x), L.ptr(y), st)
        return y

    y_grid, y_gen = spmv64(eng.pattern), spmv64(gen)
    assert torch.equal(y_grid, y_gen)
    assert (y_grid - A64.matvec(x)).abs().max().item() <= 1e-13 * y_gen.abs().max().item()

    nb = C.c_size_t()
    L.call("fem_krylov_workspace", eng.num_dofs, L.FEM_SLICED_DF48, C.byref(nb))
    ws = torch.empty(nb.value, dtype=torch.uint8, device=cuda)
    xp = _df_nodes(x, 3)

    def spmv_df(pat):
        vals = convert(pat, L.FEM_SLICED_DF48)
        yh = torch.empty(eng.num_dofs, dtype=torch.float32, device=cuda)
        yl = torch.empty_like(yh)
        dot = torch.zeros(1, dtype=torch.float64, device=cuda)
        L.call("fem_spmv_dfx", C.byref(pat), eng.num_nodes, 3, L.FEM_SLICED_DF48, L.ptr(vals), L.ptr(xp), L.ptr(yh),
               L.ptr(yl), L.ptr(dot), L.ptr(ws), nb.value, st)
        return yh.double() + yl.double(), dot.item()

    (yg, dg), (yo, do) = spmv_df(eng.pattern), spmv_df(gen)
    DeviceCSR = importlib.import_module("jax_fem_gb300.device").DeviceCSR
    ax = DeviceCSR(eng, L.FEM_F64, A64.data.abs(), L.FEM_BC_SYMMETRIC).matvec(x.abs())
    assert torch.all((yg - yo).abs() <= 1e-13 * ax)
    assert abs(dg - do) <= 1e-13 * torch.dot(x.abs(), ax).item()


def test_grid_slices_refuse_non_stencil_rows(cuda):
    """fem_pattern_slices_grid refuses (FEM_ERR_ARG) a pattern with a block outside a row's 27-point
    stencil and a grid whose size is not the node count; Problem then keeps the general layout."""
    import jax_fem_gb300 as jf
    import cases
    L = jf._lib
    prob, _, _ = cases.simp_box(4, 3, 3)
    eng = prob._engine
    st = L.stream_handle()
    sp = torch.empty(eng.n_slices + 1, dtype=torch.int64, device=cuda)
    sc = torch.empty(27 * eng.n_slices * 32, dtype=torch.int32, device=cuda)
    cols = eng.block_cols.clone()
    cols[-1] = 0     # the last node's last block now couples node 0, far outside its stencil
    with pytest.raises(L.FemError) as e:
        L.call("fem_pattern_slices_grid", eng.num_nodes, L.ptr(eng.block_ptr), L.ptr(cols), *eng.grid, L.ptr(sp),
               L.ptr(sc), st)
    assert e.value.code == L.FEM_ERR_ARG
    nx, ny, nz = eng.grid
    with pytest.raises(L.FemError):
        L.call("fem_pattern_slices_grid", eng.num_nodes, L.ptr(eng.block_ptr), L.ptr(eng.block_cols), nx, ny, nz + 1,
               L.ptr(sp), L.ptr(sc), st)
    L.call("fem_pattern_slices_grid", eng.num_nodes, L.ptr(eng.block_ptr), L.ptr(eng.block_cols), nx, ny, nz,
           L.ptr(sp), L.ptr(sc), st)
    assert torch.equal(sp.cpu(), 27 * torch.arange(eng.n_slices + 1))


def test_custom_solver_hook_petsc_style(cuda):
    """custom_solver plug-in (solver.py:278-280) written against the PETSc Mat interface of the
    documented example (A.getValuesCSR(), A.getSize(); scipy direct solve on the host) gives the
    built-in solve's solution on the cube case (1e-9 of max|u|; both stop at Newton rel 1e-10)."""
    import scipy.sparse
    import scipy.sparse.linalg
    import jax_fem_gb300 as jf
    import cases

    def host_direct(A, b, x0, opts):
        indptr, indices, data = A.getValuesCSR()
        As = scipy.sparse.csr_array((data, indices, indptr), shape=A.getSize())
        return scipy.sparse.linalg.spsolve(As.tocsc(), b.cpu().numpy())

    prob, _ = cases.cube_elasticity(golden("linear_elasticity_cube"))[:2]
    ref = jf.solver(prob, {"petsc_solver": {"ksp_type": "cg", "pc_type": "bjacobi", "rtol": 1e-13},
                           "rel_tol": 1e-10, "tol": 0.0})[0]
    got = jf.solver(prob, {"custom_solver": host_direct, "rel_tol": 1e-10, "tol": 0.0})[0]
    assert (got - ref).abs().max().item() <= 1e-9 * ref.abs().max().item()


def test_cube_gold_through_vtu_round_trip(cuda, tmp_path):
    """The reference's regression flow (test_linear_elasticity_cube.py:45-83): solve, write the
    solution with save_sol (float32 point data), read the file back and compare with the
    FEniCSx gold at decimal 5."""
    import jax_fem_gb300 as jf
    import cases
    g = golden("linear_elasticity_cube")
    prob, _ = cases.cube_elasticity(g)
    sol = jf.solver(prob, {"petsc_solver": {"ksp_type": "cg", "pc_type": "bjacobi", "rtol": 1e-12}})[0]
    path = tmp_path / "u.vtu"
    jf.save_sol(prob.fes[0], sol, str(path))
    _, _, pd, _ = jf.read_vtu(str(path))
    np.testing.assert_array_almost_equal(g["sol"], pd["sol"], decimal=5)
