"""GPU parity tests for the remaining workload shapes of this path: Neo-Hookean load stepping
(HEX8, x=1 face u_x ramp), Kuhn-split TET10 linear elasticity and J2 with a modulus field over
load steps.  Each runs a small case against the CPU oracle and the full-size case through
size-independent properties (Newton convergence, mixed against FP64 agreement, finite
differences of the gradient).  Inputs are seeded synthetic fields."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _stretch_bc(Lx):
    left = lambda p: np.isclose(p[0], 0.0, atol=1e-5)
    right = lambda p: np.isclose(p[0], Lx, atol=1e-5)
    zero = lambda p: 0.0
    return [[left] * 3 + [right] * 3, [0, 1, 2, 0, 1, 2], [zero] * 3 + [lambda p: 0.0, zero, zero]]


def _set_stretch(prob, bc, d):
    bc[2][3] = (lambda p, d=d: d)
    prob.fes[0].update_Dirichlet_boundary_conditions(bc)


def _neo_hookean(n, E=10.0, nu=0.3):
    import jax_fem_gb300 as jf
    m = jf.box_mesh(n, n, n, 1.0, 1.0, 1.0)
    pts, cells = m.points, m.cells_dict["hexahedron"]
    bc = _stretch_bc(1.0)

    class P(jf.Problem):
        def get_tensor_map(self):
            return jf.NeoHookean(E, nu)

    return P(jf.Mesh(pts, cells), vec=3, dim=3, dirichlet_bc_info=bc), bc, pts, cells


def _newton_opts(precision, rel_tol, guess=None):
    o = {"petsc_solver": {"ksp_type": "cg", "pc_type": "bjacobi", "rtol": 1e-12}, "rel_tol": rel_tol, "tol": 0.0,
         "precision": precision}
    if guess is not None:
        o["initial_guess"] = guess
    return o


def test_neo_hookean_load_steps_vs_oracle(cuda):
    """Neo-Hookean (E=10, nu=0.3) on HEX8 4^3, x=0 clamped, x=1 u_x = 0.01 k for k = 1..3, each
    step from the previous solution, Newton to rel 1e-10: every step within 1e-9 of max|u| of the
    oracle's Newton solve (scipy direct solves)."""
    import jax_fem_gb300 as jf
    from oracle import fem as ofem, materials as omat, solve as osolve
    prob, bc, pts, cells = _neo_hookean(4)
    obc = _stretch_bc(1.0)
    oprob = ofem.OracleProblem(pts, cells, 3, dirichlet_bc_info=obc, tensor_map=omat.neo_hookean(10.0, 0.3))
    sol = None
    osol = None
    for k in range(1, 4):
        d = 0.01 * k
        _set_stretch(prob, bc, d)
        obc[2][3] = (lambda p, d=d: d)
        oprob.fe.update_Dirichlet_boundary_conditions(obc)
        sol = jf.solver(prob, _newton_opts("fp64", 1e-10, None if sol is None else sol))[0]
        oo = {"spsolve_solver": {}, "rel_tol": 1e-10, "tol": 0.0}
        if osol is not None:
            oo["initial_guess"] = osol
        osol = osolve.newton_solve(oprob, oo)
        ref = np.asarray(osol).reshape(-1)
        got = sol.reshape(-1).cpu().numpy()
        assert np.abs(got - ref).max() <= 1e-9 * np.abs(ref).max(), k


def test_neo_hookean_50cube_ten_steps_mixed_vs_fp64(cuda):
    """The full Neo-Hookean load-stepping case: HEX8 50^3 (397,953 dofs), ten steps u_x = 0.01 k,
    Newton to rel 1e-10 in both precisions.  Every step converges; the mixed solution stays within
    1e-8 of the FP64 one (relative to max|u|) at every step."""
    import jax_fem_gb300 as jf
    prob, bc, _, _ = _neo_hookean(50)
    s64 = smx = None
    for k in range(1, 11):
        _set_stretch(prob, bc, 0.01 * k)
        s64 = jf.solver(prob, _newton_opts("fp64", 1e-10, s64))[0]
        info64 = dict(prob.newton_info)
        smx = jf.solver(prob, _newton_opts("mixed", 1e-10, smx))[0]
        infomx = dict(prob.newton_info)
        assert info64["rel"] <= 1e-10 and infomx["rel"] <= 1e-10, (k, info64, infomx)
        err = (smx - s64).abs().max().item() / s64.abs().max().item()
        assert err <= 1e-8, (k, err)


def _tet10_elastic(n):
    import jax_fem_gb300 as jf
    m = jf.box_mesh_tet10(n, n, n, 1.0, 1.0, 1.0)
    pts, cells = m.points, m.cells_dict["tetra10"]
    bc = _stretch_bc(1.0)

    class P(jf.Problem):
        def get_tensor_map(self):
            return jf.LinearElastic(1.0, 0.3)

    prob = P(jf.Mesh(pts, cells), vec=3, dim=3, ele_type="TET10", dirichlet_bc_info=bc)
    _set_stretch(prob, bc, 0.01)
    return prob, bc, pts, cells


def test_tet10_kuhn_solution_vs_oracle(cuda):
    """Kuhn-split TET10 (4-point rule), E=1, nu=0.3, x=0 clamped, x=1 u_x = 0.01, on 4^3 cubes
    (384 tets): the FP64 and the mixed solves refined to rel 1e-10 both within 1e-9 of max|u| of
    the oracle's direct solve."""
    import jax_fem_gb300 as jf
    from oracle import fem as ofem, materials as omat, solve as osolve
    prob, bc, pts, cells = _tet10_elastic(4)
    obc = _stretch_bc(1.0)
    obc[2][3] = (lambda p: 0.01)
    oprob = ofem.OracleProblem(pts, cells, 3, ele_type="TET10", dirichlet_bc_info=obc,
                               tensor_map=omat.linear_elastic(1.0, 0.3))
    ref = np.asarray(osolve.newton_solve(oprob, {"spsolve_solver": {}, "rel_tol": 1e-12, "tol": 0.0})).reshape(-1)
    for precision in ("fp64", "mixed"):
        sol = jf.solver(prob, _newton_opts(precision, 1e-10))[0].reshape(-1).cpu().numpy()
        assert np.abs(sol - ref).max() <= 1e-9 * np.abs(ref).max(), precision


def test_tet10_kuhn_64cube_mixed_vs_fp64(cuda):
    """The full TET10 case: Kuhn split of 64^3 cubes (1,572,864 tets, 6,440,067 dofs,
    nnz 547,739,145), refined to rel 1e-10 in both precisions; the CSR pattern has the exact
    count and the mixed solution is within 1e-8 of the FP64 one."""
    import jax_fem_gb300 as jf
    prob, bc, _, _ = _tet10_elastic(64)
    eng = prob._engine
    assert eng.num_dofs == 6440067 and eng.nnz == 547739145
    s64 = jf.solver(prob, _newton_opts("fp64", 1e-10))[0]
    assert prob.newton_info["rel"] <= 1e-10
    smx = jf.solver(prob, _newton_opts("mixed", 1e-10))[0]
    assert prob.newton_info["rel"] <= 1e-10
    err = (smx - s64).abs().max().item() / s64.abs().max().item()
    assert err <= 1e-8, err


def _j2_mu_problem(n):
    import jax_fem_gb300 as jf
    m = jf.box_mesh(n, n, n, 1.0, 1.0, 1.0)
    pts, cells = m.points, m.cells_dict["hexahedron"]
    bc = _stretch_bc(1.0)

    class P(jf.Problem):
        def get_tensor_map(self):
            return jf.J2Plasticity(70e3, 0.3, 250.0, modulus_field=True)

        def set_params(self, params):
            mu, sig, eps = params
            self.internal_vars = [sig, eps, mu[:, None].expand(-1, 8)]

    return P(jf.Mesh(pts, cells), vec=3, dim=3, dirichlet_bc_info=bc), bc


def _j2_objective(prob, bc, mu, disps, u_target, opts):
    import jax_fem_gb300 as jf
    eng = prob._engine
    nc, nq = eng.num_cells, eng.num_quads
    sig = torch.zeros(nc, nq, 3, 3, dtype=torch.float64, device=mu.device)
    eps = torch.zeros_like(sig)
    fwd = jf.ad_wrapper(prob, opts, opts)
    sol = None
    for d in disps:
        _set_stretch(prob, bc, d)
        sol = fwd([mu, sig, eps])[0]
        sig, eps = jf.update_j2_history(prob, sol, sig, eps, mu[:, None].expand(-1, nq))
    return ((sol - u_target) ** 2).sum()


@pytest.mark.parametrize("n", [8, 100])
def test_j2_modulus_field_five_steps_gradient(cuda, n):
    """J2 (E=70e3, nu=0.3, sig0=250) with a per-cell modulus field mu0 * exp(0.2 z - 0.02),
    z ~ N(0,1) seed 0, five load steps of the x=1 face u_x ramp, objective ||u_5 - u_target||^2.
    The gradient (implicit adjoint of every step + reverse mode of every history update) matches
    central finite differences along a smooth direction to 1e-4 relative (h = 1e-5), and along a
    random per-cell direction the difference quotient moves towards it as h shrinks (h = 1e-3,
    2.5e-4, 6.25e-5), on 8^3 and on the full 100^3 (3,090,903 dofs) case."""
    prob, bc = _j2_mu_problem(n)
    eng = prob._engine
    g = torch.Generator().manual_seed(0)
    z = torch.randn(eng.num_cells, generator=g, dtype=torch.float64)
    mu0 = torch.exp(0.2 * z - 0.02).to(cuda)
    disps = [1.5e-3 * k for k in range(1, 6)]
    u_target = (torch.rand(eng.num_nodes, 3, generator=g, dtype=torch.float64) * 5e-3).to(cuda)
    opts = {"petsc_solver": {"ksp_type": "cg", "pc_type": "bjacobi", "rtol": 1e-13}, "rel_tol": 1e-11, "tol": 0.0}
    mu = mu0.clone().requires_grad_(True)
    J = _j2_objective(prob, bc, mu, disps, u_target, opts)
    J.backward()
    grad = mu.grad.detach()
    assert torch.isfinite(grad).all() and grad.abs().max().item() > 0
    # a smooth direction (plus a little noise): a purely random per-cell field averages out over
    # 10^6 cells and would bury the directional derivative under the solves' rounding
    fe = prob.fes[0]
    xc = torch.as_tensor(np.asarray(fe.points)[np.asarray(fe.cells)].mean(1), dtype=torch.float64)
    v = (torch.cos(2 * np.pi * xc[:, 0]) + 0.5 * xc[:, 1] +
         0.1 * torch.randn(eng.num_cells, generator=g, dtype=torch.float64)).to(cuda)
    h = 1e-5
    with torch.no_grad():
        Jp = _j2_objective(prob, bc, mu0 + h * v, disps, u_target, opts).item()
        Jm = _j2_objective(prob, bc, mu0 - h * v, disps, u_target, opts).item()
    fd = (Jp - Jm) / (2 * h)
    an = torch.dot(grad, v).item()
    assert abs(fd - an) <= 1e-4 * max(abs(fd), abs(an)), (fd, an)
    # A purely random per-cell direction moves many quadrature points across the yield surface,
    # where the return map has a kink: J along the ray is only piecewise smooth, and a central
    # difference over [-h, h] carries an error from the kinks inside it that shrinks with h (the
    # number of points crossing is proportional to h), not the O(h^2) of a smooth function.  A
    # bias in the adjoint gradient would instead leave a floor.  The solves' rounding is far below
    # these gaps (measured on 100^3: J agrees to 7e-15 between Newton tolerances 1e-11 and 1e-12,
    # i.e. 3e-8 of the quotient at the smallest h).  So the difference quotient must move towards
    # the adjoint value at every 4x step of h over a 16x range and close at least a quarter of
    # the gap (8^3: 1.1e-2 -> 1.5e-5; 100^3: 1.8e-2 -> 9.8e-3).
    w = torch.randn(eng.num_cells, generator=g, dtype=torch.float64).to(cuda)
    an_w = torch.dot(grad, w).item()
    hs = (1e-3, 2.5e-4, 6.25e-5)
    gaps = []
    for hw in hs:
        with torch.no_grad():
            Jp = _j2_objective(prob, bc, mu0 + hw * w, disps, u_target, opts).item()
            Jm = _j2_objective(prob, bc, mu0 - hw * w, disps, u_target, opts).item()
        gaps.append(abs((Jp - Jm) / (2 * hw) - an_w) / abs(an_w))
    print(f"J2 n={n}: random direction, relative FD gap " + ", ".join(f"h={hw:g}: {gp:.3e}" for hw, gp in zip(hs, gaps)))
    assert gaps[1] < gaps[0] and gaps[2] < gaps[1], gaps
    assert gaps[2] <= 0.75 * gaps[0], gaps
    assert gaps[0] <= 5e-2, gaps


def test_tet4_pattern_values_solution_vs_oracle(cuda):
    """TET4 (one-point rule, basis.py:55-60) on the Kuhn split of 4^3 cubes: CSR pattern
    bit-exact, FP64 tangent 1e-12 and the stretch solution 1e-9 against the oracle."""
    import jax_fem_gb300 as jf
    from oracle import fem as ofem, materials as omat, solve as osolve
    m = jf.box_mesh_tet10(4, 4, 4, 1.0, 1.0, 1.0)
    nv = 5 ** 3
    pts, cells = np.asarray(m.points)[:nv], np.asarray(m.cells_dict["tetra10"])[:, :4]
    bc = _stretch_bc(1.0)
    bc[2][3] = (lambda p: 0.01)

    class P(jf.Problem):
        def get_tensor_map(self):
            return jf.LinearElastic(1.0, 0.3)

    prob = P(jf.Mesh(pts, cells), vec=3, dim=3, ele_type="TET4", dirichlet_bc_info=bc)
    oprob = ofem.OracleProblem(pts, cells, 3, ele_type="TET4", dirichlet_bc_info=bc,
                               tensor_map=omat.linear_elastic(1.0, 0.3))
    eng = prob._engine
    ip, ix = ofem.coo_pattern(oprob.I, oprob.J, oprob.num_total_dofs_all_vars)
    np.testing.assert_array_equal(eng.indptr.cpu().numpy(), ip)
    np.testing.assert_array_equal(eng.scalar_indices().cpu().numpy(), ix)
    u = np.random.default_rng(4).standard_normal(oprob.num_total_dofs_all_vars) * 1e-2
    prob.newton_update([torch.tensor(u, device=cuda).reshape(-1, 3)])
    A = jf.get_A(prob)
    oprob.newton_update(torch.tensor(u))
    Ao = ofem.assemble_petsc(oprob)
    assert np.abs(A.data.cpu().numpy() - Ao.data).max() <= 1e-12 * np.abs(Ao.data).max()
    ref = np.asarray(osolve.newton_solve(oprob, {"spsolve_solver": {}, "rel_tol": 1e-12, "tol": 0.0})).reshape(-1)
    sol = jf.solver(prob, _newton_opts("fp64", 1e-10))[0].reshape(-1).cpu().numpy()
    assert np.abs(sol - ref).max() <= 1e-9 * np.abs(ref).max()
