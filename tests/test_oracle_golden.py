"""The oracle pinned against the reference's own FEniCSx gold fixtures at the reference's
tolerances (tests/benchmarks/*/test_*.py): decimal 5 (cube, Poisson, Neo-Hookean),
decimal 3 (cylinder solution, J2 averaged stress), decimal 4 (cylinder area)."""
import numpy as np
import pytest
import torch

from conftest import golden
from oracle import fem, materials as M, solve

top = lambda p: np.isclose(p[2], 10.0, atol=1e-5)
bottom = lambda p: np.isclose(p[2], 0.0, atol=1e-5)
x0 = lambda p: np.isclose(p[0], 0.0, atol=1e-5)
x1 = lambda p: np.isclose(p[0], 1.0, atol=1e-5)
zero = lambda p: 0.0


def test_cube_linear_elasticity():
    g = golden("linear_elasticity_cube")
    p = fem.OracleProblem(g["points"], g["cells"], 3, dirichlet_bc_info=[[x0] * 3, [0, 1, 2], [lambda q: 1.0] * 3],
                          location_fns=[x1], tensor_map=M.linear_elastic(70e3, 0.3),
                          mass_map=lambda u, x: -torch.tensor([0., 10., 10.]),
                          surface_maps=[lambda u, x: -torch.tensor([10., 0., 0.])])
    sol = solve.newton_solve(p, {})       # default jax_solver semantics (BiCGStab + Jacobi)
    np.testing.assert_array_almost_equal(g["sol"], sol, decimal=5)


def test_poisson():
    g = golden("linear_poisson")
    p = fem.OracleProblem(g["points"], g["cells"], 1, dirichlet_bc_info=[[x0, x1], [0, 0], [zero, lambda q: 1.0]],
                          tensor_map=M.laplace())
    np.testing.assert_array_almost_equal(g["sol"], solve.newton_solve(p, {}), decimal=5)


def test_cylinder_and_area():
    g = golden("linear_elasticity_cylinder")
    p = fem.OracleProblem(g["points"], g["cells"], 3, dirichlet_bc_info=[[bottom] * 3, [0, 1, 2], [zero] * 3],
                          location_fns=[top], tensor_map=M.linear_elastic(70e3, 0.3),
                          mass_map=lambda u, x: -torch.stack([1e3 * x[0], 2e3 * x[1], 3e3 * x[2]]),
                          surface_maps=[lambda u, x: -torch.stack([1e3 * x[0] ** 2 + 1e3 * x[1] ** 2, 0 * x[0], 0 * x[0]])])
    sol = solve.newton_solve(p, {"spsolve_solver": {}})
    np.testing.assert_array_almost_equal(g["sol"], sol, decimal=3)
    _, nanson = p.fe.get_face_shape_grads(p.boundary_inds_list[0])
    np.testing.assert_almost_equal(g["surface_area"][0], nanson.sum(), decimal=4)


def test_hyperelasticity_and_traction():
    g = golden("hyperelasticity")
    bc = [[bottom] * 3 + [top] * 3, [0, 1, 2, 0, 1, 2], [zero] * 5 + [lambda q: 1.0]]
    p = fem.OracleProblem(g["points"], g["cells"], 3, dirichlet_bc_info=bc, tensor_map=M.neo_hookean(1e3, 0.3))
    sol = solve.newton_solve(p, {"spsolve_solver": {}})
    np.testing.assert_array_almost_equal(g["sol"], sol, decimal=5)
    b = p.fe.get_boundary_conditions_inds([top])[0]
    fg, nanson = p.fe.get_face_shape_grads(b)
    ug = np.einsum("fnv,fqnd->fqvd", sol[p.fe.cells][b[:, 0]], fg)
    P = torch.func.vmap(M.neo_hookean(1e3, 0.3))(torch.from_numpy(ug.reshape(-1, 3, 3))).numpy().reshape(ug.shape)
    trac = ((P @ np.array([0, 0, 1.0])) * nanson[:, :, None]).sum((0, 1))[2]
    np.testing.assert_almost_equal(g["traction"][0], trac, decimal=5)


def test_plasticity_steps():
    g = golden("plasticity")
    strain, rmap = M.j2_maps(70e3, 0.3, 250.0)
    disps = g["disps"]
    bc = [[bottom] * 3 + [top] * 3, [0, 1, 2, 0, 1, 2], [zero] * 5 + [lambda q, d=disps[0]: d]]
    p = fem.OracleProblem(g["points"], g["cells"], 3, dirichlet_bc_info=bc, tensor_map=rmap)
    C, nq = p.num_cells, p.fe.num_quads
    sig = torch.zeros(C, nq, 3, 3)
    eps = torch.zeros(C, nq, 3, 3)
    p.internal_vars = [sig, eps]
    avg = []
    for d in disps:
        bc[2][-1] = (lambda q, d=d: d)
        p.fe.update_Dirichlet_boundary_conditions(bc)
        sol = solve.newton_solve(p, {"spsolve_solver": {}})
        ug = torch.from_numpy(p.fe.sol_to_grad(sol))
        sig = torch.func.vmap(torch.func.vmap(rmap))(ug, sig, eps)
        eps = torch.func.vmap(torch.func.vmap(strain))(ug)
        p.internal_vars = [sig, eps]
        jxw = torch.from_numpy(p.fe.JxW)
        avg.append(((sig * jxw[:, :, None, None]).sum((0, 1)) / jxw.sum())[2, 2].item())
    np.testing.assert_array_almost_equal(g["sol"], sol, decimal=5)
    np.testing.assert_array_almost_equal(g["avg_stresses"], np.array(avg), decimal=3)


def test_pattern_size_formula():
    """HEX8 vec=3 nnz = 9 (3Nx+1)(3Ny+1)(3Nz+1) on a structured box (counts quoted for the workloads)."""
    for n in [(2, 3, 4), (10, 10, 10)]:
        pts, cells = fem.box_mesh(*n, 1.0, 1.0, 1.0)
        p = fem.OracleProblem(pts, cells, 3, tensor_map=M.linear_elastic(1.0, 0.3))
        ip, ix = fem.coo_pattern(p.I, p.J, p.num_total_dofs_all_vars)
        assert len(ix) == 9 * (3 * n[0] + 1) * (3 * n[1] + 1) * (3 * n[2] + 1)


def test_bicgstab_restatement_solves():
    """The restated jax bicgstab loop converges to the direct solution on an SPD system."""
    import scipy.sparse as sp
    n = 50
    A = sp.diags([-1.0, 2.05, -1.0], [-1, 0, 1], shape=(n, n)).tocsr()
    b = np.random.default_rng(0).standard_normal(n)
    x, k = solve.bicgstab_jax(A, b, None, None, 1e-12, 1e-12, 1000)
    assert k > 0
    np.testing.assert_allclose(A @ x, b, atol=1e-9)


def test_oracle_adjoint_matches_fd():
    """The oracle's implicit_vjp (SIMP compliance) agrees with central differences."""
    pts, cells = fem.box_mesh(4, 2, 2, 2.0, 1.0, 0.5)
    left = lambda p: np.isclose(p[0], 0.0, atol=1e-5)
    right = lambda p: np.isclose(p[0], 2.0, atol=1e-5)
    p = fem.OracleProblem(pts, cells, 3, dirichlet_bc_info=[[left] * 3, [0, 1, 2], [zero] * 3], location_fns=[right],
                          tensor_map=M.simp_elastic(1.0, 1e-3, 0.3, 3.0),
                          surface_maps=[lambda u, x: torch.tensor([0.0, 0.0, 1.0])])
    setp = lambda pr, th: [th[:, None, :].expand(-1, 8, -1)]
    th = 0.5 + np.random.default_rng(0).uniform(-0.05, 0.05, size=(len(cells), 1))
    p.internal_vars = setp(p, torch.tensor(th))
    f = p.compute_residual(torch.zeros(p.num_total_dofs_all_vars)).numpy()
    sol = solve.newton_solve(p, {"spsolve_solver": {}})
    v = f.copy()
    v[p.bc_rows()[0]] = 0
    g, _ = solve.implicit_vjp(p, sol, th, setp, v)
    h = 1e-6
    for c in [0, 5, 11]:
        vals = []
        for s in (1, -1):
            t2 = th.copy()
            t2[c, 0] += s * h
            p.internal_vars = setp(p, torch.tensor(t2))
            vals.append(f @ solve.newton_solve(p, {"spsolve_solver": {}}).reshape(-1))
        assert abs((vals[0] - vals[1]) / (2 * h) - g[c, 0]) <= 1e-6 * np.abs(g).max()


@pytest.mark.parametrize("ele", ["HEX8", "TET10", "TET4"])
def test_isotropic_node_pair_tangent_identity(ele):
    """The identity the assembly kernel's isotropic tangent rests on: for lam / mu the same at
    every quadrature point (linear-elastic and SIMP materials; only E varies), the element block
    sum_q JxW (lam g_a g_b^T + mu g_b g_a^T + mu (g_a . g_b) I) equals (lam/mu) M_ab + M_ab^T +
    tr(M_ab) I with M_ab = sum_q JxW mu g_a g_b^T, and K_ba = K_ab^T.  Checked on a distorted
    element with a different E at each point against B^T D B in Voigt form (1e-13)."""
    from oracle import basis
    rng = np.random.default_rng(7)
    t = basis.element_tables(ele)
    grads_ref, w = t["shape_grads_ref"], t["quad_weights"]
    nq, nn, _ = grads_ref.shape
    nu = 0.3
    E = 1.0 + rng.random(nq)                                     # a different modulus per point
    lam, mu = E * nu / ((1 + nu) * (1 - 2 * nu)), E / (2 * (1 + nu))
    X = np.eye(3) + 0.2 * rng.standard_normal((3, 3))            # affine map of the reference cell
    Kd = np.zeros((nn * 3, nn * 3))
    Kp = np.zeros_like(Kd)
    for q in range(nq):
        G = grads_ref[q] @ np.linalg.inv(X)                      # physical gradients (nn, 3)
        jxw = abs(np.linalg.det(X)) * w[q]
        B = np.zeros((6, nn * 3))                                # Voigt strain-displacement matrix
        for a in range(nn):
            gx, gy, gz = G[a]
            B[:, 3 * a:3 * a + 3] = [[gx, 0, 0], [0, gy, 0], [0, 0, gz],
                                     [gy, gx, 0], [0, gz, gy], [gz, 0, gx]]
        D = np.zeros((6, 6))
        D[:3, :3] = lam[q]
        D[:3, :3] += 2 * mu[q] * np.eye(3)
        D[3:, 3:] = mu[q] * np.eye(3)
        Kd += jxw * B.T @ D @ B
        for a in range(nn):
            for b in range(nn):
                Kp[3 * a:3 * a + 3, 3 * b:3 * b + 3] += jxw * mu[q] * np.outer(G[a], G[b])
    cr = 2 * nu / (1 - 2 * nu)
    Kn = np.zeros_like(Kd)
    for a in range(nn):
        for b in range(a, nn):
            M_ab = Kp[3 * a:3 * a + 3, 3 * b:3 * b + 3]
            K_ab = cr * M_ab + M_ab.T + np.trace(M_ab) * np.eye(3)
            Kn[3 * a:3 * a + 3, 3 * b:3 * b + 3] = K_ab
            Kn[3 * b:3 * b + 3, 3 * a:3 * a + 3] = K_ab.T
    assert np.abs(Kn - Kd).max() <= 1e-13 * np.abs(Kd).max()
