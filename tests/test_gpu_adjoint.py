"""Adjoint paths beyond the symmetric, parameter-in-the-material case:

* a non-symmetric tangent (an anisotropic conduction law whose matrix is not symmetric): the
  adjoint must solve with A^T (the reference transposes the PETSc matrix before the adjoint
  solve, jax_fem/solver.py:1405-1409);
* parameters that set Dirichlet values through set_params (the reference's compute_gradients
  example, docs/source/learn/compute_gradients/example.ipynb cells 11 and 16): their gradient
  is lam_b = v_b - K_fb^T lam_f on the Dirichlet rows of A^T lam = v.

Both are checked against the oracle (scipy direct solve of A^T lam = v with the restated
PETSc-semantics matrix) and against central finite differences.
"""
import numpy as np
import pytest
import scipy.sparse.linalg as spla
import torch

pytestmark = pytest.mark.gpu

A_ANISO = np.array([[1.0, 0.4, 0.0], [-0.3, 1.2, 0.1], [0.0, 0.2, 0.8]])


def _aniso(cuda, n=(5, 4, 3)):
    """vec-1 conduction with flux A grad u (A not symmetric), source 1, u = s (1 + y) on x = 0
    and u = 0 on x = 1; the parameter s sets the x = 0 Dirichlet values."""
    import jax_fem_gb300 as jf
    from oracle import fem as ofem
    m = jf.box_mesh(*n, 1.0, 1.0, 1.0)
    pts, cells = m.points, m.cells_dict["hexahedron"]
    x0 = lambda p: np.isclose(p[0], 0.0, atol=1e-5)
    x1 = lambda p: np.isclose(p[0], 1.0, atol=1e-5)
    bc = [[x0, x1], [0, 0], [lambda p: 1.0 + p[1], lambda p: 0.0]]

    class P(jf.Problem):
        def get_tensor_map(self):
            return lambda u_grad: u_grad @ A_ANISO.T

        def get_mass_map(self):
            return lambda u, x: np.array([-1.0])

        def set_params(self, s):
            fe = self.fes[0]
            fe.dirichlet_bc_info[2][0] = lambda p: s * (1.0 + p[1])
            fe.update_Dirichlet_boundary_conditions(fe.dirichlet_bc_info)

    prob = P(jf.Mesh(pts, cells), vec=1, dim=3, dirichlet_bc_info=[list(b) for b in bc])
    At = torch.tensor(A_ANISO)

    def oracle(s):
        obc = [bc[0], bc[1], [lambda p, s=s: s * (1.0 + p[1]), bc[2][1]]]
        return ofem.OracleProblem(pts, cells, 1, dirichlet_bc_info=obc, tensor_map=lambda g: g @ At.T,
                                  mass_map=lambda u, x: torch.tensor([-1.0], dtype=torch.float64))
    return prob, oracle


def test_nonsymmetric_tangent_and_dirichlet_param_gradient(cuda):
    import jax_fem_gb300 as jf
    from oracle import fem as ofem, solve as osolve
    prob, oracle = _aniso(cuda)
    assert not prob._engine.tangent_symmetric
    w = torch.tensor(np.random.default_rng(3).standard_normal(prob._engine.num_dofs), device=cuda)
    opts = {"jax_solver": {"tol": 1e-13, "atol": 1e-30}, "rel_tol": 1e-12, "tol": 0.0}
    adj = {"jax_solver": {"tol": 1e-13, "atol": 1e-30}}
    fwd = jf.ad_wrapper(prob, opts, adj)
    s0 = 0.7
    s = torch.tensor(s0, dtype=torch.float64, device=cuda, requires_grad=True)
    sol = fwd(s)[0]
    J = torch.dot(w, sol.reshape(-1))
    J.backward()
    g = s.grad.item()
    # oracle: u*, A = zeroRows(K) at u*, lam = A^-T w; dJ/ds = lam_b . dg/ds with g_b = s (1 + y_b)
    op = oracle(s0)
    osol = osolve.newton_solve(op, {"spsolve_solver": {}, "rel_tol": 1e-13, "tol": 0.0}).reshape(-1)
    assert np.abs(sol.detach().cpu().numpy().reshape(-1) - osol).max() <= 1e-10 * np.abs(osol).max()
    op.newton_update(torch.from_numpy(osol))
    A = ofem.assemble_petsc(op)
    asym = abs(A - A.T).max()
    assert asym > 1e-3 * abs(A).max()                       # the tangent really is non-symmetric
    lam = spla.spsolve(A.T.tocsc(), w.cpu().numpy())
    rows, _ = op.bc_rows()
    pts = op.fe.points
    nodes = rows                                           # vec 1: row = node
    dg = np.where(np.isclose(pts[nodes, 0], 0.0, atol=1e-5), 1.0 + pts[nodes, 1], 0.0)
    g_or = float(lam[rows] @ dg)
    assert abs(g - g_or) <= 1e-9 * abs(g_or)
    # central finite differences (the problem is linear in s: FD is exact up to rounding)
    vals = []
    for sg in (+1, -1):
        with torch.no_grad():
            u = fwd(torch.tensor(s0 + sg * 1e-4, dtype=torch.float64, device=cuda))[0]
        vals.append(torch.dot(w, u.reshape(-1)).item())
    fd = (vals[0] - vals[1]) / 2e-4
    assert abs(fd - g) <= 1e-8 * abs(g)


def test_transpose_matches_oracle(cuda):
    """fem_matrix_transpose on the non-symmetric tangent equals the transposed oracle matrix."""
    import jax_fem_gb300 as jf
    from oracle import fem as ofem
    prob, oracle = _aniso(cuda, (3, 2, 2))
    eng = prob._engine
    z = torch.zeros(eng.num_dofs, dtype=torch.float64, device=cuda)
    K = eng.tangent(z, jf._lib.FEM_F64, jf._lib.FEM_BC_NONE, cache=False)
    Kt = K.transpose().to_scipy().toarray()
    op = oracle(1.0)
    op.newton_update(torch.zeros(op.num_total_dofs_all_vars, dtype=torch.float64))
    n = op.num_total_dofs_all_vars
    import scipy.sparse as sp
    Ko = sp.coo_matrix((op.V, (op.I, op.J)), shape=(n, n)).toarray()
    assert np.abs(Kt - Ko.T).max() <= 1e-12 * np.abs(Ko).max()


def test_neo_hookean_density_and_dirichlet_scale_gradient(cuda):
    """The compute_gradients example's parameters on a small mesh: per-cell density rho (scales E
    of a Neo-Hookean solid) and the scale of the bottom face's prescribed u_z, objective sum u^2.
    d/drho against the oracle's implicit_vjp, d/dscale against lam_b and central differences."""
    import jax_fem_gb300 as jf
    from oracle import fem as ofem, materials as omat, solve as osolve
    Lz = 1.0
    m = jf.box_mesh(3, 3, 3, 1.0, 1.0, Lz)
    pts, cells = m.points, m.cells_dict["hexahedron"]
    bottom = lambda p: np.isclose(p[2], 0.0, atol=1e-5)
    top = lambda p: np.isclose(p[2], Lz, atol=1e-5)
    zero = lambda p: 0.0
    bc = [[bottom] * 3, [0, 1, 2], [zero, zero, lambda p: 0.01 * Lz]]

    class HyperElasticity(jf.Problem):
        def get_tensor_map(self):
            return jf.NeoHookean(1e3, 0.3, with_rho=True)

        def get_surface_maps(self):
            return [lambda u, x: np.array([0.0, 0.0, 10.0])]

        def set_params(self, params):
            rho, scale_d = params
            self.internal_vars = [rho]
            fe = self.fes[0]
            fe.dirichlet_bc_info[-1][-1] = lambda p: scale_d * Lz
            fe.update_Dirichlet_boundary_conditions(fe.dirichlet_bc_info)

    prob = HyperElasticity(jf.Mesh(pts, cells), vec=3, dim=3, dirichlet_bc_info=[list(b) for b in bc],
                           location_fns=[top])
    opts = {"petsc_solver": {"ksp_type": "cg", "pc_type": "bjacobi", "rtol": 1e-13}, "rel_tol": 1e-12, "tol": 0.0}
    fwd = jf.ad_wrapper(prob, opts, {"petsc_solver": {"ksp_type": "cg", "pc_type": "bjacobi", "rtol": 1e-13}})
    rng = np.random.default_rng(0)
    rho_np = 0.8 + 0.4 * rng.uniform(size=(len(cells), 1))
    sd0 = 0.01
    rho = torch.tensor(rho_np, device=cuda, requires_grad=True)
    sd = torch.tensor(sd0, dtype=torch.float64, device=cuda, requires_grad=True)
    sol = fwd([rho, sd])[0]
    J = (sol ** 2).sum()
    J.backward()
    g_rho, g_sd = rho.grad.cpu().numpy(), sd.grad.item()
    # oracle
    obc = [bc[0], bc[1], [zero, zero, lambda p: sd0 * Lz]]
    op = ofem.OracleProblem(pts, cells, 3, dirichlet_bc_info=obc, location_fns=[top],
                            tensor_map=omat.neo_hookean(1e3, 0.3, with_rho=True),
                            surface_maps=[lambda u, x: torch.tensor([0.0, 0.0, 10.0], dtype=torch.float64)])
    set_p = lambda pr, p: [p[:, None, :].expand(-1, 8, -1)]
    op.internal_vars = set_p(op, torch.tensor(rho_np))
    osol = osolve.newton_solve(op, {"spsolve_solver": {}, "rel_tol": 1e-13, "tol": 0.0}).reshape(-1)
    assert np.abs(sol.detach().cpu().numpy().reshape(-1) - osol).max() <= 1e-9 * np.abs(osol).max()
    v = 2.0 * osol
    g_or, lam = osolve.implicit_vjp(op, osol, rho_np, set_p, v)
    assert np.abs(g_rho - g_or).max() <= 1e-8 * np.abs(g_or).max()
    rows, _ = op.bc_rows()
    zrows = rows[rows % 3 == 2]
    g_sd_or = float(lam[zrows].sum() * Lz)
    assert abs(g_sd - g_sd_or) <= 1e-8 * abs(g_sd_or)
    h = 1e-6
    vals = []
    for sg in (+1, -1):
        with torch.no_grad():
            u = fwd([torch.tensor(rho_np, device=cuda), torch.tensor(sd0 + sg * h, dtype=torch.float64,
                                                                     device=cuda)])[0]
        vals.append((u ** 2).sum().item())
    fd = (vals[0] - vals[1]) / (2 * h)
    assert abs(fd - g_sd) <= 1e-5 * abs(g_sd)
