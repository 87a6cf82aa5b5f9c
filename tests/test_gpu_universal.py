"""get_universal_kernel / get_universal_kernels_surface (problem.py:289-294, :318-323) on the GPU:
the reference's Robin example (applications/robin_bc/example.py:19-80, body source and 5 u^2 Robin
faces, written with numpy) on a 3D HEX8 box, traced, compiled with NVRTC and run as cell / face
kernels.  Against the oracle, which evaluates the same kernels written in torch and differentiates
them with jacfwd like the reference: residual and tangent (1e-12), Newton solution (1e-10); a
conductivity internal variable's ad_wrapper gradient against the oracle's implicit_vjp (1e-9) and
central differences; a vec-3 universal kernel (linear elasticity) against the built-in law."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

from test_jit_host import _kernels  # noqa: E402


def _robin_problem(cuda, n=(5, 4, 3), with_iv=False):
    import jax_fem_gb300 as jf
    from oracle import basis as obasis, fem as ofem
    m = jf.box_mesh(*n, 1.0, 1.0, 1.0)
    pts, cells = m.points, m.cells_dict["hexahedron"]
    t = obasis.element_tables("HEX8")
    uk_np, rk_np = _kernels(t["shape_vals"], 8, 1)
    uk_t, rk_t = _kernels(torch.tensor(t["shape_vals"]), 8, 1, xp=torch,
                          vm=lambda f: (lambda a: torch.stack([f(a[i]) for i in range(a.shape[0])])))
    x0 = lambda p: np.isclose(p[0], 0.0, atol=1e-5)
    x1 = lambda p: np.isclose(p[0], 1.0, atol=1e-5)
    y1 = lambda p: np.isclose(p[1], 1.0, atol=1e-5)
    bc = [[x0], [0], [lambda p: 0.0]]

    class Poisson(jf.Problem):
        def get_universal_kernel(self):
            return uk_np

        def get_universal_kernels_surface(self):
            return [rk_np, rk_np]

        def set_params(self, theta):
            self.internal_vars = [theta]

    prob = Poisson(jf.Mesh(pts, cells), vec=1, dim=3, dirichlet_bc_info=bc, location_fns=[x1, y1])
    oprob = ofem.OracleProblem(pts, cells, 1, dirichlet_bc_info=bc, location_fns=[x1, y1], universal_kernel=uk_t,
                               universal_kernels_surface=[rk_t, rk_t])
    return prob, oprob


def test_universal_residual_tangent_and_solution(cuda):
    import jax_fem_gb300 as jf
    from oracle import fem as ofem, solve as osolve
    prob, oprob = _robin_problem(cuda)
    th = np.random.default_rng(0).uniform(0.5, 1.5, (prob.num_cells, 8, 1))
    prob.set_params(torch.tensor(th, device=cuda))
    oprob.internal_vars = [torch.tensor(th)]
    u = np.random.default_rng(1).standard_normal(oprob.num_total_dofs_all_vars) * 0.3
    r = prob.compute_residual([torch.tensor(u, device=cuda).reshape(-1, 1)])[0].reshape(-1).cpu().numpy()
    ro = oprob.compute_residual(torch.tensor(u)).numpy()
    assert np.abs(r - ro).max() <= 1e-12 * np.abs(ro).max()
    prob.newton_update([torch.tensor(u, device=cuda).reshape(-1, 1)])
    A = jf.get_A(prob)
    oprob.newton_update(torch.tensor(u))
    Ao = ofem.assemble_petsc(oprob)
    assert np.abs(A.data.cpu().numpy() - Ao.data).max() <= 1e-12 * np.abs(Ao.data).max()
    # the tangent action (dual sweep along w) equals the assembled tangent times w
    eng = prob._engine
    w = torch.tensor(np.random.default_rng(2).standard_normal(eng.num_dofs), device=cuda)
    K = eng.tangent(torch.tensor(u, device=cuda), jf._lib.FEM_F64, jf._lib.FEM_BC_NONE, cache=False)
    assert (eng.apply(torch.tensor(u, device=cuda), w, skip_bc_rows=False) - K.matvec(w)).abs().max().item() <= \
        1e-12 * K.matvec(w).abs().max().item()
    opts = {"jax_solver": {"tol": 1e-13, "atol": 1e-30}, "rel_tol": 1e-12, "tol": 0.0}
    sol = jf.solver(prob, opts)[0].reshape(-1).cpu().numpy()
    osol = osolve.newton_solve(oprob, {"spsolve_solver": {}, "rel_tol": 1e-12, "tol": 0.0}).reshape(-1)
    assert np.abs(sol - osol).max() <= 1e-10 * np.abs(osol).max()


def test_universal_internal_variable_gradient(cuda):
    import jax_fem_gb300 as jf
    from oracle import solve as osolve
    prob, oprob = _robin_problem(cuda, n=(4, 3, 3))
    rng = np.random.default_rng(3)
    th = rng.uniform(0.5, 1.5, (prob.num_cells, 8, 1))
    wv = torch.tensor(rng.standard_normal(prob._engine.num_dofs), device=cuda)
    opts = {"jax_solver": {"tol": 1e-13, "atol": 1e-30}, "rel_tol": 1e-12, "tol": 0.0}
    fwd = jf.ad_wrapper(prob, opts, {"jax_solver": {"tol": 1e-13, "atol": 1e-30}})
    theta = torch.tensor(th, device=cuda, requires_grad=True)
    sol = fwd(theta)[0]
    J = torch.dot(wv, sol.reshape(-1))
    J.backward()
    g = theta.grad.cpu().numpy()
    set_p = lambda pr, p: [p]
    oprob.internal_vars = [torch.tensor(th)]
    osol = osolve.newton_solve(oprob, {"spsolve_solver": {}, "rel_tol": 1e-12, "tol": 0.0}).reshape(-1)
    g_or, _ = osolve.implicit_vjp(oprob, osol, th, set_p, wv.cpu().numpy())
    assert np.abs(g - g_or).max() <= 1e-9 * np.abs(g_or).max()
    c, q = 5, 3
    h = 1e-6
    vals = []
    for s in (+1, -1):
        tp = th.copy()
        tp[c, q, 0] += s * h
        with torch.no_grad():
            vals.append(torch.dot(wv, fwd(torch.tensor(tp, device=cuda))[0].reshape(-1)).item())
    fd = (vals[0] - vals[1]) / (2 * h)
    assert abs(fd - g[c, q, 0]) <= 1e-6 * np.abs(g).max()


def test_universal_vec3_matches_builtin_elasticity(cuda):
    """Linear elasticity written as a universal kernel (vec 3) gives the built-in LinearElastic
    residual and tangent: the dof layout of the compiled kernels (node*vec + comp) is the engine's."""
    import jax_fem_gb300 as jf
    m = jf.box_mesh(3, 3, 2, 1.0, 1.0, 1.0)
    pts, cells = m.points, m.cells_dict["hexahedron"]
    x0 = lambda p: np.isclose(p[0], 0.0, atol=1e-5)
    bc = [[x0] * 3, [0, 1, 2], [lambda p: 0.0] * 3]
    E, nu = 70e3, 0.3
    lam, mu = E * nu / ((1 + nu) * (1 - 2 * nu)), E / (2 * (1 + nu))

    def elastic_kernel(cell_sol_flat, x, cell_shape_grads, cell_JxW, cell_v_grads_JxW):
        cs = cell_sol_flat.reshape(8, 3)
        ug = (cs[None, :, :, None] * cell_shape_grads[:, :, None, :]).sum(1)        # (nq, 3, 3)
        eps = 0.5 * (ug + ug.transpose(0, 2, 1))
        tr = eps[:, 0, 0] + eps[:, 1, 1] + eps[:, 2, 2]
        sig = lam * tr[:, None, None] * np.eye(3)[None] + 2 * mu * eps
        return (sig[:, None, :, :] * cell_v_grads_JxW).sum((0, 3)).reshape(-1)

    class U(jf.Problem):
        def get_universal_kernel(self):
            return elastic_kernel

    class B(jf.Problem):
        def get_tensor_map(self):
            return jf.LinearElastic(E, nu)

    pu = U(jf.Mesh(pts, cells), vec=3, dim=3, dirichlet_bc_info=bc)
    pb = B(jf.Mesh(pts, cells), vec=3, dim=3, dirichlet_bc_info=bc)
    u = torch.tensor(np.random.default_rng(4).standard_normal(3 * len(pts)) * 1e-3, device=cuda)
    ru = pu.compute_residual([u.reshape(-1, 3)])[0].reshape(-1)
    rb = pb.compute_residual([u.reshape(-1, 3)])[0].reshape(-1)
    assert (ru - rb).abs().max().item() <= 1e-12 * rb.abs().max().item()
    L = jf._lib
    for mode in (L.FEM_BC_NONE, L.FEM_BC_ROWS, L.FEM_BC_SYMMETRIC):
        Ku = pu._engine.tangent(u, L.FEM_F64, mode, cache=False).data
        Kb = pb._engine.tangent(u, L.FEM_F64, mode, cache=False).data
        assert (Ku - Kb).abs().max().item() <= 1e-12 * Kb.abs().max().item(), mode
