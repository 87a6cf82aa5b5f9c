"""GPU tests of the J2 history adjoint (gradients over load steps, the reference's jax.grad over
fwd_pred + update_int_vars_gp loops): the kernel's reverse mode against torch autograd of the
oracle's return map, and a multi-step gradient against central finite differences."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

E, NU, SIG0 = 70e3, 0.3, 250.0


def _j2_problem(n, modulus_field=True, ramp_face=False):
    import jax_fem_gb300 as jf
    m = jf.box_mesh(n, n, n, 1.0, 1.0, 1.0)
    pts, cells = m.points, m.cells_dict["hexahedron"]
    left = lambda p: np.isclose(p[0], 0.0, atol=1e-5)
    right = lambda p: np.isclose(p[0], 1.0, atol=1e-5)
    zero = lambda p: 0.0
    if ramp_face:
        bc = [[left] * 3 + [right] * 3, [0, 1, 2, 0, 1, 2], [zero] * 3 + [lambda p: 0.0, zero, zero]]
    else:
        bc = [[left] * 3, [0, 1, 2], [zero] * 3]

    class P(jf.Problem):
        def get_tensor_map(self):
            return jf.J2Plasticity(E, NU, SIG0, modulus_field=modulus_field)

        def set_params(self, params):
            mu, sig, eps = params
            self.internal_vars = [sig, eps, mu[:, None].expand(-1, 8)]

    prob = P(jf.Mesh(pts, cells), vec=3, dim=3, dirichlet_bc_info=bc)
    return prob, bc, pts, cells


def _oracle_fe(pts, cells, bc):
    from oracle import fem as ofem
    return ofem.OracleProblem(pts, cells, 3, dirichlet_bc_info=bc)


def test_j2_history_vjp_matches_autograd(cuda):
    """fem_j2_history_vjp against torch autograd of the oracle's return map
    (test_plasticity.py:54-78), at a state with both elastic and plastic points:
    update mode (cotangents of sigma_new, eps_new -> u, sigma_old, eps_old, modulus scale) and
    adjoint mode (-lam^T dR/d history).  Tolerance 1e-10 of the largest entry."""
    from oracle import materials as omat
    prob, bc, pts, cells = _j2_problem(2)
    eng = prob._engine
    nc, nq = eng.num_cells, eng.num_quads
    g = torch.Generator().manual_seed(7)
    u = (torch.rand(eng.num_dofs, generator=g, dtype=torch.float64) - 0.5) * 6e-3
    A = torch.randn(nc, nq, 3, 3, generator=g, dtype=torch.float64) * 80.0
    sig_old = 0.5 * (A + A.transpose(-1, -2))
    B = torch.randn(nc, nq, 3, 3, generator=g, dtype=torch.float64) * 1e-3
    eps_old = 0.5 * (B + B.transpose(-1, -2))
    mu = 0.8 + 0.4 * torch.rand(nc, generator=g, dtype=torch.float64)
    hbar = torch.randn(nc, nq, 18, generator=g, dtype=torch.float64)
    lam = torch.randn(eng.num_dofs, generator=g, dtype=torch.float64)

    prob.set_params([mu.to(cuda), sig_old.to(cuda), eps_old.to(cuda)])
    dofs = u.to(cuda)
    hg, sg, ug = eng.j2_history_vjp(dofs, hist_bar=hbar.to(cuda), want_scale=True, want_u=True)
    hg_a, sg_a, _ = eng.j2_history_vjp(dofs, lam=lam.to(cuda), want_scale=True)

    # oracle: per-point return map under torch autograd
    of = _oracle_fe(pts, cells, bc)
    strain, rmap = omat.j2_maps(E, NU, SIG0, mu_field=True)
    uu = u.clone().requires_grad_(True)
    so = sig_old.clone().requires_grad_(True)
    eo = eps_old.clone().requires_grad_(True)
    mq = mu[:, None].expand(-1, nq).clone().requires_grad_(True)
    ug_c = torch.einsum("cnv,cqnd->cqvd", uu.reshape(-1, 3)[torch.as_tensor(cells)], of.shape_grads)
    f = torch.func.vmap(torch.func.vmap(rmap))
    sig_new = f(ug_c, so, eo, mq[..., None])
    eps_new = 0.5 * (ug_c + ug_c.transpose(-1, -2))
    # both modes are checked to reach elastic and plastic points
    s_dev = sig_new - torch.einsum("cqii->cq", sig_new)[..., None, None] / 3 * torch.eye(3, dtype=torch.float64)
    q = torch.sqrt(1.5 * (s_dev ** 2).sum((-1, -2)))
    n_plastic = int((q > SIG0 * (1 - 1e-9)).sum())
    assert 0 < n_plastic < nc * nq, n_plastic
    L = (hbar[..., :9].reshape(nc, nq, 3, 3) * sig_new).sum() + (hbar[..., 9:].reshape(nc, nq, 3, 3) * eps_new).sum()
    gu, gso, geo, gm = torch.autograd.grad(L, [uu, so, eo, mq])
    ref_h = torch.cat([gso.reshape(nc, nq, 9), geo.reshape(nc, nq, 9)], 2)

    def close(a, b, tol=1e-10):
        a = a.detach().cpu().double().reshape(-1)
        b = b.detach().double().reshape(-1)
        assert (a - b).abs().max().item() <= tol * b.abs().max().item()

    close(hg, ref_h)
    close(sg, gm)
    close(ug, gu)

    # adjoint mode: -lam^T R(u; history, scale) with lam masked on Dirichlet dofs
    mask = torch.zeros(eng.num_dofs, dtype=torch.bool)
    rows, _ = of.bc_rows()
    mask[torch.as_tensor(rows, dtype=torch.long)] = True
    lam_m = torch.where(mask, torch.zeros_like(lam), lam)
    so2 = sig_old.clone().requires_grad_(True)
    eo2 = eps_old.clone().requires_grad_(True)
    mq2 = mu[:, None].expand(-1, nq).clone().requires_grad_(True)
    ug_c2 = torch.einsum("cnv,cqnd->cqvd", u.reshape(-1, 3)[torch.as_tensor(cells)], of.shape_grads)
    sig2 = f(ug_c2, so2, eo2, mq2[..., None])
    R = torch.einsum("cqvd,cqnd->cnv", sig2, of.v_grads_JxW)   # per-cell residual (cells, nn, 3)
    lam_c = lam_m.reshape(-1, 3)[torch.as_tensor(cells)]
    Lr = (lam_c * R).sum()
    a_so, a_eo, a_m = torch.autograd.grad(Lr, [so2, eo2, mq2])
    close(hg_a, -torch.cat([a_so.reshape(nc, nq, 9), a_eo.reshape(nc, nq, 9)], 2))
    close(sg_a, -a_m)


def _multi_step_objective(prob, bc, mu, disps, u_target, opts):
    import jax_fem_gb300 as jf
    eng = prob._engine
    nc, nq = eng.num_cells, eng.num_quads
    sig = torch.zeros(nc, nq, 3, 3, dtype=torch.float64, device=mu.device)
    eps = torch.zeros_like(sig)
    fwd = jf.ad_wrapper(prob, opts, opts)
    sol = None
    for d in disps:
        bc[2][3] = (lambda p, d=d: d)
        prob.fes[0].update_Dirichlet_boundary_conditions(bc)
        sol = fwd([mu, sig, eps])[0]
        sig, eps = jf.update_j2_history(prob, sol, sig, eps, mu[:, None].expand(-1, nq))
    return ((sol - u_target) ** 2).sum()


def test_j2_multi_step_gradient_vs_fd(cuda):
    """Gradient of ||u_3 - u_target||^2 with respect to a per-cell modulus field through three
    load steps (x=1 face u_x ramp) -- the implicit adjoint of every step plus the reverse mode of
    every history update -- against central finite differences along two random directions
    (h = 1e-5; tolerance 1e-5 relative)."""
    prob, bc, pts, cells = _j2_problem(3, ramp_face=True)
    eng = prob._engine
    disps = [2e-3, 4e-3, 6e-3]
    opts = {"petsc_solver": {"ksp_type": "cg", "pc_type": "jacobi", "rtol": 1e-14}, "rel_tol": 1e-12, "tol": 1e-10}
    g = torch.Generator().manual_seed(3)
    mu0 = (0.8 + 0.4 * torch.rand(eng.num_cells, generator=g, dtype=torch.float64)).to(cuda)
    u_target = (torch.rand(eng.num_nodes, 3, generator=g, dtype=torch.float64) * 1e-3).to(cuda)

    mu = mu0.clone().requires_grad_(True)
    J = _multi_step_objective(prob, bc, mu, disps, u_target, opts)
    J.backward()
    grad = mu.grad.detach()
    assert torch.isfinite(grad).all() and grad.abs().max().item() > 0
    for k in range(2):
        v = torch.randn(eng.num_cells, generator=g, dtype=torch.float64).to(cuda)
        h = 1e-5
        with torch.no_grad():
            Jp = _multi_step_objective(prob, bc, mu0 + h * v, disps, u_target, opts).item()
            Jm = _multi_step_objective(prob, bc, mu0 - h * v, disps, u_target, opts).item()
        fd = (Jp - Jm) / (2 * h)
        an = torch.dot(grad, v).item()
        assert abs(fd - an) <= 1e-5 * max(abs(fd), abs(an)), (k, fd, an)
