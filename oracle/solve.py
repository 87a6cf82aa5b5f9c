"""FP64 CPU restatement of jax-fem's solver layer (test infrastructure).

  linear solvers          jax_fem/solver.py:63-134, 261-284
  Newton loop             jax_fem/solver.py:390-421, 1112-1356
  implicit adjoint        jax_fem/solver.py:1362-1418
"""
import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla
import torch

from . import fem


def bicgstab_jax(A, b, x0=None, M=None, tol=1e-10, atol=1e-10, maxiter=10000):
    """Restates the published jax.scipy.sparse.linalg.bicgstab iteration used by
    jax_solve (solver.py:78-84): stop when ||r||^2 <= max(tol^2 ||b||^2, atol^2),
    initial p = q = r0, rho = alpha = omega = 1, early exit on ||s|| small,
    breakdown when rho, alpha or omega is 0.  Returns (x, iterations)."""
    x = np.zeros_like(b) if x0 is None else np.array(x0, dtype=np.float64)
    Mf = (lambda v: v) if M is None else M
    bs = b @ b
    atol2 = max(tol * tol * bs, atol * atol)
    r = b - A @ x
    rhat = r.copy()
    p = r.copy()
    q = r.copy()
    rho = alpha = omega = 1.0
    k = 0
    while (r @ r) > atol2 and k < maxiter and k >= 0:
        rho_ = rhat @ r
        beta = rho_ / rho * alpha / omega
        p = r + beta * (p - omega * q)
        phat = Mf(p)
        q = A @ phat
        alpha_ = rho_ / (rhat @ q)
        s = r - alpha_ * q
        exit_early = (s @ s) < atol2
        shat = Mf(s)
        t = A @ shat
        omega_ = (t @ s) / (t @ t)
        if exit_early:
            x = x + alpha_ * phat
            r = s
        else:
            x = x + alpha_ * phat + omega_ * shat
            r = s - omega_ * t
        k = k + 1
        if omega_ == 0 or alpha_ == 0:
            k = -11
        if rho_ == 0:
            k = -10
        rho, alpha, omega = rho_, alpha_, omega_
    return x, k


def pcg(A, b, x0=None, Minv=None, rtol=1e-10, atol=0.0, maxiter=100000):
    """Preconditioned CG (PETSc KSPCG + PCJACOBI semantics on an SPD system),
    stopping on the unpreconditioned residual: ||r|| <= max(rtol ||b||, atol)."""
    x = np.zeros_like(b) if x0 is None else np.array(x0, dtype=np.float64)
    Minv = (lambda v: v) if Minv is None else Minv
    r = b - A @ x
    thresh = max(rtol * np.linalg.norm(b), atol)
    z = Minv(r)
    p = z.copy()
    rz = r @ z
    it = 0
    while np.linalg.norm(r) > thresh and it < maxiter:
        q = A @ p
        alpha = rz / (p @ q)
        x += alpha * p
        r -= alpha * q
        z = Minv(r)
        rz_new = r @ z
        p = z + (rz_new / rz) * p
        rz = rz_new
        it += 1
    return x, it


def linear_solver(A, b, x0, linear_options):
    """solver.py:261-284 dispatch (CPU)."""
    opts = dict(linear_options)
    if len(opts.keys() & {"jax_solver", "spsolve_solver", "petsc_solver", "custom_solver", "oracle_pcg"}) == 0:
        opts["jax_solver"] = {}
    if "jax_solver" in opts:
        precond = opts["jax_solver"].get("precond", True)
        jac = A.diagonal()
        M = (lambda v: v / jac) if precond else None
        x, _ = bicgstab_jax(A, b, x0, M)
        err = np.linalg.norm(A @ x - b)
        assert err < 0.1, f"JAX linear solver failed to converge with err = {err}"
        return x
    if "oracle_pcg" in opts:
        jac = A.diagonal()
        x, _ = pcg(A, b, x0, lambda v: v / jac, rtol=opts["oracle_pcg"].get("rtol", 1e-12))
        return x
    if "spsolve_solver" in opts or "petsc_solver" in opts:
        return spla.spsolve(sp.csr_matrix(A), b)
    if "custom_solver" in opts:
        return opts["custom_solver"](A, b, x0, opts)
    raise NotImplementedError("Unknown linear solver.")


def newton_solve(problem, solver_options=None, return_info=False):
    """solver.py:1112-1356 (Newton branch): BC row elimination, x0 BC-consistent,
    stop when rel_res <= rel_tol or res <= tol."""
    opts = dict(solver_options or {})
    linear = {k: opts[k] for k in ("jax_solver", "spsolve_solver", "petsc_solver", "custom_solver", "oracle_pcg") if k in opts}
    rel_tol = opts.get("rel_tol", 1e-8)
    tol = opts.get("tol", 1e-6)
    if "initial_guess" in opts:
        dofs = np.asarray(opts["initial_guess"], dtype=np.float64).reshape(-1).copy()
    else:
        dofs = np.zeros(problem.num_total_dofs_all_vars)

    def update(d):
        res = problem.newton_update(torch.from_numpy(d)).numpy()
        res = fem.apply_bc_vec(res, d, problem)
        A = fem.assemble_petsc(problem)
        return res, A

    res, A = update(dofs)
    res0 = np.linalg.norm(res)
    rel = 1.0 if res0 == 0 else np.linalg.norm(res) / res0
    its = 0
    while rel > rel_tol and np.linalg.norm(res) > tol:
        its += 1
        x0 = fem.assign_bc(np.zeros_like(dofs), problem) - fem.copy_bc(dofs, problem)
        inc = linear_solver(A, -res, x0, linear)
        dofs = dofs + inc
        res, A = update(dofs)
        rel = np.linalg.norm(res) / res0
        if its > 200:
            raise RuntimeError("oracle Newton did not converge")
    assert np.all(np.isfinite(dofs))
    sol = dofs.reshape(-1, problem.vec)
    if return_info:
        return sol, dict(iterations=its, res=np.linalg.norm(res), res0=res0, A=A)
    return sol


def implicit_vjp(problem, sol, params, set_params, v, adjoint_options=None):
    """solver.py:1362-1418: A = get_A at u*, solve A^T lam = v, return -vjp_p[c](lam)
    with c(u, p) = apply_bc(R(u; set_params(p))).  `set_params(problem, p)` must
    return the internal_vars list (torch, differentiable in p)."""
    dofs = np.asarray(sol, dtype=np.float64).reshape(-1)
    problem.internal_vars = [t.detach() for t in set_params(problem, torch.as_tensor(params))]
    problem.newton_update(torch.from_numpy(dofs))
    A = fem.assemble_petsc(problem)
    lam = linear_solver(A.T.tocsr(), np.asarray(v, dtype=np.float64).reshape(-1), None,
                        adjoint_options or {"spsolve_solver": {}})
    p = torch.as_tensor(params).clone().requires_grad_(True)
    iv = set_params(problem, p)
    res = problem.compute_residual(torch.from_numpy(dofs), iv, problem.internal_vars_surfaces)
    # BC rows of c are u_b - g (solver.py:290-304): independent of p, so mask them
    rows, _ = problem.bc_rows()
    lam_t = torch.from_numpy(lam.copy())
    lam_t[torch.from_numpy(rows)] = 0.0
    (g,) = torch.autograd.grad(res, p, grad_outputs=lam_t)
    return -g.numpy(), lam
