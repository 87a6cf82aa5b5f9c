"""Nonlinear drivers besides Newton: Crisfield arc-length continuation (displacement or force
control) and dynamic relaxation, following jax_fem/solver.py:559-1049.

Both reuse the path's kernels: residual assembly, the tangent, and the Krylov solves.  The
reference's inner solves are direct (scipy spsolve on the row-eliminated matrix); here they are
block-Jacobi PCG to a relative residual of 1e-12 on the symmetric elimination with the Dirichlet
columns lifted, which solves the same row-eliminated system.  Dynamic relaxation's per-iteration
vector work runs in the fused kernels of csrc/fem_drivers.cu.
"""
import ctypes as C
import math
import time

import numpy as np
import torch

from . import _lib
from ._lib import call, ptr
from .logger import logger

LAMBDA_TARGET = 1.0      # solver.py:1085
ARC_MAX_CORRECTIONS = 200


def _dot(a, b):
    return float(torch.dot(a, b).item())


def _solve_rows(eng, dofs, rhs_list, rtol=1e-12):
    """Solve A x = rhs for each rhs, A the row-eliminated tangent at dofs (rows of Dirichlet dofs
    are identity): x_b = rhs_b and K_ff x_f = rhs_f - K_fb rhs_b."""
    A = eng.tangent(dofs, _lib.FEM_SLICED_F64, _lib.FEM_BC_SYMMETRIC)
    rows = eng.bc_rows_long
    out = []
    for rhs in rhs_list:
        b = rhs.clone()
        x = torch.zeros_like(rhs)
        if eng.n_bc:
            x[rows] = rhs[rows]
            if bool((x[rows] != 0).any()):
                b = b - eng.apply(dofs, x, skip_bc_rows=True)
            b[rows] = rhs[rows]
        it, rn, st = eng.krylov("cg", A, b, x, _lib.FEM_PC_BJACOBI, rtol, 0.0, 100000)
        if st == _lib.FEM_SOLVE_NAN:
            raise FloatingPointError("arc-length inner solve produced NaN")
        out.append(x)
    return out


def _arc_length_step(problem, eng, u_prev, lam_prev, du_dir, dlam_dir, delta_l, psi, q_m=None):
    """One continuation step (arc_length_solver_disp_driven, solver.py:559-634, or the force-driven
    variant, solver.py:645-721 when q_m -- the load with zeroed Dirichlet rows -- is given)."""
    from .solver import apply_bc_vec, assign_bc
    u = u_prev.clone()
    lam = lam_prev
    ref = assign_bc(torch.zeros_like(u_prev), problem) if q_m is None else q_m
    ref2 = _dot(ref, ref)

    def pair_dot(a_u, a_l, b_u, b_l):
        return _dot(a_u, b_u) + psi ** 2 * a_l * b_l * ref2

    res_val = 1.0
    corrections = 0
    while res_val > 1e-6:
        corrections += 1
        if corrections > ARC_MAX_CORRECTIONS:
            raise RuntimeError(f"arc-length corrector did not converge in {ARC_MAX_CORRECTIONS} iterations "
                               f"(residual {res_val:.3g})")
        res = eng.residual(u, apply_bc=False)
        if q_m is None:
            res = apply_bc_vec(res, u, problem, lam)
        else:
            res = apply_bc_vec(res, u, problem) + (1.0 - lam) * q_m
        res_val = float(torch.linalg.norm(res).item())
        logger.debug(f"Arc length solver: res_val = {res_val}")
        du_bar, du_t = _solve_rows(eng, u, [-res, ref])
        Du = u - u_prev
        Dl = lam - lam_prev
        w = Du + du_bar
        a1 = _dot(du_t, du_t) + psi ** 2 * ref2
        a2 = 2.0 * _dot(w, du_t) + 2.0 * psi ** 2 * Dl * ref2
        a3 = _dot(w, w) + psi ** 2 * Dl ** 2 * ref2 - delta_l ** 2
        disc = a2 ** 2 - 4.0 * a1 * a3
        if not (disc >= 0.0) or a1 == 0.0:
            raise ValueError(f"No valid solutions for delta lambda, a1 = {a1}, a2 = {a2}, a3 = {a3}")
        r = math.sqrt(disc)
        dl1 = (-a2 + r) / (2.0 * a1)
        dl2 = (-a2 - r) / (2.0 * a1)
        d1 = pair_dot(du_dir, dlam_dir, w + dl1 * du_t, Dl + dl1)
        d2 = pair_dot(du_dir, dlam_dir, w + dl2 * du_t, Dl + dl2)
        if abs(d1) < 1e-10 and abs(d2) < 1e-10:
            dl = max(dl1, dl2)
        elif d1 > d2:
            dl = dl1
        else:
            dl = dl2
        lam = lam + dl
        u = u + du_bar + dl * du_t
        du_dir = u - u_prev
        dlam_dir = lam - lam_prev
    logger.debug(f"Arc length solver: finished for one step, with Delta lambda = {lam - lam_prev}")
    return u, lam, du_dir, dlam_dir


def solve_arc_length(problem, cfg):
    """_solve_arc_length (solver.py:724-855): continuation to lambda = 1, then a Newton polish at
    full load.  Returns (sol_list, info)."""
    from .solver import solver
    eng = problem._engine
    control = cfg.get("control")
    if control not in ("displacement", "force"):
        raise ValueError("arc_length requires cfg['control']; use 'displacement' or 'force'.")
    q_m = None
    if control == "force":
        q_aux = cfg.get("q_vec_aux")
        if q_aux is None:
            raise ValueError("arc_length force control requires cfg['q_vec_aux'].")
        q = torch.as_tensor(q_aux, dtype=torch.float64, device=eng.device).reshape(-1).clone()
        eng.refresh_bc()
        if eng.n_bc:
            q[eng.bc_rows_long] = 0.0
        q_m = q
        psi = cfg.get("psi", 0.5)
        max_steps = cfg.get("max_continuation_steps", 500)
    else:
        psi = cfg.get("psi", 1.0)
        max_steps = cfg.get("max_continuation_steps", 600)
    delta_l = cfg.get("Delta_l", 0.1)
    delta_l_late = cfg.get("Delta_l_late", 1.0)
    switch = cfg.get("Delta_l_switch_step", 200)
    callback = cfg.get("step_callback")
    u = torch.zeros(eng.num_dofs, dtype=torch.float64, device=eng.device)
    lam, du_dir, dlam_dir = 0.0, torch.zeros_like(u), 0.0
    history = []
    logger.info(f"Arc-length solve started ({control} control, Crisfeld).")
    t0 = time.time()
    for step in range(max_steps):
        dl = delta_l if (control == "displacement" or step < switch) else delta_l_late
        u, lam, du_dir, dlam_dir = _arc_length_step(problem, eng, u, lam, du_dir, dlam_dir, dl, psi, q_m)
        rec = {"step": step, "lam": float(lam), "u": u.clone()}
        history.append(rec)
        if callback is not None:
            callback(step, rec["u"], lam)
        if lam >= LAMBDA_TARGET:
            break
    logger.info("Arc-length finished in %.3f s, %d continuation steps, final lambda=%.6f",
                time.time() - t0, len(history), lam)
    sol_list = problem.unflatten_fn_sol_list(u)
    reached = lam >= LAMBDA_TARGET
    if reached:
        polish = dict(cfg.get("newton", {}))
        polish["initial_guess"] = sol_list
        if cfg.get("linear"):
            polish["linear"] = cfg["linear"]
        sol_list = solver(problem, {"newton": polish})
    else:
        logger.warning("Arc-length stopped at lambda=%.6f after %d continuation steps; lambda=1 was not reached",
                       lam, len(history))
    return sol_list, {"lam": float(lam), "lambda_target": LAMBDA_TARGET, "polished": reached, "history": history,
                      "control": control}


def _calc_c(t, cmin, cmax):
    """calC (solver.py:891-899)."""
    t = max(t, 0.0)
    return min(max(2.0 * math.sqrt(t), cmin), cmax)


def dynamic_relax_solve(problem, tol=1e-6, nKMat=1000, nPrint=500, info=True, info_force=True, initial_guess=None,
                        linear_options=None, max_iters=None):
    """dynamic_relax_solve (solver.py:918-1049): one Newton step, then damped explicit dynamics
    with the lumped mass h~^2/4 sum_j |K_ij| of the row-eliminated tangent, recomputed when
    max eps > 1 after nKMat iterations.  Returns sol_list."""
    from .solver import _newton_step, assign_bc, resolve_linear
    eng = problem._engine
    spec = resolve_linear(linear_options or {"spsolve_solver": {}})
    n = eng.num_dofs
    dev = eng.device
    dofs = torch.zeros(n, dtype=torch.float64, device=dev)
    res = eng.residual(dofs, apply_bc=True)
    dofs = _newton_step(problem, eng, dofs, res, spec, "fp64", {})
    if initial_guess is not None:
        dofs = assign_bc(torch.as_tensor(initial_guess, dtype=torch.float64, device=dev).reshape(-1), problem)
    cmin, cmax, h_t, h = 1e-3, 3.9, 1.1, 1.0
    z = lambda: torch.zeros(n, dtype=torch.float64, device=dev)
    q, q_old, qdot, qdot_old, qdd, qdd_old, R_old, M = z(), z(), z(), z(), z(), z(), z(), z()
    ws = torch.empty(4 * 2048 + 4, dtype=torch.float64, device=dev)
    out4 = (C.c_double * 4)()
    s = _lib.stream_handle()

    def residual_zero_bc(x):
        r = eng.residual(x, apply_bc=False)
        if eng.n_bc:
            r[eng.bc_rows_long] = 0.0
        return r

    def lumped_mass(x):
        A = eng.tangent(x, _lib.FEM_F64, _lib.FEM_BC_ROWS, cache=False)
        call("fem_row_abs_sum", n, ptr(eng.indptr), ptr(A.data), h_t * h_t / 4.0, ptr(M), s)

    R = residual_zero_bc(dofs)
    lumped_mass(dofs)
    q.copy_(dofs)
    qdot.copy_(-h / 2.0 * R / M)
    if not (bool(torch.isfinite(M).all()) and bool(torch.isfinite(qdot).all())):
        raise FloatingPointError("dynamic relaxation: non-finite mass or velocity")
    n_iters, i_k = 0, 0
    error = float(R.abs().max().item())
    t0 = time.time()
    while error > tol:
        if max_iters is not None and n_iters >= max_iters:
            break
        call("fem_dr_march", n, h, ptr(q), ptr(q_old), ptr(qdot), ptr(R), ptr(R_old), s)
        R = residual_zero_bc(q)
        n_iters += 1
        i_k += 1
        call("fem_dr_measure", n, h, h_t, ptr(R), ptr(R_old), ptr(qdot), ptr(M), ptr(q), ptr(q_old), ptr(qdd),
             ptr(qdd_old), out4, ptr(ws), ws.numel() * 8, s)
        error, s0, den, eps_max = out4[0], out4[1], out4[2], out4[3]
        t = s0 / den if den != 0.0 else 0.0
        c = _calc_c(t, cmin, cmax)
        if eps_max > 1.0 and i_k > nKMat:
            if info:
                print("\nRecalculating the tangent matrix: ", n_iters)
            i_k = 0
            lumped_mass(q)
        call("fem_dr_velocity", n, h, c, ptr(R), ptr(M), ptr(qdot), ptr(qdot_old), ptr(qdd), ptr(qdd_old), s)
        if n_iters % nPrint == 1 and info_force:
            print(f"\nDR Iteration {n_iters}: Max force (residual error) = {error:g} (tol = {tol:g})")
        if not math.isfinite(error):
            break
    if math.isfinite(error):
        print("DRSolve finished in %d iterations and %fs" % (n_iters, time.time() - t0))
    else:
        print("FAILED to converged")
    problem.dr_info = {"iterations": n_iters, "error": error}
    return problem.unflatten_fn_sol_list(q)
