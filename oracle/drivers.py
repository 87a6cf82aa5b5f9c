"""CPU restatement of jax-fem's arc-length and dynamic-relaxation drivers (test infrastructure
only): arc_length_solver_disp_driven / _force_driven (solver.py:559-721), the outer loops
(solver.py:759-837) and dynamic_relax_solve (solver.py:918-1049), on the oracle FE with scipy
direct solves of the row-eliminated matrix as in the reference."""
import numpy as np
import scipy.sparse.linalg as spla
import torch

from . import fem


def _res_and_A(problem, dofs, scale=1.0):
    res = problem.newton_update(torch.from_numpy(dofs)).numpy()
    res = fem.apply_bc_vec(res, dofs, problem, scale)
    return res, fem.assemble_petsc(problem)


def arc_length_step(problem, u_prev, lam_prev, du_dir, dlam_dir, delta_l, psi, q_m=None):
    """One continuation step; q_m (force control) is the load with zeroed Dirichlet rows."""
    u, lam = u_prev.copy(), lam_prev
    ref = fem.assign_bc(np.zeros_like(u_prev), problem) if q_m is None else q_m
    ref2 = np.sum(ref ** 2)
    res_val = 1.0
    while res_val > 1e-6:
        if q_m is None:
            res, A = _res_and_A(problem, u, lam)
        else:
            res, A = _res_and_A(problem, u)
            res = res + (1.0 - lam) * q_m
        res_val = np.linalg.norm(res)
        A = A.tocsc()
        du_bar = spla.spsolve(A, -res)
        du_t = spla.spsolve(A, ref)
        Du, Dl = u - u_prev, lam - lam_prev
        a1 = np.sum(du_t ** 2) + psi ** 2 * ref2
        a2 = 2 * np.sum((Du + du_bar) * du_t) + 2 * psi ** 2 * Dl * ref2
        a3 = np.sum((Du + du_bar) ** 2) + psi ** 2 * Dl ** 2 * ref2 - delta_l ** 2
        r = np.sqrt(a2 ** 2 - 4 * a1 * a3)
        roots = [(-a2 + r) / (2 * a1), (-a2 - r) / (2 * a1)]
        dots = [np.sum(du_dir * (u + du_bar + dl * du_t - u_prev)) + psi ** 2 * dlam_dir * (lam + dl - lam_prev) * ref2
                for dl in roots]
        if abs(dots[0]) < 1e-10 and abs(dots[1]) < 1e-10:
            dl = max(roots)
        else:
            dl = roots[0] if dots[0] > dots[1] else roots[1]
        lam = lam + dl
        u = u + du_bar + dl * du_t
        du_dir, dlam_dir = u - u_prev, lam - lam_prev
    return u, lam, du_dir, dlam_dir


def arc_length(problem, control, delta_l=0.1, psi=None, max_steps=600, q_aux=None, delta_l_late=1.0, switch=200):
    """Outer continuation loop to lambda >= 1; returns (u, lam, lam history)."""
    n = problem.num_total_dofs_all_vars
    u, lam, du_dir, dlam_dir = np.zeros(n), 0.0, np.zeros(n), 0.0
    q_m = None
    if control == "force":
        q_m = np.asarray(q_aux, dtype=np.float64).copy()
        rows, _ = problem.bc_rows()
        q_m[rows] = 0.0
        psi = 0.5 if psi is None else psi
    else:
        psi = 1.0 if psi is None else psi
    lams = []
    for step in range(max_steps):
        dl = delta_l if (control == "displacement" or step < switch) else delta_l_late
        u, lam, du_dir, dlam_dir = arc_length_step(problem, u, lam, du_dir, dlam_dir, dl, psi, q_m)
        lams.append(lam)
        if lam >= 1.0:
            break
    return u, lam, lams


def dynamic_relax(problem, tol=1e-6, nKMat=1000, max_iters=None):
    """dynamic_relax_solve (solver.py:918-1049) without printing; returns (dofs, iterations)."""
    n = problem.num_total_dofs_all_vars
    rows, _ = problem.bc_rows()
    dofs = np.zeros(n)
    res, A = _res_and_A(problem, dofs)
    dofs = dofs + spla.spsolve(A.tocsc(), -res)

    def resid(x):
        r = problem.compute_residual(torch.from_numpy(x)).numpy().copy()
        r[rows] = 0.0
        return r

    def mass(x):
        _, K = _res_and_A(problem, x)
        return 1.1 * 1.1 / 4.0 * np.asarray(np.abs(K).sum(axis=1)).reshape(-1)

    cmin, cmax, h = 1e-3, 3.9, 1.0
    R = resid(dofs)
    M = mass(dofs)
    q = dofs.copy()
    qdot = -h / 2.0 * R / M
    qdd, qdd_old, q_old = np.zeros(n), np.zeros(n), np.zeros(n)
    it, ik = 0, 0
    error = np.max(np.abs(R))
    while error > tol:
        if max_iters is not None and it >= max_iters:
            break
        q_old[:] = q
        R_old = R.copy()
        q += h * qdot
        R = resid(q)
        it += 1
        ik += 1
        error = np.max(np.abs(R))
        t = np.dot((R - R_old) / h, qdot) / np.einsum("i,i,i", qdot, M, qdot)
        c = min(max(2.0 * np.sqrt(max(t, 0.0)), cmin), cmax)
        dq = q - q_old
        eps = 1.1 * 1.1 / 4.0 * np.abs(np.divide(qdd - qdd_old, dq, out=np.zeros(n), where=dq != 0))
        if np.max(eps) > 1 and ik > nKMat:
            ik = 0
            M = mass(q)
        qdot_old, qdd_old = qdot.copy(), qdd.copy()
        qdot = (2.0 - c * h) / (2.0 + c * h) * qdot_old - 2.0 * h / (2.0 + c * h) * R / M
        qdd = (qdot - qdot_old) / h
    return q, it
