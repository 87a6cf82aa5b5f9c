"""solver(), linear_solver(), get_A(), implicit_vjp() and ad_wrapper() on the GB300 engine.

Mirrors jax_fem/solver.py (Newton branch, 63-553 and 1079-1455):

  * solver_options has the same layout: a 'newton' block (or the legacy flat
    dict) with tol / rel_tol / line_search_flag / initial_guess and a 'linear'
    block naming jax_solver / petsc_solver / spsolve_solver / custom_solver.
    Additional keys: 'precision' ('fp64' default; 'mixed': CG on a DF48 copy of
    the FP64 tangent (sliced storage) with double-float vectors and FP64
    reliable updates; 'mixed_sliced' is the same; 'mixed_ssym': on a structured
    box grid of nodes, only the diagonal and upper stencil blocks
    (FEM_SSYM_DF48, half the matrix bytes, slower on GB300: issue bound);
    'mixed_sym': upper-block storage of a general pattern with the transposed
    half by FP64 atomics; 'mixed32': FP32 matrix and
    vectors with FP64 reliable updates -- BiCGStab under a mixed precision runs
    in FP32 and Newton's FP64 residual refines it), 'inner_rtol' (that
    BiCGStab's tolerance), 'refine_delta', 'max_iter' (Newton cap).
  * jax_solver -> BiCGStab with jax.scipy's iteration and stopping rule on the
    row-eliminated matrix (solver.py:63-92), Jacobi if precond.
  * petsc_solver ksp_type 'cg' -> PCG on the symmetrically eliminated matrix
    (Dirichlet columns lifted to the right-hand side: same solution as the
    reference's row elimination because x0 is BC-consistent, solver.py:402-409);
    other Krylov types -> BiCGStab.  pc_type 'jacobi' -> Jacobi, 'none' -> none,
    anything else -> 3x3 node-block Jacobi.
  * spsolve_solver has no direct GPU counterpart here: it is served by
    block-Jacobi PCG to a relative residual of 1e-12.
  * amgx_solver is not part of this build (NotImplementedError).
"""
import time

import numpy as np
import torch

from . import _lib
from .logger import logger

_METHOD_KEYS = frozenset({"newton", "arc_length", "dynamic_relax"})
_LINEAR_OPTION_KEYS = frozenset({"jax_solver", "amgx_solver", "spsolve_solver", "petsc_solver", "custom_solver"})
_NEWTON_OPTION_KEYS = frozenset({"tol", "rel_tol", "line_search_flag", "initial_guess", "precision", "inner_rtol",
                                 "max_iter", "refine_delta"})


def _resolve_solver_options(solver_options):
    """solver.py:1088-1106 (same rules) -> ('newton', cfg)."""
    opts = solver_options or {}
    methods = [m for m in _METHOD_KEYS if m in opts]
    if not methods:
        linear = {k: opts[k] for k in _LINEAR_OPTION_KEYS if k in opts}
        cfg = {k: opts[k] for k in _NEWTON_OPTION_KEYS if k in opts}
        if linear:
            cfg["linear"] = linear
        return "newton", cfg
    if len(methods) > 1:
        raise ValueError(f"Pick one nonlinear method, got {methods}.")
    method = methods[0]
    if not isinstance(opts[method], dict):
        raise ValueError(f"solver_options['{method}'] must be a dict.")
    return method, opts[method]


class LinearSpec:
    """Resolved linear solver: Krylov method, preconditioner, Dirichlet handling, tolerances."""

    def __init__(self, method, pc, bc_mode, rtol, atol, maxiter, custom=None, options=None):
        self.method, self.pc, self.bc_mode = method, pc, bc_mode
        self.rtol, self.atol, self.maxiter = rtol, atol, maxiter
        self.custom, self.options = custom, options

    def __repr__(self):
        return f"LinearSpec({self.method}, pc={self.pc}, rtol={self.rtol}, atol={self.atol})"


_PC = {"jacobi": _lib.FEM_PC_JACOBI, "none": _lib.FEM_PC_NONE, "bjacobi": _lib.FEM_PC_BJACOBI}


def resolve_linear(linear_options):
    """solver.py:261-284 dispatch rules -> LinearSpec."""
    lo = linear_options if linear_options is not None else {}
    if len(lo.keys() & _LINEAR_OPTION_KEYS) == 0:
        lo["jax_solver"] = {}
    if "jax_solver" in lo:
        precond = lo["jax_solver"].get("precond", True)
        o = lo["jax_solver"]
        return LinearSpec("bicgstab", _lib.FEM_PC_JACOBI if precond else _lib.FEM_PC_NONE, _lib.FEM_BC_ROWS,
                          o.get("tol", 1e-10), o.get("atol", 1e-10), o.get("maxiter", 10000))
    if "amgx_solver" in lo:
        raise NotImplementedError("amgx_solver is not part of this build (use petsc_solver cg + jacobi/bjacobi)")
    if "spsolve_solver" in lo:
        o = lo["spsolve_solver"]
        return LinearSpec("cg", _lib.FEM_PC_BJACOBI, _lib.FEM_BC_SYMMETRIC, o.get("rtol", 1e-12), o.get("atol", 0.0),
                          o.get("max_it", 100000))
    if "petsc_solver" in lo:
        o = lo["petsc_solver"]
        ksp = o.get("ksp_type", "bcgsl")
        pc = o.get("pc_type", "ilu")
        if ksp == "preonly":
            raise NotImplementedError("ksp_type 'preonly' (direct factorisation) is not part of this build")
        method = "cg" if ksp == "cg" else "bicgstab"
        pck = _PC.get(pc, _lib.FEM_PC_BJACOBI)
        if pc not in _PC:
            logger.info("pc_type %r served by 3x3 node-block Jacobi", pc)
        bc = _lib.FEM_BC_SYMMETRIC if method == "cg" else _lib.FEM_BC_ROWS
        return LinearSpec(method, pck, bc, o.get("rtol", 1e-5), o.get("atol", 1e-50), o.get("max_it", 10000))
    if "custom_solver" in lo:
        return LinearSpec("custom", _lib.FEM_PC_NONE, _lib.FEM_BC_ROWS, 0.0, 0.0, 0, custom=lo["custom_solver"],
                          options=lo)
    raise NotImplementedError("Unknown linear solver.")


def _precision(cfg):
    p = cfg.get("precision", "fp64")
    if p not in ("fp64", "mixed", "mixed_sliced", "mixed_ssym", "mixed_sym", "mixed32"):
        raise ValueError("precision must be 'fp64', 'mixed' or 'mixed_sliced' (sliced DF48 matrix, double-float "
                         "vectors), 'mixed_ssym' (the same with structured symmetric stencil storage on a box "
                         "grid), 'mixed_sym' (upper-block DF48 storage of a general pattern) or 'mixed32' (FP32)")
    return p


def _mixed_matrix_precision(precision, eng=None):
    """Solver copy of the tangent.  'mixed' / 'mixed_sliced': sliced DF48 (the fastest measured on
    GB300: the SpMV streams at ~0.9 of the copy peak); 'mixed_ssym': the structured symmetric DF48
    layout (diagonal and upper stencil blocks, implicit columns; the transposed half in registers
    and warp shuffles) when the nodes form a box grid (eng.grid) and the tangent is symmetric,
    sliced DF48 otherwise -- it moves 0.52x the bytes but its double-float arithmetic is issue
    bound (456 us against 260-277 us per SpMV at 1M cells); 'mixed_sym': upper node blocks of the
    general pattern with the transposed half through FP64 atomics (slower on GB300: the atomics
    cost more than the bytes saved); sliced FP32 for 'mixed32'."""
    if precision == "mixed_sym" and eng is not None and eng.vec == 3 and getattr(eng._mat, "symmetric", False):
        return _lib.FEM_SYM_DF48
    if precision == "mixed_ssym" and eng is not None and eng.grid is not None and eng.tangent_symmetric:
        return _lib.FEM_SSYM_DF48
    if precision in ("mixed", "mixed_sym", "mixed_sliced", "mixed_ssym"):
        return _lib.FEM_SLICED_DF48
    return _lib.FEM_SLICED_F32


_FP64_SOLVER_FORMAT = _lib.FEM_SLICED_F64     # FP64 Krylov iterations run on the sliced FP64 copy


def get_A(problem):
    """solver.py:540-553: tangent at the last newton_update point with PETSc zeroRows
    semantics (rows := 0, diag := 1, pattern kept), FP64."""
    eng = problem._engine
    point = getattr(problem, "_newton_point", None)
    if point is None:
        raise RuntimeError("call problem.newton_update(sol_list) first")
    return eng.tangent(point, _lib.FEM_F64, _lib.FEM_BC_ROWS, cache=False)


def linear_solver(A, b, x0, linear_options, precision="fp64", inner_rtol=1e-5):
    """Solve A x = b on the device (solver.py:261-284).  A is a DeviceCSR; b, x0 FP64 tensors."""
    spec = resolve_linear(linear_options)
    eng = A.eng
    if spec.custom is not None:
        return spec.custom(A, b, x0, linear_options)
    if A.precision in (_lib.FEM_DF48, _lib.FEM_SLICED_DF48, _lib.FEM_SYM_DF48, _lib.FEM_SSYM_DF48):
        raise NotImplementedError("DF48 matrices are solved by the mixed Newton / adjoint paths (fem_pcg_refined)")
    x = torch.zeros_like(b) if x0 is None else x0.clone()
    if A.vector_dtype == torch.float64:
        it, rn, st = eng.krylov(spec.method, A, b.contiguous(), x, spec.pc, spec.rtol, spec.atol, spec.maxiter)
        return x, (it, rn, st)
    b32 = eng.cast32(b)
    x32 = eng.cast32(x)
    it, rn, st = eng.krylov(spec.method, A, b32, x32, spec.pc, inner_rtol, 0.0, spec.maxiter)
    return x32.double(), (it, rn, st)


def _timed(eng, key, t0):
    if eng.sync_timing:
        torch.cuda.current_stream().synchronize()
    eng.timing[key] += time.perf_counter() - t0


def _newton_step(problem, eng, dofs, res, spec, precision, cfg):
    """One Newton correction A inc = -res (solver.py:390-421) with the Dirichlet rows of the
    increment equal to g - u_b."""
    prec = _FP64_SOLVER_FORMAT if precision == "fp64" else _mixed_matrix_precision(precision, eng)
    if prec in (_lib.FEM_SLICED_DF48, _lib.FEM_SYM_DF48, _lib.FEM_SSYM_DF48) and spec.method != "cg":
        prec = _lib.FEM_SLICED_F32   # BiCGStab mixed path runs in FP32 with Newton-level refinement
    eng.refresh_bc()
    rows = eng.bc_rows_long
    du_b = eng.bc_vals - dofs[rows] if eng.n_bc else None
    t0 = time.perf_counter()
    if spec.custom is not None:
        A = eng.tangent(dofs, _lib.FEM_F64, _lib.FEM_BC_ROWS)
        x0 = torch.zeros_like(dofs)
        if eng.n_bc:
            x0[rows] = du_b
        inc = torch.as_tensor(spec.custom(A, -res, x0, spec.options), dtype=torch.float64, device=dofs.device)
        eng.timing["linear"] += time.perf_counter() - t0
        return dofs + inc.reshape(-1)
    A = eng.tangent(dofs, prec, spec.bc_mode)
    _timed(eng, "global_matrix", t0)
    t0 = time.perf_counter()
    b = -res
    x0 = torch.zeros_like(dofs)
    if eng.n_bc:
        x0[rows] = du_b
        if spec.bc_mode == _lib.FEM_BC_SYMMETRIC and bool((du_b != 0).any()):
            # lift the eliminated Dirichlet columns: b_f -= K_fb (g - u_b)
            b = b - eng.apply(dofs, x0, skip_bc_rows=True)
        b[rows] = du_b
    inner = cfg.get("inner_rtol", 1e-5)
    if prec == _FP64_SOLVER_FORMAT:
        x = x0.clone()
        it, rn, st = eng.krylov(spec.method, A, b, x, spec.pc, spec.rtol, spec.atol, spec.maxiter)
        if spec.method == "bicgstab":
            err = torch.linalg.norm(A.matvec(x) - b).item()      # solver.py:86-89
            assert err < 0.1, f"linear solver failed to converge with err = {err}"
        inc = x
    elif spec.method == "cg":
        # PCG with FP64 reliable updates (double-float on the DF48 copy for 'mixed', FP32 for
        # 'mixed32'): converges on the FP64 true residual
        x = x0.clone()
        it, up, rn, st = eng.pcg_refined(A, b, x, dofs, spec.pc, spec.rtol, spec.atol,
                                         cfg.get("refine_delta", 0.1), spec.maxiter)
        inc = x
    else:
        # BiCGStab in FP32; the Newton loop's FP64 residual acts as the refinement
        b32 = eng.cast32(b)
        x32 = eng.cast32(x0)
        it, rn, st = eng.krylov(spec.method, A, b32, x32, spec.pc, inner, 0.0, spec.maxiter)
        inc = None
    _timed(eng, "linear", t0)
    if st == _lib.FEM_SOLVE_NAN:
        raise FloatingPointError("linear solve produced NaN")
    if cfg.get("line_search_flag", False):
        if inc is None:
            inc = x32.double()
        return _line_search(problem, eng, dofs, inc)
    if inc is None:
        new = dofs.clone()
        eng.axpy32(1.0, x32, new)
        if eng.n_bc:
            new[rows] = eng.bc_vals      # constraints hold exactly in FP64
        return new
    new = dofs + inc
    if prec != _FP64_SOLVER_FORMAT and eng.n_bc:
        new[rows] = eng.bc_vals
    return new


def _line_search(problem, eng, dofs, inc):
    """solver.py:424-463: three step halvings on ||R_bc(u + alpha inc)||."""
    def norm(alpha):
        return torch.linalg.norm(eng.residual(dofs + alpha * inc, apply_bc=True)).item()

    alpha = 1.0
    rn = norm(alpha)
    for i in range(3):
        alpha *= 0.5
        rh = norm(alpha)
        logger.debug("Line search (step halving): i = %d, alpha = %g, res_norm = %g, res_norm_half = %g",
                     i, alpha, rn, rh)
        if rh > rn:
            alpha *= 2.0
            break
        rn = rh
    return dofs + alpha * inc


def solver(problem, solver_options={}):
    """Newton solve (solver.py:1112-1356).  Returns sol_list = [tensor (num_nodes, vec)] (FP64, device)."""
    method, cfg = _resolve_solver_options(solver_options)
    if method == "arc_length":
        from .drivers import solve_arc_length
        sol_list, info = solve_arc_length(problem, cfg)
        return (sol_list, info) if cfg.get("return_info", False) else sol_list
    if method == "dynamic_relax":
        from .drivers import dynamic_relax_solve
        ig = cfg.get("initial_guess")
        if ig is not None:
            ig = _flat_v(ig, problem._engine.device)
        return dynamic_relax_solve(problem, tol=cfg.get("tol", 1e-6), nKMat=cfg.get("nKMat", 1000),
                                   nPrint=cfg.get("nPrint", 500), info=cfg.get("info", True),
                                   info_force=cfg.get("info_force", True), initial_guess=ig,
                                   linear_options=cfg.get("linear", {}), max_iters=cfg.get("max_iters"))
    eng = problem._engine
    spec = resolve_linear(cfg.get("linear", {}))
    precision = _precision(cfg)
    wall0 = time.perf_counter()
    if "initial_guess" in cfg:
        ig = cfg["initial_guess"]
        if isinstance(ig, (list, tuple)):
            ig = ig[0]
        dofs = torch.as_tensor(ig, dtype=torch.float64, device=eng.device).detach().reshape(-1).clone()
    else:
        dofs = torch.zeros(eng.num_dofs, dtype=torch.float64, device=eng.device)
    rel_tol = cfg.get("rel_tol", 1e-8)
    tol = cfg.get("tol", 1e-6)
    max_iter = cfg.get("max_iter", 200)

    t0 = time.perf_counter()
    res = eng.residual(dofs, apply_bc=True)
    res_val = torch.linalg.norm(res).item()
    _timed(eng, "local_assembly", t0)
    res0 = res_val
    rel = res_val / res0 if res0 > 0 else 0.0
    logger.info("  iter 0: nonlinear residual L2 norm = %.3g (relative to initial = %.3g)", res_val, rel)
    n_iters = 0
    while rel > rel_tol and res_val > tol:
        n_iters += 1
        if n_iters > max_iter:
            raise RuntimeError(f"Newton did not converge in {max_iter} iterations (rel res {rel:.3g})")
        dofs = _newton_step(problem, eng, dofs, res, spec, precision, cfg)
        t0 = time.perf_counter()
        res = eng.residual(dofs, apply_bc=True)
        res_val = torch.linalg.norm(res).item()
        _timed(eng, "local_assembly", t0)
        rel = res_val / res0
        logger.info("  iter %d: nonlinear residual L2 norm = %.3g (relative to initial = %.3g)", n_iters, res_val, rel)
    if not np.isfinite(res_val):
        raise FloatingPointError("res_val contains NaN, stop the program!")   # solver.py:1335
    problem._newton_point = dofs
    problem.newton_info = dict(iterations=n_iters, res=res_val, res0=res0, rel=rel,
                               wall=time.perf_counter() - wall0)
    return problem.unflatten_fn_sol_list(dofs)


def _flat_v(v_list, device):
    if isinstance(v_list, (list, tuple)):
        v_list = v_list[0]
    return torch.as_tensor(v_list, dtype=torch.float64, device=device).reshape(-1).contiguous()


def adjoint_solve(problem, dofs, v, adjoint_solver_options=None, precision="fp64", inner_rtol=1e-5,
                  max_refine=30):
    """lam_f = K_ff^-T v_f (the free block of A^T lam = v, solver.py:1399-1409).  Dirichlet
    entries of lam are returned as 0 (lam_b = v_b - K_fb^T lam_f is formed by
    dirichlet_adjoint when a Dirichlet value is differentiated).

    A non-symmetric tangent (GeneralLinear with C != C^T) is transposed on the device
    (fem_matrix_transpose, the reference's A.transpose()) and solved in FP64 whatever the
    precision; symmetric tangents solve K_ff itself.

    precision 'mixed': FP32 Krylov corrections inside FP64 iterative refinement whose
    residual v_f - K_ff lam_f is the matrix-free FP64 tangent action; it stops at the
    linear solver's relative tolerance measured on that FP64 residual."""
    eng = problem._engine
    opts = dict(adjoint_solver_options or {})
    prec_opt = opts.pop("precision", precision)
    inner_rtol = opts.pop("inner_rtol", inner_rtol)
    refine_delta = opts.pop("refine_delta", 0.1)
    spec = resolve_linear(opts)
    eng.refresh_bc()
    b = v.clone()
    if eng.n_bc:
        b[eng.bc_rows_long] = 0.0
    symmetric = eng.tangent_symmetric
    if spec.custom is not None:
        A = eng.tangent(dofs, _lib.FEM_F64, _lib.FEM_BC_SYMMETRIC)
        A = A if symmetric else A.transpose()
        return torch.as_tensor(spec.custom(A, b, None, spec.options), dtype=torch.float64, device=dofs.device)
    t0 = time.perf_counter()
    if not symmetric:
        At = eng.tangent(dofs, _lib.FEM_F64, _lib.FEM_BC_SYMMETRIC).transpose()
        lam = torch.zeros_like(b)
        _, _, st = eng.krylov(spec.method, At, b, lam, spec.pc, spec.rtol, spec.atol, spec.maxiter)
        if st == _lib.FEM_SOLVE_NAN:
            raise FloatingPointError("adjoint solve produced NaN")
        _timed(eng, "linear", t0)
        return lam
    if prec_opt == "fp64":
        A = eng.tangent(dofs, _FP64_SOLVER_FORMAT, _lib.FEM_BC_SYMMETRIC)
        lam = torch.zeros_like(b)
        eng.krylov(spec.method, A, b, lam, spec.pc, spec.rtol, spec.atol, spec.maxiter)
        _timed(eng, "linear", t0)
        return lam
    mprec = _mixed_matrix_precision(prec_opt, eng) if spec.method == "cg" else _lib.FEM_SLICED_F32
    A = eng.tangent(dofs, mprec, _lib.FEM_BC_SYMMETRIC)
    lam = torch.zeros_like(b)
    if spec.method == "cg":
        eng.pcg_refined(A, b, lam, dofs, spec.pc, spec.rtol, spec.atol, refine_delta, spec.maxiter)
        _timed(eng, "linear", t0)
        return lam
    r = b
    bn = torch.linalg.norm(b).item()
    if bn == 0.0:
        return lam
    target = max(spec.rtol * bn, spec.atol)
    for _ in range(max_refine):
        r32 = eng.cast32(r, eng.bc_mask)
        d32 = torch.zeros_like(r32)
        _, _, st = eng.krylov(spec.method, A, r32, d32, spec.pc, inner_rtol, 0.0, spec.maxiter)
        if st == _lib.FEM_SOLVE_NAN:
            raise FloatingPointError("adjoint inner solve produced NaN")
        eng.axpy32(1.0, d32, lam)
        if eng.n_bc:
            lam[eng.bc_rows_long] = 0.0
        r = b - eng.apply(dofs, lam, skip_bc_rows=True)
        if eng.n_bc:
            r[eng.bc_rows_long] = 0.0
        if torch.linalg.norm(r).item() <= target:
            break
    _timed(eng, "linear", t0)
    return lam


def dirichlet_adjoint(problem, dofs, v, lam):
    """lam_b = v_b - K_fb^T lam_f: the Dirichlet rows of A^T lam = v (solver.py:1405-1409) with
    A = [[K_ff, K_fb], [0, I]] (zeroRows).  K^T lam_f is the FP64 tangent action for a symmetric
    tangent and the transposed FP64 CSR tangent otherwise.  Returns lam_b in bc_rows order."""
    eng = problem._engine
    rows = eng.bc_rows_long
    lam_f = lam.clone()
    lam_f[rows] = 0.0
    if eng.tangent_symmetric:
        kt = eng.apply(dofs, lam_f, skip_bc_rows=False)
    else:
        kt = eng.tangent(dofs, _lib.FEM_F64, _lib.FEM_BC_NONE, cache=False).transpose().matvec(lam_f)
    return v[rows] - kt[rows]


def _iv_cotangent(iv, g, eng, what):
    """Reshape a per-point cotangent g to the internal variable iv's shape."""
    if iv.numel() == g.numel():
        return g.reshape(iv.shape)
    if what == "qp" and iv.numel() == eng.num_cells:
        return g.reshape(eng.num_cells, eng.num_quads).sum(1).reshape(iv.shape)
    raise ValueError(f"unexpected shape {tuple(iv.shape)} of a differentiable internal variable ({what})")


def implicit_vjp(problem, sol_list, params, v_list, adjoint_solver_options, precision="fp64"):
    """solver.py:1362-1418: returns -lam^T dc/dp with c = apply_bc(R(u, set_params(p))).

    params is a tensor or a list/tuple of tensors (the reference's params pytree); the result has
    the same structure.  The cotangent reaches params through set_params by torch autograd, from
    every differentiable internal variable of the material (per-point parameters; for J2 also the
    history sigmas_old / epsilons_old, so gradients chain over load steps)."""
    eng = problem._engine
    t0 = time.perf_counter()
    seq = isinstance(params, (list, tuple))
    plist = list(params) if seq else [params]
    with torch.no_grad():
        problem.set_params([p.detach() for p in plist] if seq else params.detach())
        dofs = _flat_v(sol_list, eng.device)
        v = _flat_v(v_list, eng.device)
        lam = adjoint_solve(problem, dofs, v, adjoint_solver_options, precision)
        m = eng._mat
        dv = m.diff_vars()
        cot = {}
        if m.history:
            kinds = {k for _, k in dv}
            hg, sg, _ = eng.j2_history_vjp(dofs, lam=lam, want_scale="qp" in kinds)
            cot["sigma"] = hg[:, :, :9]
            cot["eps"] = hg[:, :, 9:]
            if sg is not None:
                cot["qp"] = sg
        elif dv:
            cot["qp"] = eng.param_vjp(dofs, lam)
    with torch.enable_grad():
        ps = [p.detach().clone().requires_grad_(True) if torch.is_tensor(p) and p.is_floating_point() else p
              for p in plist]
        problem.set_params(ps if seq else ps[0])
        ivs, gos = [], []
        for idx, what in dv:
            iv = problem.internal_vars[idx] if idx < len(problem.internal_vars) else None
            if torch.is_tensor(iv) and iv.requires_grad:
                ivs.append(iv)
                gos.append(_iv_cotangent(iv, cot[what], eng, what).to(iv.dtype))
        if eng.has_universal:
            # the compiled universal kernels' part of -lam^T dR/d(internal vars)
            with torch.no_grad():
                ucot = eng.universal_param_vjp(dofs, lam)
            if ucot is not None:
                for iv, g in zip(problem.internal_vars, ucot):
                    if torch.is_tensor(iv) and iv.requires_grad:
                        ivs.append(iv)
                        gos.append(g.to(iv.dtype).reshape(iv.shape))
        eng.refresh_bc()
        if eng.bc_value_terms:
            # Dirichlet values built from params (set_params -> update_Dirichlet_boundary_conditions):
            # c_b = u_b - g(p), so -lam^T dc/dp gets +lam_b^T dg/dp
            with torch.no_grad():
                lam_b = dirichlet_adjoint(problem, dofs, v, lam)
            for pos, t in eng.bc_value_terms:
                ivs.append(t)
                gos.append(lam_b[pos].to(t.device, t.dtype))
        if not ivs:
            raise RuntimeError("set_params must build internal_vars (or Dirichlet values) from params with torch "
                               "operations so the parameter chain rule can be applied")
        diff_ps = [p for p in ps if torch.is_tensor(p) and p.requires_grad]
        gs = torch.autograd.grad(ivs, diff_ps, grad_outputs=gos, allow_unused=True)
    with torch.no_grad():
        problem.set_params([p.detach() for p in plist] if seq else params.detach())
    eng.timing["adjoint"] += time.perf_counter() - t0
    it = iter(gs)
    out = []
    for p, q in zip(plist, ps):
        if torch.is_tensor(q) and q.requires_grad:
            g = next(it)
            out.append(torch.zeros_like(p) if g is None else g.to(p.dtype))
        else:
            out.append(None)
    return out if seq else out[0]


def ad_wrapper(problem, solver_options={}, adjoint_solver_options={}):
    """solver.py:1421-1455: differentiable fwd_pred(params) -> sol_list (torch.autograd).
    params may be a tensor or a list/tuple of tensors."""
    _, cfg = _resolve_solver_options(solver_options)
    precision = _precision(cfg)

    class _ForwardPrediction(torch.autograd.Function):
        @staticmethod
        def forward(ctx, seq, *params):
            problem.set_params(list(params) if seq else params[0])
            sol_list = solver(problem, solver_options)
            ctx.save_for_backward(*params)
            ctx.seq = seq
            ctx.sol_list = [s.detach() for s in sol_list]
            return tuple(sol_list)

        @staticmethod
        def backward(ctx, *v):
            params = ctx.saved_tensors
            logger.info("Running backward and solving the adjoint problem...")
            p = list(params) if ctx.seq else params[0]
            g = implicit_vjp(problem, ctx.sol_list, p, list(v), adjoint_solver_options, precision)
            return (None,) + (tuple(g) if ctx.seq else (g,))

    def fwd_pred(params):
        if isinstance(params, (list, tuple)):
            return list(_ForwardPrediction.apply(True, *params))
        return list(_ForwardPrediction.apply(False, params))

    return fwd_pred


class _J2HistoryUpdate(torch.autograd.Function):
    @staticmethod
    def forward(ctx, problem, sol, sigmas_old, epsilons_old, scale):
        eng = problem._engine
        saved = problem.internal_vars
        ivs = [sigmas_old.detach(), epsilons_old.detach()] + ([] if scale is None else [scale.detach()])
        problem.internal_vars = ivs
        try:
            dofs = sol.detach().reshape(-1).to(torch.float64).contiguous()
            sig, eps = eng.j2_update(dofs)
        finally:
            problem.internal_vars = saved
        ctx.problem = problem
        ctx.has_scale = scale is not None
        ctx.save_for_backward(sol, sigmas_old, epsilons_old, *( [] if scale is None else [scale]))
        return sig.reshape(sigmas_old.shape), eps.reshape(epsilons_old.shape)

    @staticmethod
    def backward(ctx, g_sig, g_eps):
        problem = ctx.problem
        eng = problem._engine
        sol, sigmas_old, epsilons_old = ctx.saved_tensors[:3]
        scale = ctx.saved_tensors[3] if ctx.has_scale else None
        nc, nq = eng.num_cells, eng.num_quads
        gz = lambda g: torch.zeros(nc, nq, 9, dtype=torch.float64, device=eng.device) if g is None \
            else g.reshape(nc, nq, 9).to(torch.float64)
        hbar = torch.cat([gz(g_sig), gz(g_eps)], dim=2)
        saved = problem.internal_vars
        problem.internal_vars = [sigmas_old.detach(), epsilons_old.detach()] + \
            ([] if scale is None else [scale.detach()])
        try:
            dofs = sol.detach().reshape(-1).to(torch.float64).contiguous()
            hg, sg, ug = eng.j2_history_vjp(dofs, hist_bar=hbar, want_scale=scale is not None, want_u=True)
        finally:
            problem.internal_vars = saved
        g_scale = None
        if scale is not None:
            g_scale = _iv_cotangent(scale, sg, eng, "qp").to(scale.dtype)
        return (None, ug.reshape(sol.shape).to(sol.dtype), hg[:, :, :9].reshape(sigmas_old.shape),
                hg[:, :, 9:].reshape(epsilons_old.shape), g_scale)


def update_j2_history(problem, sol, sigmas_old, epsilons_old, scale=None):
    """Differentiable J2 history update (test_plasticity.py:73-78, the reference's
    update_stress_strain / update_int_vars_gp): returns (sigmas_new, epsilons_new) of shape
    (num_cells, num_quads, 3, 3) for the displacement sol, given the previous history and the
    optional modulus-scale field.  Its backward is fem_j2_history_vjp in update mode, so
    torch.autograd chains gradients across load steps."""
    return _J2HistoryUpdate.apply(problem, sol, sigmas_old, epsilons_old, scale)


# ---- BC helpers of the reference, device versions (solver.py:290-363) ----------------
def get_q_vec(problem):
    """solver.py:637-642: the residual at u = 0 without Dirichlet rows (force-controlled
    arc-length's reference load)."""
    eng = problem._engine
    return eng.residual(torch.zeros(eng.num_dofs, dtype=torch.float64, device=eng.device), apply_bc=False)


def apply_bc_vec(res_vec, dofs, problem, scale=1.0):
    eng = problem._engine
    eng.refresh_bc()
    res = res_vec.clone().contiguous()
    if eng.n_bc:
        res[eng.bc_rows_long] = dofs[eng.bc_rows_long] - eng.bc_vals * scale
    return res


def assign_bc(dofs, problem):
    eng = problem._engine
    eng.refresh_bc()
    out = dofs.clone()
    if eng.n_bc:
        out[eng.bc_rows_long] = eng.bc_vals
    return out


def copy_bc(dofs, problem):
    eng = problem._engine
    eng.refresh_bc()
    out = torch.zeros_like(dofs)
    if eng.n_bc:
        out[eng.bc_rows_long] = dofs[eng.bc_rows_long]
    return out
