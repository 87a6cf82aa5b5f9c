"""Benchmark: one SIMP topology-optimisation iteration (assemble + solve + adjoint gradient).

Workload (metric "assemble+solve+adjoint s/iter at 3M DOF: mixed vs FP64 on GB300 @1e-8"):
HEX8 cantilever 200x100x50 on [0,2]x[0,1]x[0,0.5] (1,000,000 cells, 1,035,351 nodes,
3,106,053 dofs, CSR nnz 245,844,459), clamped at x=0, traction (0,0,1) on x=2 as the
surface map, SIMP E = 1e-3 + (1 - 1e-3) theta^3, nu = 0.3, theta = 0.5 + U(-0.05, 0.05)
(torch.Generator seed 0).  One step = fwd_pred(theta) through ad_wrapper (Newton with PCG
to relative residual 1e-8), compliance J = f.u, J.backward() (adjoint solve + parameter VJP).

value   : mixed precision (FP64 assembly; block-Jacobi PCG on the DF48 copy of the tangent with
          double-float vectors on the FP32 pipes and FP64 reliable updates), s/iter, inputs
          resident in HBM, CUDA events over exactly K steps.
fp64    : the same iteration in plain FP64 (FP64 tangent, FP64 PCG), reported beside it.
e2e     : the mixed iteration through the public API from pinned host theta to host J and
          gradient, copies inside the timed region.
roofline: the DF48 SpMV (the dominant kernel): algorithmic bytes over its mean duration inside the
          timed steps (CUDA events on the solver's stream around sampled launches).
--impl reference: the FP64 CPU restatement (oracle) of the same iteration on the host cores.
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
# The CPU port runs its SpMV on a thread pool of its own; BLAS level-1 calls between the SpMVs
# run single-threaded, or idle BLAS worker threads spin against that pool (measured: 2.5x slower
# PCG iterations).  Set before numpy loads its BLAS.
os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")

import numpy as np  # noqa: E402

METRIC = "assemble+solve+adjoint s/iter at 3M DOF: mixed vs FP64 on GB300 @1e-8; HBM GB/s"
UNIT = "s/iter"
DEFAULT_SIZE = (200, 100, 50)
L = (2.0, 1.0, 0.5)
RTOL = 1e-8
# FP64 block-Jacobi PCG iterations (forward, adjoint) that the full 200x100x50 workload needs to
# reach RTOL; measured by this bench on a GB300 (printed as fp64.pcg_iterations) and used only to
# scale the bounded CPU-baseline sample to a full iteration.
FULL_SIZE_PCG_ITERS = (2649, 2622)


def workload_name(n, extent=None):
    nx, ny, nz = n
    cells = nx * ny * nz
    nodes = (nx + 1) * (ny + 1) * (nz + 1)
    nnz = 9 * (3 * nx + 1) * (3 * ny + 1) * (3 * nz + 1)
    ext = tuple(extent or L)
    dom = "" if ext == L else f" on [0,{ext[0]:g}]x[0,{ext[1]:g}]x[0,{ext[2]:g}]"
    return (f"SIMP compliance TO iteration, HEX8 cantilever {nx}x{ny}x{nz}{dom} ({cells:,} cells, "
            f"{3 * nodes:,} dofs, CSR nnz {nnz:,})"), cells, nodes, nnz


def theta_init(ncells, seed=0):
    import torch
    g = torch.Generator().manual_seed(seed)
    return (0.5 + (torch.rand(ncells, 1, generator=g, dtype=torch.float64) - 0.5) * 0.1)


def theta_step(theta0, k):
    """Design for step k: a distinct theta every step (as in an optimisation loop), so the
    tangent is re-assembled inside every timed step."""
    return theta0 * (1.0 + 1e-4 * (k + 1))


def make_problem(n, extent=None):
    import jax_fem_gb300 as jf
    Lx, Ly, Lz = extent or L
    m = jf.box_mesh(*n, Lx, Ly, Lz)
    mesh = jf.Mesh(m.points, m.cells_dict["hexahedron"])
    left = lambda p: np.isclose(p[0], 0.0, atol=1e-5)
    right = lambda p: np.isclose(p[0], Lx, atol=1e-5)
    zero = lambda p: 0.0

    class Cantilever(jf.Problem):
        def get_tensor_map(self):
            return jf.SIMPElastic(1.0, 1e-3, 0.3, 3.0)

        def get_surface_maps(self):
            return [lambda u, x: np.array([0.0, 0.0, 1.0])]

        def set_params(self, params):
            self.internal_vars = [params[:, None, :].expand(-1, 8, -1)]

    return Cantilever(mesh, vec=3, dim=3, dirichlet_bc_info=[[left] * 3, [0, 1, 2], [zero] * 3],
                      location_fns=[right])


def options(precision):
    """Same solver settings for both precisions: block-Jacobi PCG to half the Newton tolerance
    (so one Newton step meets rel_tol on the FP64 residual), adjoint to RTOL."""
    fwd = {"petsc_solver": {"ksp_type": "cg", "pc_type": "bjacobi", "rtol": 0.5 * RTOL},
           "rel_tol": RTOL, "tol": 0.0, "precision": precision}
    adj = {"petsc_solver": {"ksp_type": "cg", "pc_type": "bjacobi", "rtol": RTOL}, "precision": precision}
    return fwd, adj


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    def __init__(self, index=0):
        self.index = index
        self.samples = []
        self.proc = None

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) == 7:
                self.samples.append(parts)

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = [nm for k, nm in enumerate(names) if any(s[3 + k].lower().startswith("active") for s in self.samples)]
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def run_steps(prob, fwd, theta, J_out=None):
    """One TO iteration through the public API: fwd_pred, compliance, backward."""
    import torch
    th = theta.detach().requires_grad_(True)
    sol = fwd(th)[0]
    J = torch.dot(prob._engine.f_ext, sol.reshape(-1))
    J.backward()
    return J.detach(), th.grad, sol.detach()


def spmv_roofline(prob, peak):
    """Time each cached SpMV format with CUDA events on the launching stream (direct C-ABI calls,
    input vector prepared once).  DF48 is timed through fem_spmv_dfx, the kernel the mixed CG
    runs (node-interleaved double-float x, double-float y, fused dot).  Algorithmic bytes per
    launch: values (6 B/nnz DF48, 8 B FP64, 4 B FP32) + one 4-byte block column per vec*vec
    values + slice or row pointers + x read + y write (no block columns for the DF48 copy in the
    grid layout of a box-numbered mesh)."""
    import ctypes as C
    import torch
    import jax_fem_gb300 as jf
    from jax_fem_gb300._lib import call, ptr, stream_handle
    eng = prob._engine
    out = {}
    n, nnz, nnzb = eng.num_dofs, eng.nnz, eng.nnzb
    L_ = jf._lib
    fmts = ((L_.FEM_SSYM_DF48, "ssym_df48", 6, 8, 16), (L_.FEM_SYM_DF48, "sym_df48", 6, 8, 16),
            (L_.FEM_SLICED_DF48, "df48", 6, 8, 8),
            (L_.FEM_SLICED_F32, "fp32", 4, 4, 4), (L_.FEM_SLICED_F64, "fp64", 8, 8, 8))
    for prec, name, es, xs, ys in fmts:
        A = eng._tangent_cache.get((prec, jf._lib.FEM_BC_SYMMETRIC))
        if A is None:
            continue
        if prec in (L_.FEM_SLICED_DF48, L_.FEM_SYM_DF48, L_.FEM_SSYM_DF48):
            pad = 4 if eng.vec == 3 else 1
            x = torch.zeros(eng.num_nodes, pad, 2, dtype=torch.float32, device="cuda")
            x[:, :eng.vec, 0] = torch.randn(eng.num_nodes, eng.vec, device="cuda")
            yh = torch.empty(n, dtype=torch.float32, device="cuda")
            yl = torch.empty_like(yh)
            nb = C.c_size_t()
            call("fem_krylov_workspace", n, prec, C.byref(nb))
            ws = torch.empty(nb.value, dtype=torch.uint8, device="cuda")

            def launch():
                call("fem_spmv_dfx", C.byref(eng.pattern), eng.num_nodes, eng.vec, prec, ptr(A.data), ptr(x),
                     ptr(yh), ptr(yl), None, ptr(ws), nb.value, stream_handle())
        else:
            x = torch.randn(n, dtype=A.vector_dtype, device="cuda")
            y = torch.empty_like(x)

            def launch():
                call("fem_spmv", C.byref(eng.pattern), eng.num_nodes, eng.vec, prec, ptr(A.data), ptr(x), ptr(y),
                     stream_handle())
        s = torch.cuda.current_stream()
        for _ in range(3):
            launch()
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        reps = 20
        torch.cuda.synchronize()
        ev[0].record(s)
        for _ in range(reps):
            launch()
        ev[1].record(s)
        torch.cuda.synchronize()
        t = ev[0].elapsed_time(ev[1]) / 1e3 / reps
        if prec == L_.FEM_SSYM_DF48:
            # the 14 stored stencil blocks of every grid row (zero blocks at the boundary included,
            # implicit columns); x read, y (double-float) and the FP64 transposed part written once
            gx, gy, gz = eng.grid
            rows_stored = ((gx * gy + 31) // 32) * 32 * gz
            algo = rows_stored * 14 * 9 * es + n * xs + n * ys
        elif prec == L_.FEM_SYM_DF48:
            # the upper node blocks only; y is the double-float direct part plus the FP64
            # transposed part (atomics), both written once per dof
            nb_u = (nnzb - eng.num_nodes) // 2 + eng.num_nodes
            algo = nb_u * eng.vec ** 2 * es + nb_u * 4 + (eng.n_slices + 1) * 8 + n * xs + n * ys
        elif prec == L_.FEM_SLICED_DF48 and eng.slices_grid:
            # grid layout (box numbering): the block columns follow from the node grid, none is read
            algo = nnz * es + (eng.n_slices + 1) * 8 + n * xs + n * ys
        else:
            algo = nnz * es + nnzb * 4 + (eng.num_nodes + 1) * 8 + n * xs + n * ys
        out[name] = {"seconds": t, "algorithmic_bytes": algo, "achieved_gbs": algo / t / 1e9,
                     "frac": algo / t / 1e9 / peak}
    return out


def assembly_roofline(prob, peak):
    """Time the assembly launches with CUDA events on the launching stream (direct C-ABI calls,
    5 launches each after 2 warm-ups, output zeroed outside the bracket): the double-float matrix
    (fem_assemble FEM_OUT_MATRIX with FEM_DF48, the mixed path's), the FP64 matrix (the FP64
    path's) and the FP64 residual, each with the cached geometry.  Algorithmic bytes per launch:
    per cell its connectivity (4 B per node), slot table (1 B per node pair), cached shape
    gradients and JxW (8 B x nq x (3 nn + 1)) and qp parameter (8 B x nq); the matrix launches
    read and write every CSR value once (16 B per nonzero) and read the row pointers; the
    residual launch reads u and reads and writes the residual (8 B x 3 per dof)."""
    import ctypes as C
    import torch
    import jax_fem_gb300 as jf
    from jax_fem_gb300._lib import call, ptr, stream_handle
    eng = prob._engine
    L_ = jf._lib
    if eng.shape_grads is None:
        return None
    eng.refresh_bc()
    _, ms = eng.material()
    cells, nq, nn, nd = eng.num_cells, eng.num_quads, eng.nn, eng.num_dofs
    per_cell = 4 * nn + nn * nn + 8 * nq * (3 * nn + 1) + 8 * nq
    u = torch.zeros(nd, dtype=torch.float64, device="cuda")
    vals = torch.zeros(eng.nnz, dtype=torch.float64, device="cuda")
    res = torch.zeros(nd, dtype=torch.float64, device="cuda")
    s = torch.cuda.current_stream()
    out = {}
    # flops per cell of the isotropic node-pair tangent: per node pair a <= b and quadrature point
    # m = mu g_a (3 mul) and M += m (x) g_b (9 FMA); per pair K_ab = cr M + M^T + tr(M) I (9 FMA +
    # 9 add + trace); the residual: grad u (nn*3*3 FMA), the stress (~30), the row sums (nn*3*3 FMA)
    n_pairs = nn * (nn + 1) // 2
    mat_flops = cells * (n_pairs * nq * (3 + 18) + n_pairs * (27 + 2))
    res_flops = cells * nq * (2 * nn * 9 + 30 + 2 * nn * 9)
    cases = (("matrix_df48", L_.FEM_OUT_MATRIX, L_.FEM_DF48, cells * per_cell + 16 * eng.nnz + 8 * (nd + 1) + nd,
              mat_flops),
             ("matrix_fp64", L_.FEM_OUT_MATRIX, L_.FEM_F64, cells * per_cell + 16 * eng.nnz + 8 * (nd + 1) + nd,
              mat_flops),
             ("residual_fp64", L_.FEM_OUT_RESIDUAL, L_.FEM_F64, cells * per_cell + 24 * nd + nd, res_flops))
    for name, outputs, prec, algo, flops in cases:
        def launch():
            call("fem_assemble", C.byref(eng.mesh), C.byref(ms), C.byref(eng.pattern), outputs, prec, ptr(u), None,
                 ptr(eng.bc_mask), L_.FEM_BC_SYMMETRIC, ptr(res), ptr(vals), None, stream_handle())
        ts = []
        for k in range(7):
            vals.zero_()
            res.zero_()
            ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
            ev[0].record(s)
            launch()
            ev[1].record(s)
            torch.cuda.synchronize()
            if k >= 2:
                ts.append(ev[0].elapsed_time(ev[1]) / 1e3)
        t = float(np.median(ts))
        out[name] = {"seconds": t, "algorithmic_bytes": int(algo), "achieved_gbs": algo / t / 1e9,
                     "frac": algo / t / 1e9 / peak, "flops": int(flops), "tflops": flops / t / 1e12}
    return out


def measured_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


TRAFFIC_PROFILES = {
    "df48": os.path.join(ROOT, "profiles", "spmv_sliced_dfdf_bulk_grid_hex8_160x80x40.txt"),
    "sym_df48": os.path.join(ROOT, "profiles", "spmv_sym_df48_bulk_hex8_100x50x25.txt"),
}


def traffic_from_profile(n_units, kind="df48"):
    """DRAM bytes (read + write) per DF48 SpMV launch: the committed ncu summary's bytes per
    nonzero (of the full matrix) on a smaller case, scaled to this workload's nnz (traffic grows
    with nnz)."""
    if kind not in TRAFFIC_PROFILES:
        return None
    try:
        with open(TRAFFIC_PROFILES[kind]) as f:
            for line in f:
                if line.startswith("dram_bytes_per_nnz:"):
                    return float(line.split(":", 1)[1]) * n_units
    except (OSError, ValueError):
        pass
    return None


class CpuPort:
    """The oracle port of one SIMP TO iteration (oracle/simp_fast.py: FP64 numpy/scipy) built at the
    workload's own size on the host: element stiffnesses, the COO -> CSR slot map of the PETSc
    pattern, the end-face load.  Each cost is then timed on the full-size objects: one assembly
    (E(theta) K0_e summed into the CSR slots, Dirichlet elimination, block-Jacobi set-up), block-
    Jacobi PCG iterations (SpMV on row blocks in a thread pool over the host cores, vector work
    numpy), the residual SpMV and the parameter VJP."""

    def __init__(self, n, threads):
        from oracle import fem as ofem, simp_fast
        t0 = time.perf_counter()
        pts, cells = ofem.box_mesh(*n, *L)
        left = np.isclose(pts[:, 0], 0.0, atol=1e-5)
        right = np.isclose(pts[:, 0], L[0], atol=1e-5)
        bc_rows = (3 * np.argwhere(left).reshape(-1)[:, None] + np.arange(3)[None, :]).reshape(-1)
        f = simp_fast.traction_load(pts, cells, right, [0.0, 0.0, 1.0])
        self.sc = simp_fast.SimpCantilever(pts, cells, bc_rows, f)
        _ = self.sc.csr_map
        self.simp_fast = simp_fast
        self.theta = theta_init(len(cells)).numpy()
        self.threads = threads
        self.cells = len(cells)
        self.setup_s = time.perf_counter() - t0
        self.A = self.At = self.P = None

    def assemble(self):
        t0 = time.perf_counter()
        self.A = self.sc.assemble_csr(self.theta)
        self.P = self.sc.csr_map.block_jacobi(self.A)
        t = time.perf_counter() - t0
        self.At = self.simp_fast.ThreadedCSR(self.A, self.threads)
        return t

    def spmv(self, reps=3):
        x = np.random.default_rng(0).standard_normal(self.sc.N)
        t0 = time.perf_counter()
        for _ in range(reps):
            self.At @ x
        return (time.perf_counter() - t0) / reps

    def pcg_iteration(self, iters):
        t0 = time.perf_counter()
        self.sc.pcg(self.At, self.sc.f, 1e-30, iters=iters, precond=self.P)
        return (time.perf_counter() - t0) / iters

    def solve(self, rtol):
        t0 = time.perf_counter()
        u, it = self.sc.pcg(self.At, self.sc.f, rtol, precond=self.P)
        return u, it, time.perf_counter() - t0

    def vjp(self, u):
        t0 = time.perf_counter()
        th = self.theta.reshape(-1)
        dE = 3.0 * (1 - 1e-3) * th ** 2
        ue = u[self.sc.dofs]
        g = -dE * np.einsum("ci,cij,cj->c", ue, self.sc.K0, ue)
        return g, time.perf_counter() - t0


def _blas_threads():
    try:
        from threadpoolctl import threadpool_info
        return max((i.get("num_threads", 1) for i in threadpool_info() if i.get("user_api") == "blas"), default=1)
    except Exception:  # noqa: BLE001
        return 1


# systems up to this many dofs are solved to the tolerance on the host (nothing projected);
# larger ones time PCG iterations at full size and take the iteration counts of the GPU's FP64 run
CPU_SOLVE_DOFS = 400_000


def cpu_baseline(n, iters_full, pcg_sample=10, port=None):
    """One TO iteration of the oracle port on the host cores, every unit cost timed at the
    workload's full size.  Small workloads run to the tolerance (value_kind 'measured'); at full
    size the forward and adjoint block-Jacobi PCG iteration counts are those of the GPU's FP64
    block-Jacobi run (value_kind 'projected': assembly, residual SpMVs and VJP measured once each,
    PCG iterations timed in a sample of `pcg_sample`)."""
    threads = len(os.sched_getaffinity(0))
    port = port or CpuPort(n, threads)
    t_asm = port.assemble()
    t_spmv = port.spmv()
    name, cells, nodes, nnz = workload_name(n)
    if port.sc.N <= CPU_SOLVE_DOFS:
        u, it_f, t_f = port.solve(RTOL)
        _, it_a, t_a = port.solve(RTOL)          # adjoint: A^T lam = dJ/du = f (compliance)
        _, t_vjp = port.vjp(u)
        value = t_asm + 2 * t_spmv + t_f + t_a + t_vjp
        kind = "measured"
        proj = {"assembly_s": t_asm, "residual_spmv_s": t_spmv, "forward_s": t_f, "adjoint_s": t_a, "vjp_s": t_vjp,
                "pcg_iterations": [it_f, it_a], "setup_s": port.setup_s}
        how = (f"forward + adjoint block-Jacobi PCG to {RTOL:g} on the host ({it_f} + {it_a} iterations, "
               f"{t_f + t_a:.2f} s)")
    else:
        t_it = port.pcg_iteration(pcg_sample)
        # the VJP's cost does not depend on the values of u: time it on a seeded field
        _, t_vjp = port.vjp(np.random.default_rng(0).standard_normal(port.sc.N))
        value = t_asm + 2 * t_spmv + t_it * (iters_full[0] + iters_full[1]) + t_vjp
        kind = "projected"
        proj = {"assembly_s": t_asm, "residual_spmv_s": t_spmv, "pcg_iteration_s": t_it, "vjp_s": t_vjp,
                "pcg_iterations": list(iters_full), "pcg_iterations_source": "GPU FP64 block-Jacobi run",
                "setup_s": port.setup_s}
        how = (f"{pcg_sample} block-Jacobi PCG iterations timed at full size ({t_it * 1e3:.1f} ms each) x "
               f"{iters_full[0]}+{iters_full[1]} iterations (forward+adjoint, counts of the GPU FP64 run)")
    sample = (f"oracle (numpy/scipy FP64) at the full {n[0]}x{n[1]}x{n[2]} size ({cells} cells, {port.sc.N} dofs, "
              f"nnz {port.sc.csr_map.nnz}): assembly {t_asm:.2f} s (E K0_e summed into the PETSc-pattern CSR "
              f"slots, Dirichlet elimination, block-Jacobi set-up; numpy, one thread), residual SpMV "
              f"{t_spmv * 1e3:.1f} ms x 2, {how}, VJP {t_vjp:.2f} s; SpMV is scipy's CSR kernel on "
              f"{threads} row blocks in a thread pool, vector work BLAS level 1 in place on "
              f"{_blas_threads()} BLAS thread(s)")
    out = {"value": value, "unit": UNIT, "cores": int(threads), "kind": "port", "value_kind": kind, "sample": sample,
           "host_cores": len(os.sched_getaffinity(0)), "components": proj}
    return out, port


def bench_reference(args):
    """The reference arm: the oracle port of the same iteration on all host cores.  Set-up and
    the once-per-iteration costs (assembly, residual SpMVs, VJP) are measured once at full size;
    each step times a sample of block-Jacobi PCG iterations at full size (or, for small
    workloads, a complete forward + adjoint solve), and the line's value is the iteration
    assembled from those measured unit costs."""
    n = tuple(args.size)
    name, cells, nodes, nnz = workload_name(n)
    iters = FULL_SIZE_PCG_ITERS if n == DEFAULT_SIZE else _default_iters(n)
    threads = len(os.sched_getaffinity(0))
    port = CpuPort(n, threads)
    first, port = cpu_baseline(n, iters, port=port)
    small = port.sc.N <= CPU_SOLVE_DOFS
    samples = []
    for _ in range(args.warmup):
        if small:
            port.solve(RTOL)
        else:
            port.pcg_iteration(10)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        if small:
            _, _, tf = port.solve(RTOL)
            samples.append(tf)
        else:
            samples.append(port.pcg_iteration(10))
    wall = time.perf_counter() - t0
    comp = first["components"]
    if small:
        # both solves are the same system and right-hand side (compliance is self-adjoint)
        t_solve = statistics.median(samples) if samples else 0.5 * (comp["forward_s"] + comp["adjoint_s"])
        v = comp["assembly_s"] + 2 * comp["residual_spmv_s"] + 2 * t_solve + comp["vjp_s"]
    else:
        t_it = statistics.median(samples) if samples else comp["pcg_iteration_s"]
        comp["pcg_iteration_s"] = t_it
        v = comp["assembly_s"] + 2 * comp["residual_spmv_s"] + t_it * sum(iters) + comp["vjp_s"]
    cb = dict(first, value=v)
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": wall / max(args.steps, 1) * 1e3, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "value_kind": first["value_kind"],
            "config": {"workload": name, "precision": "fp64", "tolerance": RTOL,
                       "solver": "block-Jacobi PCG (scipy CSR SpMV on all host cores)",
                       "step": ("one forward block-Jacobi PCG solve to the tolerance at full size" if small else
                                "10 block-Jacobi PCG iterations at full size (ms_per_step is this sample's wall "
                                "time; value is the whole iteration from the measured unit costs)")},
            "impl": "reference", "cpu_baseline": cb,
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def max_over_ranks(t, dist=None, device="cuda"):
    """The slowest rank's time (replicas: every rank runs its own copy of the workload)."""
    if dist is None:
        return t
    import torch
    tt = torch.tensor([t], dtype=torch.float64, device=device)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    return float(tt.item())


def job_seconds_per_iter(t_max, steps, world):
    """Whole-job s/iter with `world` replicas each running `steps` iterations in t_max seconds."""
    return t_max / (steps * world)


def kernel_shares(args):
    """Per-kernel device time of one warm TO step in each precision, from a CUPTI activity trace
    (torch.profiler): launches, total, share and time per launch.  A profile, not a bench line."""
    import collections
    import torch
    import jax_fem_gb300 as jf
    from torch.profiler import profile, ProfilerActivity
    n = tuple(args.size)
    prob = make_problem(n)
    th0 = theta_init(prob.num_cells).cuda()
    with profile(activities=[ProfilerActivity.CUDA]):
        torch.ones(8, device="cuda").sum().item()     # CUPTI start-up outside the traced step
    for prec in (args.precision, "fp64"):
        fwd_o, adj_o = options(prec)
        fwd = jf.ad_wrapper(prob, fwd_o, adj_o)
        run_steps(prob, fwd, theta_step(th0, 0))
        torch.cuda.synchronize()
        with profile(activities=[ProfilerActivity.CUDA]) as p:
            run_steps(prob, fwd, theta_step(th0, 1))
            torch.cuda.synchronize()
        tot, cnt = collections.defaultdict(float), collections.Counter()
        spans = []
        for e in p.events():
            if e.device_type == torch.autograd.DeviceType.CUDA:
                k = e.name.split("(")[0]
                tot[k] += getattr(e, "device_time_total", 0.0) or e.cuda_time_total
                cnt[k] += 1
                tr = getattr(e, "time_range", None)
                if tr is not None and tr.end > tr.start:
                    spans.append((tr.start, tr.end))
        T = sum(tot.values())
        print(f"{prec} step, {workload_name(n)[0]}: {T / 1e3:.1f} ms of kernel time, {sum(cnt.values())} launches")
        print(f"{'launches':>9} {'total_ms':>10} {'share':>7} {'us/launch':>10}  kernel")
        for k, v in sorted(tot.items(), key=lambda kv: -kv[1])[:16]:
            print(f"{cnt[k]:9d} {v / 1e3:10.2f} {100 * v / T:6.2f}% {v / cnt[k]:10.2f}  {k}")
        if len(spans) > 1:   # device idle between consecutive device activities, by gap size
            spans.sort()
            gaps, end = [], spans[0][1]
            for a, b in spans[1:]:
                if a > end:
                    gaps.append(a - end)
                end = max(end, b)
            g = np.asarray(gaps) if gaps else np.zeros(1)
            print(f"device span {(end - spans[0][0]) / 1e3:.1f} ms, idle {g.sum() / 1e3:.1f} ms in {len(gaps)} gaps: "
                  + ", ".join(f"{(g[(g >= lo) & (g < hi)]).sum() / 1e3:.1f} ms in {int(((g >= lo) & (g < hi)).sum())} "
                              f"gaps of {lo:g}-{hi:g} us"
                              for lo, hi in ((0, 5), (5, 20), (20, 100), (100, 1e3), (1e3, 1e9))))


def _neo_box(n, traction=None, stretch=None):
    """Neo-Hookean (E=10, nu=0.3) unit cube, x=0 clamped; an end traction on x=1 or a stretch
    u_x = stretch there.  Returns (GPU problem, oracle problem builder)."""
    import torch
    import jax_fem_gb300 as jf
    m = jf.box_mesh(n, n, n, 1.0, 1.0, 1.0)
    pts, cells = m.points, m.cells_dict["hexahedron"]
    left = lambda p: np.isclose(p[0], 0.0, atol=1e-5)
    right = lambda p: np.isclose(p[0], 1.0, atol=1e-5)
    zero = lambda p: 0.0
    if stretch is not None:
        bc = [[left] * 3 + [right] * 3, [0, 1, 2, 0, 1, 2], [zero] * 3 + [lambda p: stretch, zero, zero]]
    else:
        bc = [[left] * 3, [0, 1, 2], [zero] * 3]
    locs = [right] if traction is not None else None

    class P(jf.Problem):
        def get_tensor_map(self):
            return jf.NeoHookean(10.0, 0.3)

        if traction is not None:
            def get_surface_maps(self):
                return [lambda u, x: np.array(traction)]

    def oracle():
        from oracle import fem as ofem, materials as omat
        return ofem.OracleProblem(pts, cells, 3, dirichlet_bc_info=bc, location_fns=locs,
                                  tensor_map=omat.neo_hookean(10.0, 0.3),
                                  surface_maps=None if traction is None else
                                  [lambda u, x: torch.tensor(traction, dtype=torch.float64)])
    return P(jf.Mesh(pts, cells), vec=3, dim=3, dirichlet_bc_info=bc, location_fns=locs), oracle


def widened_bench(args):
    """The nonlinear drivers and Robin maps beside the step: each solve timed end to end on the
    GPU (CUDA-synchronised wall clock) and as the oracle port on the host, on the same small
    case.  Prints one JSON line; not the headline metric."""
    import torch
    import jax_fem_gb300 as jf

    def timed(fn):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out = fn()
        torch.cuda.synchronize()
        return time.perf_counter() - t0, out

    rows = {}
    # dynamic relaxation (solver.py:918-1049)
    prob, oracle = _neo_box(10, traction=[0.0, 0.0, -0.2])
    opts = {"dynamic_relax": {"tol": 1e-6, "nKMat": 50, "info": False, "info_force": False}}
    jf.solver(prob, opts)
    t_gpu, _ = timed(lambda: jf.solver(prob, opts))
    rec = {"case": "Neo-Hookean HEX8 10^3, end traction, tol 1e-6", "gpu_s": t_gpu,
           "iterations": prob.dr_info["iterations"]}
    if not args.no_cpu:
        from oracle import drivers as odr
        op = oracle()
        t0 = time.perf_counter()
        _, it_o = odr.dynamic_relax(op, tol=1e-6, nKMat=50)
        rec.update(cpu_s=time.perf_counter() - t0, cpu_iterations=it_o)
    rows["dynamic_relax"] = rec
    # arc length, displacement control (solver.py:559-634, 759-793)
    prob, oracle = _neo_box(6, stretch=0.3)
    opts = {"arc_length": {"control": "displacement", "Delta_l": 0.1, "return_info": True,
                           "newton": {"rel_tol": 1e-10, "tol": 1e-10},
                           "linear": {"petsc_solver": {"ksp_type": "cg", "pc_type": "bjacobi", "rtol": 1e-12}}}}
    jf.solver(prob, opts)
    t_gpu, (_, info) = timed(lambda: jf.solver(prob, opts))
    rec = {"case": "Neo-Hookean HEX8 6^3, x=1 stretch 0.3, Delta_l 0.1", "gpu_s": t_gpu,
           "steps": len(info["history"])}
    if not args.no_cpu:
        from oracle import drivers as odr
        op = oracle()
        t0 = time.perf_counter()
        _, _, lams = odr.arc_length(op, "displacement", delta_l=0.1, psi=1.0)
        rec.update(cpu_s=time.perf_counter() - t0, cpu_steps=len(lams))
    rows["arc_length"] = rec
    # u-dependent (Robin) surface map, Newton (problem.py:238-259)
    m = jf.box_mesh(20, 20, 20, 1.0, 1.0, 1.0)
    pts, cells = m.points, m.cells_dict["hexahedron"]
    left = lambda p: np.isclose(p[0], 0.0, atol=1e-5)
    right = lambda p: np.isclose(p[0], 1.0, atol=1e-5)

    class R(jf.Problem):
        def get_tensor_map(self):
            return jf.Laplace()

        def get_surface_maps(self):
            return [lambda u, x: 5.0 * u ** 2]

    prob = R(jf.Mesh(pts, cells), vec=1, dim=3, dirichlet_bc_info=[[left], [0], [lambda p: 1.0]],
             location_fns=[right])
    opts = {"petsc_solver": {"ksp_type": "cg", "pc_type": "jacobi", "rtol": 1e-12}, "rel_tol": 1e-10, "tol": 0.0}
    jf.solver(prob, opts)
    t_gpu, _ = timed(lambda: jf.solver(prob, opts))
    rec = {"case": "Laplace HEX8 20^3, u=1 at x=0, Robin 5u^2 on x=1, Newton rel 1e-10", "gpu_s": t_gpu,
           "newton_iterations": prob.newton_info["iterations"]}
    if not args.no_cpu:
        import torch as _t
        from oracle import fem as ofem, materials as omat, solve as osolve
        op = ofem.OracleProblem(pts, cells, 1, dirichlet_bc_info=[[left], [0], [lambda p: 1.0]],
                                location_fns=[right], tensor_map=omat.laplace(),
                                surface_maps=[lambda u, x: 5.0 * u ** 2])
        t0 = time.perf_counter()
        osolve.newton_solve(op, {"spsolve_solver": {}, "rel_tol": 1e-10, "tol": 0.0})
        rec["cpu_s"] = time.perf_counter() - t0
    rows["robin_newton"] = rec
    line = {"metric": "nonlinear drivers and Robin maps, solve wall time (s)", "unit": "s",
            "higher_is_better": False, "data": "synthetic", "rows": rows,
            "cpu_kind": "port (oracle restatement on the host: torch.func element kernels, scipy direct solves)"}
    print(json.dumps(line))


def mma_update_bench(args):
    """TO update beside the step (jax_fem/mma.py): sensitivity filter + one MMA update for every
    cell of the workload as design variable (m = 1 volume constraint), GPU against the oracle's
    numpy/scipy restatement on the host.  Prints one JSON line; not the headline metric."""
    import torch
    import jax_fem_gb300 as jf
    import importlib
    M = importlib.import_module("jax_fem_gb300.mma")
    n = tuple(args.size)
    name, cells, _, _ = workload_name(n)
    prob = make_problem(n)
    fe = prob.fes[0]
    dev = torch.device("cuda")
    t0 = time.perf_counter()
    H, Hs = M.compute_filter_kd_tree(fe)
    torch.cuda.synchronize()
    t_build = time.perf_counter() - t0
    g = torch.Generator().manual_seed(1)
    rho = (0.5 + 0.1 * (torch.rand(cells, 1, generator=g, dtype=torch.float64) - 0.5)).to(dev)
    dJ = (-torch.rand(cells, 1, generator=g, dtype=torch.float64)).to(dev)
    dvc = torch.full((1, cells, 1), 1.0 / (cells * 0.5), dtype=torch.float64, device=dev)
    vc = np.array([rho.mean().item() / 0.5 - 1.0])
    ft = {"H": H, "Hs": Hs}
    mm = M.MMA()
    mm.setNumConstraints(1)
    mm.setNumDesignVariables(cells)
    mm.setMinandMaxBoundsForDesignVariables(torch.zeros(cells, 1, dtype=torch.float64, device=dev),
                                            torch.ones(cells, 1, dtype=torch.float64, device=dev))
    mm.setScalingParams(1.0, np.zeros(1), 1e4 * np.ones(1), np.zeros(1))
    mm.setMoveLimit(0.1)

    def one():
        dJf, dvcf = M.applySensitivityFilter(ft, rho, dJ, dvc)
        mm.epoch = 1
        mm.xold1, mm.xold2 = rho, rho
        mm.setLowerAndUpperAsymptotes(torch.ones_like(rho), torch.ones_like(rho))
        mm.setObjectiveWithGradient(0.0, dJf.reshape(-1, 1))
        mm.setConstraintWithGradient(vc, dvcf.reshape(1, -1))
        mm.mmasub(rho)
    for _ in range(max(args.warmup, 1)):
        one()
    torch.cuda.synchronize()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    launches0 = jf._lib.load().fem_kernel_launches()
    ev[0].record()
    for _ in range(args.steps):
        one()
    ev[1].record()
    torch.cuda.synchronize()
    t_gpu = ev[0].elapsed_time(ev[1]) / 1e3 / args.steps
    launches = (jf._lib.load().fem_kernel_launches() - launches0) // max(args.steps, 1)
    xg = mm.xmma.cpu().numpy().reshape(-1)
    cpu = None
    if not args.no_cpu:
        from oracle import mma as omma
        t0 = time.perf_counter()     # centroids, volume and neighbour search, as the GPU build
        cent = np.mean(fe.points[fe.cells], axis=1)
        Ho, Hso, _ = omma.filter_kd_tree(cent, omma.cell_volume(fe.points, fe.cells, fe.shape_grads_ref,
                                                                fe.quad_weights))
        t_cpu_build = time.perf_counter() - t0
        r, d0, dv = rho.cpu().numpy().reshape(-1), dJ.cpu().numpy().reshape(-1), dvc.cpu().numpy().reshape(1, -1)
        t0 = time.perf_counter()
        dJf, dvcf = omma.sensitivity_filter(Ho, Hso, r, d0, dv)
        xr, _, _ = omma.mmasub(1, r, r, r, np.ones(cells), np.ones(cells), np.zeros(cells), np.ones(cells), 0.1,
                               0.0, dJf, vc, dvcf, 1.0, np.zeros(1), 1e4 * np.ones(1), np.zeros(1))
        t_cpu = time.perf_counter() - t0
        cpu = {"value": t_cpu, "unit": "s/update", "cores": 1, "kind": "port",
               "sample": f"oracle numpy/scipy filter product + mmasub on the same {cells} variables (full size); "
                         f"k-d tree filter build {t_cpu_build:.1f} s (GPU build {t_build:.2f} s)",
               "max_abs_diff_vs_gpu": float(np.abs(xr - xg).max())}
    line = {"metric": "TO update (sensitivity filter + MMA) s/update", "value": t_gpu, "unit": "s/update",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "higher_is_better": False,
            "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"{cells} design cells of {name}, m=1 volume constraint, move 0.1"},
            "newton_steps": mm.newton_steps, "gpu_launches_per_update": int(launches), "cpu_baseline": cpu}
    print(json.dumps(line))


def _default_iters(n):
    # Jacobi-PCG iterations grow ~linearly with the longest mesh dimension for this cantilever
    return (int(12 * max(n)), int(12 * max(n)))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--size", type=int, nargs=3, default=list(DEFAULT_SIZE))
    ap.add_argument("--extent", type=float, nargs=3, default=list(L),
                    help="box extents Lx Ly Lz (default the 2 x 1 x 0.5 cantilever; 1 1 1 with --size 100 100 100 "
                         "is the 100^3 unit cube)")
    ap.add_argument("--precision", default="mixed", choices=["mixed", "mixed_ssym", "mixed_sym"],
                    help="mixed-precision variant of the headline run (solver copy of the tangent)")
    ap.add_argument("--no-fp64", action="store_true", help="skip the plain FP64 comparison run")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--widened", action="store_true",
                    help="time the arc-length / dynamic-relaxation drivers and a Robin Newton solve (GPU and CPU port)")
    ap.add_argument("--mma-update", action="store_true",
                    help="time the TO update (filter + MMA) beside the step and print its own JSON line")
    ap.add_argument("--kernel-shares", action="store_true",
                    help="print per-kernel device time of one step per precision (CUPTI trace) and exit")
    args = ap.parse_args()
    if args.kernel_shares:
        kernel_shares(args)
        return
    if args.mma_update:
        mma_update_bench(args)
        return
    if args.widened:
        widened_bench(args)
        return

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.impl == "reference":
        if rank == 0:
            bench_reference(args)
        return

    import torch
    import jax_fem_gb300 as jf
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    n = tuple(args.size)
    name, cells, nodes, nnz = workload_name(n, tuple(args.extent))
    prob = make_problem(n, tuple(args.extent))
    eng = prob._engine
    theta0 = theta_init(cells).cuda()
    peak, peak_kind = measured_peak()
    lib = jf._lib.load()

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    def timed(precision, steps, warmup, record=None, spmv_timer=False):
        fwd_opts, adj_opts = options(precision)
        fwd = jf.ad_wrapper(prob, fwd_opts, adj_opts)
        for k in range(warmup):
            run_steps(prob, fwd, theta_step(theta0, 1000 + k))
        thetas = [theta_step(theta0, k) for k in range(steps)]
        eng.solve_log.clear()
        for k in eng.timing:
            eng.timing[k] = 0.0
        barrier()
        s = torch.cuda.current_stream()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        l0 = lib.fem_kernel_launches()
        if spmv_timer:   # CUDA events around the second SpMV of every 16-iteration chunk of the CG
            lib.fem_spmv_timing_start()
        e0.record(s)
        out = None
        for k in range(steps):
            out = run_steps(prob, fwd, thetas[k])
        e1.record(s)
        barrier()
        launches = lib.fem_kernel_launches() - l0
        t = max_over_ranks(e0.elapsed_time(e1) / 1e3, dist, "cuda")
        its = [r["iterations"] for r in eng.solve_log]
        if spmv_timer:
            sec, cnt = ctypes.c_double(), ctypes.c_int64()
            lib.fem_spmv_timing_stop(ctypes.byref(sec), ctypes.byref(cnt))
            spmv_in_loop.update(seconds=sec.value / max(cnt.value, 1), launches_timed=cnt.value)
        return t, out, launches, its, dict(eng.timing)

    # ---- mixed (headline) ------------------------------------------------------
    spmv_in_loop = {}
    with ClockSampler(local) as clk:
        t_mx, (J_mx, g_mx, u_mx), launches, its_mx, phases_mx = timed(args.precision, args.steps, args.warmup,
                                                                       spmv_timer=True)
    clocks = clk.summary()
    roof = spmv_roofline(prob, peak)
    asm_roof = assembly_roofline(prob, peak)

    # ---- plain FP64 ------------------------------------------------------------
    fp64 = None
    if not args.no_fp64:
        t_64, (J_64, g_64, u_64), _, its_64, phases_64 = timed("fp64", max(1, args.steps), max(3, args.warmup))
        roof.update({k: v for k, v in spmv_roofline(prob, peak).items() if k == "fp64"})
        rel = lambda a, b: float((a - b).abs().max() / b.abs().max())
        fp64 = {"value": t_64 / args.steps, "unit": UNIT, "speedup_mixed_vs_fp64": (t_64 / args.steps) / (t_mx / args.steps),
                "pcg_iterations": its_64, "phases_s": {k: v / args.steps for k, v in phases_64.items()},
                "errors_mixed_vs_fp64": {"solution": rel(u_mx, u_64), "compliance": abs(J_mx.item() - J_64.item()) / abs(J_64.item()),
                                         "gradient": rel(g_mx, g_64)}}

    # ---- e2e through the public API with host buffers ----------------------------
    fwd_opts, adj_opts = options(args.precision)
    fwd = jf.ad_wrapper(prob, fwd_opts, adj_opts)
    # the timed region's designs, as pinned host buffers (same workload, same iteration counts)
    theta_hosts = [theta_step(theta0, k).cpu().pin_memory() for k in range(args.steps)]
    grad_host = torch.empty_like(theta_hosts[0]).pin_memory()
    J_host = torch.empty(1, dtype=torch.float64).pin_memory()
    run_steps(prob, fwd, theta_step(theta0, 3000))   # one untimed step after the FP64 run
    torch.cuda.synchronize()
    barrier()
    t0 = time.perf_counter()
    for k in range(args.steps):
        th = theta_hosts[k].to("cuda", non_blocking=True)
        J, g, _ = run_steps(prob, fwd, th)
        grad_host.copy_(g, non_blocking=True)
        J_host.copy_(J.reshape(1), non_blocking=True)
        torch.cuda.synchronize()
    barrier()
    t_e2e = (time.perf_counter() - t0)
    h2d = theta_hosts[0].numel() * 8
    d2h = grad_host.numel() * 8 + 8

    # ---- CPU baseline (rank 0, N=1) ----------------------------------------------
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu and tuple(args.extent) == L:   # the port builds the cantilever
        it_full = (its_64[0], its_64[1]) if fp64 is not None and len(its_64) >= 2 else \
            (FULL_SIZE_PCG_ITERS if n == DEFAULT_SIZE else _default_iters(n))
        try:
            cpu, _ = cpu_baseline(n, it_full)
        except Exception as exc:  # noqa: BLE001
            cpu = {"value": None, "unit": UNIT, "cores": 0, "kind": "port", "sample": f"failed: {exc}"}

    head = "ssym_df48" if "ssym_df48" in roof else "sym_df48" if "sym_df48" in roof else "df48"
    f32 = roof.get(head, roof.get("fp32", {}))
    isolated = dict(f32)
    if spmv_in_loop.get("launches_timed") and f32.get("algorithmic_bytes"):
        # achieved = algorithmic bytes / the kernel's mean duration inside the timed solves
        t_loop = spmv_in_loop["seconds"]
        f32 = dict(f32, seconds=t_loop, achieved_gbs=f32["algorithmic_bytes"] / t_loop / 1e9,
                   frac=f32["algorithmic_bytes"] / t_loop / 1e9 / peak)
    traffic = traffic_from_profile(nnz, head)
    value = job_seconds_per_iter(t_mx, args.steps, world)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_mx / args.steps * 1e3, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "f64 residual / VJP assembly, double-float (fp32 pair) matrix assembly; DF48 matrix (fp32 hi + int16 lo) with double-float SpMV on fp32 pipes; double-float CG vectors, f64 dot finish and reliable updates",
        "data": "synthetic",
        "config": {"workload": name, "precision": args.precision, "tolerance": RTOL,
                   "solver": "block-Jacobi PCG, DF48 SpMV + double-float CG vectors, FP64 reliable updates (true residual)",
                   "l2": "inputs larger than L2 (the DF48 matrix alone is 1.5 GB > 129 MB)",
                   "replicas": "one independent problem per GPU (no data-path collective)"},
        "pcg_iterations": its_mx,
        "throughput": {"cells_per_s": cells * world / value, "dofs_per_s": nodes * 3 * world / value,
                       "cg_iterations_per_s": sum(its_mx) / max(args.steps, 1) * world / value,
                       "note": "one TO iteration (assemble + forward solve + adjoint + gradient) per unit of value"},
        "phases_s": {k: v / args.steps for k, v in phases_mx.items()},
        "fp64": fp64,
        "e2e": {"value": t_e2e / args.steps / world, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "roofline": {"bound": "hbm", "achieved": f32.get("achieved_gbs"), "peak": peak, "unit": "GB/s",
                     "frac": f32.get("frac"), "traffic": traffic,
                     "kernel": ("spmv_ssym_bulk_kernel (fem_spmv_dfx: FEM_SSYM_DF48 structured symmetric stencil "
                                "storage, implicit columns, transposed half in registers / warp shuffles, plane i+1 by "
                                "FP64 atomics; bulk-copy staged, double-float on FP32 pipes; timed call includes the "
                                "FP64 zero-fill and fold of the transposed part)" if head == "ssym_df48" else
                                "spmv_sliced_dfdf_bulk_kernel<3,SYM> (fem_spmv_dfx: FEM_SYM_DF48 upper node blocks, "
                                "transposed half by FP64 atomics, bulk-copy staged, double-float on FP32 pipes; "
                                "timed call includes the FP64 zero-fill and fold of the transposed half)"
                                if head == "sym_df48" else
                                "spmv_sliced_dfdf_bulk_kernel<3> (fem_spmv_dfx: FEM_SLICED_DF48, bulk-copy staged, "
                                "double-float on FP32 pipes)"),
                     "peak_kind": peak_kind, "algorithmic_bytes": f32.get("algorithmic_bytes"),
                     "launch_seconds": f32.get("seconds"),
                     "timing": ("CUDA events around the second SpMV of every 16-iteration chunk inside the timed "
                                f"mixed steps ({spmv_in_loop.get('launches_timed', 0)} launches)"
                                if spmv_in_loop.get("launches_timed") else "20 back-to-back launches"),
                     "isolated": {"seconds": isolated.get("seconds"), "achieved_gbs": isolated.get("achieved_gbs"),
                                  "frac": isolated.get("frac"), "how": "20 back-to-back launches after the timed steps"},
                     "fp64": roof.get("fp64"), "fp32": roof.get("fp32"),
                     "sliced_df48": roof.get("df48") if head != "df48" else None},
        "cpu_baseline": cpu,
        "clocks": clocks,
        "assembly": asm_roof,
        "gpu_launches": int(launches),
    }
    if rank == 0:
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
