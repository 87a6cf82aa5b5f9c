"""The universal-kernel compiler on the CPU (no GPU): the tracer records the reference's kernel
forms (applications/robin_bc/example.py:19-80, written with numpy) into an expression graph whose
values -- evaluated here by a small test-side interpreter on one cell's real geometry -- equal the
oracle's torch evaluation of the same kernels, and the generated CUDA sources compile with NVRTC for
sm_103a."""
import ctypes as C
import importlib

import numpy as np
import pytest
import torch

jit = importlib.import_module("jax_fem_gb300.jit")


def _oracle_tables():
    from oracle import basis as obasis
    return obasis.element_tables("HEX8")


def _kernels(SV, nn, vec, xp=np, vm=None):
    """The Robin example's universal kernels (problem.py:289-294, :318-323 signatures), written once
    for numpy (traced) and once for torch (the oracle), 3D."""
    vm = vm or jit.vmap

    def universal_kernel(cell_sol_flat, x, cell_shape_grads, cell_JxW, cell_v_grads_JxW, *iv):
        cell_sol = cell_sol_flat.reshape(nn, vec)
        jxw = cell_JxW[0]
        dx = x[:, 0] - 0.5
        dy = x[:, 1] - 0.5
        body = x[:, 0] * xp.sin(5.0 * np.pi * x[:, 1]) + 1.0 * xp.exp(-(dx * dx + dy * dy) / 0.02)
        body = body[:, None]
        u_grads = (cell_sol[None, :, :, None] * cell_shape_grads[:, :, None, :]).sum(1)
        k = (1.0 + iv[0][:, 0] ** 2)[:, None, None] if iv else 1.0
        val = (k * u_grads[:, None, :, :] * cell_v_grads_JxW).sum((0, 3))
        bv = (body[:, None, :] * SV[:, :, None] * jxw[:, None, None]).sum(0)
        return (val - bv).reshape(-1)

    def robin_kernel(cell_sol_flat, x, face_shape_vals, face_shape_grads, face_nanson_scale):
        cell_sol = cell_sol_flat.reshape(nn, vec)
        nanson = face_nanson_scale[0]
        u = (cell_sol[None, :, :] * face_shape_vals[:, :, None]).sum(1)
        up = vm(lambda uu: 5 * uu ** 2)(u)
        return (up[:, None, :] * face_shape_vals[:, :, None] * nanson[:, None, None]).sum(0).reshape(-1)

    return universal_kernel, robin_kernel


def _evaluate(outs, leaves):
    """Test-side interpreter of a traced graph: leaves maps kind -> flat numpy array."""
    memo = {}
    fns = {"sin": np.sin, "cos": np.cos, "tan": np.tan, "exp": np.exp, "log": np.log, "sqrt": np.sqrt,
           "tanh": np.tanh, "sinh": np.sinh, "cosh": np.cosh, "atan": np.arctan, "asin": np.arcsin,
           "acos": np.arccos, "fabs": np.abs}

    def ev(n):
        if not isinstance(n, jit.Sym):
            return float(n)
        if n.nid in memo:
            return memo[n.nid]
        if n.op == "in":
            v = float(leaves[n.leaf[0]][n.leaf[1]])
        else:
            a = [ev(x) for x in n.args]
            v = {"+": lambda: a[0] + a[1], "-": lambda: a[0] - a[1], "*": lambda: a[0] * a[1],
                 "/": lambda: a[0] / a[1], "neg": lambda: -a[0], "pow": lambda: a[0] ** a[1]}.get(
                n.op, lambda: fns[n.op](a[0]))()
        memo[n.nid] = v
        return v
    return np.array([ev(o) for o in outs])


def _trace_outs(fn, args_shapes, iv_shapes=()):
    T = jit._Trace()
    jit._Trace.active = T
    try:
        ins = [jit._inputs(k, s) for k, s in args_shapes]
        off, ivs = 0, []
        for s in iv_shapes:
            k = int(np.prod(s))
            ivs.append(jit._inputs("iv", (k,), off).reshape(s))
            off += k
        return list(np.asarray(fn(*ins, *ivs), dtype=object).reshape(-1))
    finally:
        jit._Trace.active = None


def test_traced_cell_kernel_matches_torch_oracle():
    from oracle import fem as ofem
    t = _oracle_tables()
    pts, cells = ofem.box_mesh(2, 2, 2, 1.0, 1.0, 1.0)
    pts = pts + np.random.default_rng(0).uniform(-0.03, 0.03, pts.shape)
    fe = ofem.OracleFE(pts, cells, 1)
    nn, nq, vec = 8, 8, 1
    c = 3
    G, jxw = fe.shape_grads[c], fe.JxW[c]
    x = fe.get_physical_quad_points()[c]
    u = np.random.default_rng(1).standard_normal(nn)
    th = np.random.default_rng(2).uniform(0.5, 1.5, (nq, 1))
    uk_np, _ = _kernels(t["shape_vals"], nn, vec)
    uk_t, _ = _kernels(torch.tensor(t["shape_vals"]), nn, vec, xp=torch)
    outs = _trace_outs(lambda uu, xx, gc, *iv: uk_np(uu, xx, gc[:nq * nn * 3].reshape(nq, nn, 3),
                                                     gc[nq * nn * 3:nq * nn * 3 + nq].reshape(1, nq),
                                                     gc[nq * nn * 3 + nq:].reshape(nq, nn, 1, 3), *iv),
                       [("u", (nn * vec,)), ("ga", (nq, 3)), ("gc", (nq * nn * 3 + nq + nq * nn * 3,))], [(nq, 1)])
    gc = np.concatenate([G.reshape(-1), jxw.reshape(-1), (G * jxw[:, None, None]).reshape(-1)])
    got = _evaluate(outs, {"u": u, "ga": x.reshape(-1), "gc": gc, "iv": th.reshape(-1)})
    tt = lambda a: torch.tensor(a, dtype=torch.float64)
    ref = uk_t(tt(u), tt(x), tt(G), tt(jxw)[None, :], tt(G * jxw[:, None, None])[:, :, None, :], tt(th)).numpy()
    assert np.abs(got - ref).max() <= 1e-13 * np.abs(ref).max()


def test_traced_face_kernel_and_helpers():
    t = _oracle_tables()
    nn, nfq, vec = 8, 4, 1
    _, rk = _kernels(t["shape_vals"], nn, vec)
    outs = _trace_outs(rk, [("u", (nn,)), ("ga", (nfq, 3)), ("gb", (nfq, nn)), ("gc", (nfq, nn, 3)),
                            ("iv", (1, nfq))])
    rng = np.random.default_rng(5)
    u, fv, nan = rng.standard_normal(nn), rng.uniform(0, 1, (nfq, nn)), rng.uniform(0.1, 1, nfq)
    got = _evaluate(outs, {"u": u, "ga": np.zeros(nfq * 3), "gb": fv.reshape(-1), "gc": np.zeros(nfq * nn * 3),
                           "iv": nan})
    uq = fv @ u
    ref = ((5 * uq ** 2 * nan)[:, None] * fv).sum(0)
    assert np.abs(got - ref).max() <= 1e-13 * np.abs(ref).max()
    flat, unravel = jit.ravel_pytree([np.arange(6.0).reshape(2, 3), np.ones(2)])
    assert flat.shape == (8,) and np.allclose(unravel(flat)[0], np.arange(6.0).reshape(2, 3))


def test_data_dependent_branch_is_refused():
    def branchy(u, x, g, jxw, vg):
        return np.array([u[0] if u[0] > 0 else -u[0]] + [0.0] * 7)
    with pytest.raises(NotImplementedError):
        jit.trace_cell(branchy, 8, 8, 1, [])


def _nvrtc():
    for name in ("libnvrtc.so.13", "libnvrtc.so"):
        try:
            return C.CDLL(name)
        except OSError:
            continue
    pytest.skip("NVRTC not found")


def _compile(lib, src):
    prog = C.c_void_p()
    assert lib.nvrtcCreateProgram(C.byref(prog), src.encode(), b"g.cu", 0, None, None) == 0
    opts = (C.c_char_p * 4)(b"--gpu-architecture=sm_103a", b"--std=c++17", b"--fmad=true", b"-default-device")
    rc = lib.nvrtcCompileProgram(prog, 4, opts)
    n = C.c_size_t()
    lib.nvrtcGetProgramLogSize(prog, C.byref(n))
    log = C.create_string_buffer(n.value)
    lib.nvrtcGetProgramLog(prog, log)
    lib.nvrtcDestroyProgram(C.byref(prog))
    return rc, log.value.decode(errors="replace")


@pytest.mark.parametrize("vec", [1, 3])
def test_generated_sources_compile_for_sm103a(vec):
    lib = _nvrtc()
    t = _oracle_tables()
    nn, nq = 8, 8
    uk, rk = _kernels(t["shape_vals"], nn, vec)
    fsrc, ivs = jit.trace_cell(uk, nn, nq, vec, [(nq, 1)])
    rc, log = _compile(lib, jit.cell_source(fsrc, t, nn, nq, vec, ivs))
    assert rc == 0, log
    face = jit.face_source([jit.trace_face(rk, nn, t["face_shape_vals"].shape[1], vec, k) for k in range(2)], t, nn,
                           vec, 0)
    rc, log = _compile(lib, face)
    assert rc == 0, log
