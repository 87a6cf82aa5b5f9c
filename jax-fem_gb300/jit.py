"""Compiled user kernels: get_universal_kernel / get_universal_kernels_surface on the GPU.

The reference compiles the user's weak-form functions with XLA (jax.jit(jax.vmap(kernel)),
jax_fem/problem.py:335-338) and takes their tangent with jacfwd (problem.py:262-301).  Here the
user's function is traced once on the host: it is called with numpy object arrays whose entries
are symbolic scalars (every numpy operation that works elementwise on Python objects -- +, -, *,
/, **, sum, einsum, matmul, broadcasting, indexing, np.sin / exp / log / sqrt / tanh ... -- records
itself into an expression graph with common subexpressions merged).  The graph becomes a CUDA C++
device function templated on its scalar types, and a generated cell (or face) kernel evaluates it
per cell with the geometry recomputed from the element tables:

  residual          the function in FP64;
  tangent (CSR)     forward mode with a dual number per local dof, one sweep per column (jacfwd);
  tangent action    one dual sweep along the direction;
  parameter VJP     one dual sweep per internal-variable entry, contracted with the multiplier.

The source is compiled with NVRTC at run time (fem_jit_load) -- there is no CPU evaluation path.
Functions must be written with numpy (`import numpy as np` where the reference example imports
jax.numpy) and have no data-dependent branches; `vmap` and `ravel_pytree` below stand in for the
jax helpers the reference's examples use.
"""
import ctypes as C
import numbers

import numpy as np

from . import _lib
from ._lib import call

# ---------------------------------------------------------------------------------------------
# tracing


class _Trace:
    active = None

    def __init__(self):
        self.nodes = []
        self.table = {}


class Sym:
    """A scalar of the traced expression graph (hash-consed within the active trace)."""
    __slots__ = ("op", "args", "nid", "leaf")
    __array_priority__ = 1000

    def __bool__(self):
        raise NotImplementedError("data-dependent branches cannot be compiled: the kernel must be branch-free "
                                  "in the solution and the internal variables")

    # arithmetic -------------------------------------------------------------------------
    def __add__(self, o): return _bin("+", self, o)
    def __radd__(self, o): return _bin("+", o, self)
    def __sub__(self, o): return _bin("-", self, o)
    def __rsub__(self, o): return _bin("-", o, self)
    def __mul__(self, o): return _bin("*", self, o)
    def __rmul__(self, o): return _bin("*", o, self)
    def __truediv__(self, o): return _bin("/", self, o)
    def __rtruediv__(self, o): return _bin("/", o, self)
    def __pow__(self, o): return _pow(self, o)
    def __rpow__(self, o): return _pow(o, self)
    def __neg__(self): return _un("neg", self)
    def __pos__(self): return self
    def __abs__(self): return _un("fabs", self)

    def __lt__(self, o): return self.__bool__()
    __le__ = __gt__ = __ge__ = __lt__

    # numpy's object-dtype ufunc loops call these methods
    def sin(self): return _un("sin", self)
    def cos(self): return _un("cos", self)
    def tan(self): return _un("tan", self)
    def exp(self): return _un("exp", self)
    def log(self): return _un("log", self)
    def sqrt(self): return _un("sqrt", self)
    def tanh(self): return _un("tanh", self)
    def sinh(self): return _un("sinh", self)
    def cosh(self): return _un("cosh", self)
    def arctan(self): return _un("atan", self)
    def arcsin(self): return _un("asin", self)
    def arccos(self): return _un("acos", self)
    def absolute(self): return _un("fabs", self)
    def square(self): return _bin("*", self, self)
    def conjugate(self): return self


def _const(x):
    return isinstance(x, (numbers.Real, np.floating, np.integer)) and not isinstance(x, bool)


def _node(op, args, leaf=None):
    T = _Trace.active
    if T is None:
        raise RuntimeError("symbolic scalars exist only while a kernel is traced")
    key = (op, tuple(("S", a.nid) if isinstance(a, Sym) else ("c", float(a)) for a in args), leaf)
    n = T.table.get(key)
    if n is None:
        n = Sym.__new__(Sym)
        n.op, n.args, n.leaf, n.nid = op, tuple(args), leaf, len(T.nodes)
        T.nodes.append(n)
        T.table[key] = n
    return n


def _check(o):
    if isinstance(o, Sym):
        return o
    if _const(o):
        return float(o)
    raise NotImplementedError(f"unsupported operand in a compiled kernel: {type(o).__name__}")


def _bin(op, a, b):
    a, b = _check(a), _check(b)
    ca, cb = not isinstance(a, Sym), not isinstance(b, Sym)
    if ca and cb:
        return {"+": a + b, "-": a - b, "*": a * b, "/": a / b}[op]
    if op == "+":
        if ca and a == 0.0:
            return b
        if cb and b == 0.0:
            return a
    elif op == "-":
        if cb and b == 0.0:
            return a
        if ca and a == 0.0:
            return _un("neg", b)
    elif op == "*":
        if (ca and a == 0.0) or (cb and b == 0.0):
            return 0.0
        if ca and a == 1.0:
            return b
        if cb and b == 1.0:
            return a
        if ca and a == -1.0:
            return _un("neg", b)
        if cb and b == -1.0:
            return _un("neg", a)
    elif op == "/":
        if cb and b == 1.0:
            return a
        if ca and a == 0.0:
            return 0.0
    return _node(op, (a, b))


def _un(op, a):
    a = _check(a)
    if not isinstance(a, Sym):
        f = {"neg": lambda v: -v, "fabs": abs, "sin": np.sin, "cos": np.cos, "tan": np.tan, "exp": np.exp,
             "log": np.log, "sqrt": np.sqrt, "tanh": np.tanh, "sinh": np.sinh, "cosh": np.cosh, "atan": np.arctan,
             "asin": np.arcsin, "acos": np.arccos}[op]
        return float(f(a))
    if op == "neg" and a.op == "neg":
        return a.args[0]
    return _node(op, (a,))


def _pow(a, b):
    a, b = _check(a), _check(b)
    if not isinstance(a, Sym) and not isinstance(b, Sym):
        return float(a ** b)
    if not isinstance(b, Sym):
        if b == 0.0:
            return 1.0
        if b == 1.0:
            return a
        if b == 2.0:
            return _bin("*", a, a)
        if b == -1.0:
            return _bin("/", 1.0, a)
        if b == 0.5:
            return _un("sqrt", a)
    return _node("pow", (a, b))


def _inputs(kind, shape, start=0):
    n = int(np.prod(shape)) if len(shape) else 1
    arr = np.empty(n, dtype=object)
    for i in range(n):
        arr[i] = _node("in", (), leaf=(kind, start + i))
    return arr.reshape(shape)


def vmap(fn):
    """jax.vmap stand-in for traced kernels: fn over the leading axis of its (array) arguments."""
    def mapped(*args):
        outs = [fn(*[a[i] for a in args]) for i in range(len(args[0]))]
        return np.stack([np.asarray(o, dtype=object) for o in outs])
    return mapped


def ravel_pytree(tree):
    """jax.flatten_util.ravel_pytree stand-in: (flat array, unravel function) of an array or a list
    of arrays."""
    if isinstance(tree, (list, tuple)):
        parts = [np.asarray(t, dtype=object) for t in tree]
        shapes = [p.shape for p in parts]
        flat = np.concatenate([p.reshape(-1) for p in parts]) if parts else np.zeros(0, dtype=object)

        def unravel(v):
            out, o = [], 0
            for s in shapes:
                k = int(np.prod(s))
                out.append(np.asarray(v[o:o + k]).reshape(s))
                o += k
            return out
        return flat, unravel
    a = np.asarray(tree, dtype=object)
    return a.reshape(-1), (lambda v, s=a.shape: np.asarray(v).reshape(s))


# ---------------------------------------------------------------------------------------------
# code generation

_FN = {"sin": "sin", "cos": "cos", "tan": "tan", "exp": "exp", "log": "log", "sqrt": "sqrt", "tanh": "tanh",
       "sinh": "sinh", "cosh": "cosh", "atan": "atan", "asin": "asin", "acos": "acos", "fabs": "fabs"}


def _lit(v):
    v = float(v)
    if np.isnan(v):
        return "(0.0/0.0)"
    if np.isinf(v):
        return "(1.0/0.0)" if v > 0 else "(-1.0/0.0)"
    r = repr(v)
    return r if ("." in r or "e" in r or "n" in r) else r + ".0"


def _topo(outs):
    seen, order = set(), []
    stack = [(o, False) for o in outs if isinstance(o, Sym)]
    while stack:
        n, done = stack.pop()
        if n.nid in seen:
            continue
        if done:
            seen.add(n.nid)
            order.append(n)
            continue
        stack.append((n, True))
        for a in n.args:
            if isinstance(a, Sym) and a.nid not in seen:
                stack.append((a, False))
    return order


def emit_function(name, outs, leaf_names, n_out):
    """CUDA C++ of `template <TU, TI, TO> __device__ void name(...)` computing outs.  Leaves (kind, i)
    read leaf_names[kind][i]; intermediate values are `auto` so their type follows the inputs (FP64
    or dual)."""
    lines = []
    ref = {}
    for n in _topo(outs):
        if n.op == "in":
            kind, i = n.leaf
            ref[n.nid] = f"{leaf_names[kind]}[{i}]"
            continue
        a = [ref[x.nid] if isinstance(x, Sym) else _lit(x) for x in n.args]
        if n.op in ("+", "-", "*", "/"):
            e = f"{a[0]} {n.op} {a[1]}"
        elif n.op == "neg":
            e = f"-{a[0]}"
        elif n.op == "pow":
            e = f"pow({a[0]}, {a[1]})"
        else:
            e = f"{_FN[n.op]}({a[0]})"
        lines.append(f"  const auto v{n.nid} = {e};")
        ref[n.nid] = f"v{n.nid}"
    body = "\n".join(lines)
    assign = "\n".join(f"  out[{i}] = TO({ref[o.nid] if isinstance(o, Sym) else _lit(o)});"
                       for i, o in enumerate(outs))
    return (f"template <class TU, class TI, class TO>\n__device__ __forceinline__ void {name}("
            f"const TU* __restrict__ u, const double* __restrict__ ga, const double* __restrict__ gb, "
            f"const double* __restrict__ gc, const TI* __restrict__ iv, TO* __restrict__ out) {{\n"
            f"{body}\n{assign}\n}}\n")


_PRELUDE = r"""
typedef long long i64;
struct Params {
  const double* coords; const int* conn; i64 n_items; const int* face_cells; const int* face_ids;
  const double* u; const double* w; const double* lam; const double* iv; i64 iv_stride;
  const i64* indptr; const unsigned char* slots; const unsigned char* bc; i64 bc_mode; i64 outputs;
  double* res; double* vals; double* apply_out; double* vjp_out;
};
struct Dual {
  double v, d;
  __device__ Dual() : v(0.0), d(0.0) {}
  __device__ Dual(double a) : v(a), d(0.0) {}
  __device__ Dual(double a, double b) : v(a), d(b) {}
};
__device__ __forceinline__ Dual operator+(Dual a, Dual b) { return Dual(a.v + b.v, a.d + b.d); }
__device__ __forceinline__ Dual operator+(Dual a, double b) { return Dual(a.v + b, a.d); }
__device__ __forceinline__ Dual operator+(double a, Dual b) { return Dual(a + b.v, b.d); }
__device__ __forceinline__ Dual operator-(Dual a, Dual b) { return Dual(a.v - b.v, a.d - b.d); }
__device__ __forceinline__ Dual operator-(Dual a, double b) { return Dual(a.v - b, a.d); }
__device__ __forceinline__ Dual operator-(double a, Dual b) { return Dual(a - b.v, -b.d); }
__device__ __forceinline__ Dual operator-(Dual a) { return Dual(-a.v, -a.d); }
__device__ __forceinline__ Dual operator*(Dual a, Dual b) { return Dual(a.v * b.v, a.d * b.v + a.v * b.d); }
__device__ __forceinline__ Dual operator*(Dual a, double b) { return Dual(a.v * b, a.d * b); }
__device__ __forceinline__ Dual operator*(double a, Dual b) { return Dual(a * b.v, a * b.d); }
__device__ __forceinline__ Dual operator/(Dual a, Dual b) { const double q = a.v / b.v; return Dual(q, (a.d - q * b.d) / b.v); }
__device__ __forceinline__ Dual operator/(Dual a, double b) { return Dual(a.v / b, a.d / b); }
__device__ __forceinline__ Dual operator/(double a, Dual b) { const double q = a / b.v; return Dual(q, -q * b.d / b.v); }
__device__ __forceinline__ Dual sin(Dual a) { return Dual(sin(a.v), cos(a.v) * a.d); }
__device__ __forceinline__ Dual cos(Dual a) { return Dual(cos(a.v), -sin(a.v) * a.d); }
__device__ __forceinline__ Dual tan(Dual a) { const double t = tan(a.v); return Dual(t, (1.0 + t * t) * a.d); }
__device__ __forceinline__ Dual exp(Dual a) { const double e = exp(a.v); return Dual(e, e * a.d); }
__device__ __forceinline__ Dual log(Dual a) { return Dual(log(a.v), a.d / a.v); }
__device__ __forceinline__ Dual sqrt(Dual a) { const double s = sqrt(a.v); return Dual(s, 0.5 * a.d / s); }
__device__ __forceinline__ Dual tanh(Dual a) { const double t = tanh(a.v); return Dual(t, (1.0 - t * t) * a.d); }
__device__ __forceinline__ Dual sinh(Dual a) { return Dual(sinh(a.v), cosh(a.v) * a.d); }
__device__ __forceinline__ Dual cosh(Dual a) { return Dual(cosh(a.v), sinh(a.v) * a.d); }
__device__ __forceinline__ Dual atan(Dual a) { return Dual(atan(a.v), a.d / (1.0 + a.v * a.v)); }
__device__ __forceinline__ Dual asin(Dual a) { return Dual(asin(a.v), a.d / sqrt(1.0 - a.v * a.v)); }
__device__ __forceinline__ Dual acos(Dual a) { return Dual(acos(a.v), -a.d / sqrt(1.0 - a.v * a.v)); }
__device__ __forceinline__ Dual fabs(Dual a) { return a.v < 0.0 ? Dual(-a.v, -a.d) : a; }
__device__ __forceinline__ Dual pow(Dual a, double b) { const double p = pow(a.v, b); return Dual(p, b * pow(a.v, b - 1.0) * a.d); }
__device__ __forceinline__ Dual pow(double a, Dual b) { const double p = pow(a, b.v); return Dual(p, p * log(a) * b.d); }
__device__ __forceinline__ Dual pow(Dual a, Dual b) { const double p = pow(a.v, b.v); return Dual(p, p * (b.d * log(a.v) + b.v * a.d / a.v)); }
__device__ __forceinline__ double dpart(Dual a) { return a.d; }
"""


def _table(name, arr):
    a = np.asarray(arr, dtype=np.float64).reshape(-1)
    return f"__device__ const double {name}[{len(a)}] = {{{', '.join(_lit(v) for v in a)}}};\n"


_SCATTER = r"""
  // residual / tangent action / tangent / parameter VJP of one item (NN nodes, NDOF dofs)
  double uu[NDOF];
  int rows[NDOF];
  for (int a = 0; a < NN; ++a)
    for (int v = 0; v < VEC; ++v) {
      rows[a * VEC + v] = nd[a] * VEC + v;
      uu[a * VEC + v] = P.u[(i64)nd[a] * VEC + v];
    }
  const double* ivp = P.iv ? P.iv + e * P.iv_stride : nullptr;
  double ivl[IVS > 0 ? IVS : 1];
  for (int m = 0; m < IVS; ++m) ivl[m] = ivp[m];
  if (P.outputs & 1) {
    double r[NDOF];
    KFN<double, double, double>(uu, GA, GB, GC, ivl, r);
    for (int i = 0; i < NDOF; ++i)
      if (!(P.bc && P.bc[rows[i]])) atomicAdd(P.res + rows[i], r[i]);
  }
  if (P.outputs & 4) {
    Dual ud[NDOF], r[NDOF];
    for (int i = 0; i < NDOF; ++i) {
      double wv = P.w[rows[i]];
      if (P.bc && P.bc[rows[i]] && P.bc_mode == 2) wv = 0.0;
      ud[i] = Dual(uu[i], wv);
    }
    KFN<Dual, double, Dual>(ud, GA, GB, GC, ivl, r);
    for (int i = 0; i < NDOF; ++i)
      if (!(P.bc && P.bc[rows[i]])) atomicAdd(P.apply_out + rows[i], r[i].d);
  }
  if (P.outputs & 2) {
    for (int j = 0; j < NDOF; ++j) {
      const bool col_bc = P.bc && P.bc[rows[j]];
      if (col_bc && P.bc_mode == 2) continue;
      Dual ud[NDOF], r[NDOF];
      for (int i = 0; i < NDOF; ++i) ud[i] = Dual(uu[i], i == j ? 1.0 : 0.0);
      KFN<Dual, double, Dual>(ud, GA, GB, GC, ivl, r);
      const int b = j / VEC, k = j - VEC * (j / VEC);
      for (int i = 0; i < NDOF; ++i) {
        if (P.bc && P.bc[rows[i]] && P.bc_mode != 0) continue;
        const int a = i / VEC;
        const unsigned char s = P.slots[(CELL * NN + a) * NN + b];
        atomicAdd(P.vals + P.indptr[rows[i]] + VEC * s + k, r[i].d);
      }
    }
  }
  if ((P.outputs & 8) && IVS > 0) {
    double lam[NDOF];
    for (int i = 0; i < NDOF; ++i) lam[i] = (P.bc && P.bc[rows[i]]) ? 0.0 : P.lam[rows[i]];
    for (int m = 0; m < IVS; ++m) {
      Dual ivd[IVS > 0 ? IVS : 1], r[NDOF];
      for (int t = 0; t < IVS; ++t) ivd[t] = Dual(ivl[t], t == m ? 1.0 : 0.0);
      KFN<double, Dual, Dual>(uu, GA, GB, GC, ivd, r);
      double s = 0.0;
      for (int i = 0; i < NDOF; ++i) s += lam[i] * r[i].d;
      P.vjp_out[e * P.iv_stride + m] = -s;
    }
  }
"""


def cell_source(fn_src, tables, nn, nq, vec, ivs, kfn="ukernel"):
    """Generated cell kernel `fem_ucell`: geometry of each cell from the volume tables (fe.py:112-141
    conventions: J = X^T dN, grads = dN J^-1, JxW = det J w), then the user function."""
    src = [_PRELUDE, _table("SV", tables["shape_vals"]), _table("SG", tables["shape_grads_ref"]),
           _table("QW", tables["quad_weights"]), fn_src]
    src.append(f"""
#define NN {nn}
#define NQ {nq}
#define VEC {vec}
#define NDOF {nn * vec}
#define IVS {ivs}
#define KFN {kfn}
#define GA xq
#define GB gq
#define GC jv
#define CELL e
extern "C" __global__ void __launch_bounds__(128) fem_ucell(Params P) {{
  for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < P.n_items; e += (i64)gridDim.x * blockDim.x) {{
    int nd[NN];
    double X[NN * 3];
    for (int a = 0; a < NN; ++a) {{
      nd[a] = P.conn[e * NN + a];
      for (int d = 0; d < 3; ++d) X[a * 3 + d] = P.coords[(i64)nd[a] * 3 + d];
    }}
    // xq (NQ,3) physical points; gq (NQ,NN,3) shape grads; jv = [JxW (NQ) | v_grads_JxW (NQ,NN,3)]
    double xq[NQ * 3], gq[NQ * NN * 3], jv[NQ + NQ * NN * 3];
    for (int q = 0; q < NQ; ++q) {{
      double J[3][3];
      for (int d = 0; d < 3; ++d)
        for (int f = 0; f < 3; ++f) {{
          double s = 0.0;
          for (int a = 0; a < NN; ++a) s += X[a * 3 + d] * SG[(q * NN + a) * 3 + f];
          J[d][f] = s;
        }}
      const double det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) - J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
                         J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
      const double id = 1.0 / det;
      double I[3][3];
      I[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) * id; I[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) * id;
      I[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * id; I[1][0] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) * id;
      I[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * id; I[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * id;
      I[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) * id; I[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) * id;
      I[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * id;
      const double jxw = det * QW[q];
      jv[q] = jxw;
      for (int a = 0; a < NN; ++a)
        for (int d = 0; d < 3; ++d) {{
          double s = 0.0;
          for (int f = 0; f < 3; ++f) s += SG[(q * NN + a) * 3 + f] * I[f][d];
          gq[(q * NN + a) * 3 + d] = s;
          jv[NQ + (q * NN + a) * 3 + d] = s * jxw;
        }}
      for (int d = 0; d < 3; ++d) {{
        double s = 0.0;
        for (int a = 0; a < NN; ++a) s += SV[q * NN + a] * X[a * 3 + d];
        xq[q * 3 + d] = s;
      }}
    }}
{_SCATTER}
  }}
}}
""")
    return "".join(src)


def face_source(fn_srcs, tables, nn, vec, ivs):
    """Generated face kernels `fem_uface_<k>` (one per surface kernel): per selected face, the
    cell's geometry at the face quadrature points (fe.py:143-218: grads = dN J^-1, Nanson scale
    |n J^-1| det J w, physical points), then the user function."""
    fsv, fsg = np.asarray(tables["face_shape_vals"]), np.asarray(tables["face_shape_grads_ref"])
    nf, nfq = fsv.shape[0], fsv.shape[1]
    src = [_PRELUDE, _table("FSV", fsv), _table("FSG", fsg), _table("FW", tables["face_quad_weights"]),
           _table("FN", tables["face_normals"])]
    src.append(f"""
#define NN {nn}
#define NFQ {nfq}
#define VEC {vec}
#define NDOF {nn * vec}
#define IVS {ivs}
#define GA xq
#define GB fsvp
#define GC gn
#define CELL cell
__device__ __forceinline__ void face_geometry(const double* X, int f, double* xq, double* gn) {{
  // gn = [face shape grads (NFQ,NN,3) | nanson scale (NFQ)]
  for (int q = 0; q < NFQ; ++q) {{
    const double* dN = FSG + ((i64)(f * NFQ + q) * NN) * 3;
    double J[3][3];
    for (int d = 0; d < 3; ++d)
      for (int g = 0; g < 3; ++g) {{
        double s = 0.0;
        for (int a = 0; a < NN; ++a) s += X[a * 3 + d] * dN[a * 3 + g];
        J[d][g] = s;
      }}
    const double det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) - J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
                       J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
    const double id = 1.0 / det;
    double I[3][3];
    I[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) * id; I[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) * id;
    I[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * id; I[1][0] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) * id;
    I[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * id; I[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * id;
    I[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) * id; I[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) * id;
    I[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * id;
    for (int a = 0; a < NN; ++a)
      for (int d = 0; d < 3; ++d) {{
        double s = 0.0;
        for (int g = 0; g < 3; ++g) s += dN[a * 3 + g] * I[g][d];
        gn[(q * NN + a) * 3 + d] = s;
      }}
    double nv = 0.0;
    for (int d = 0; d < 3; ++d) {{
      double s = 0.0;
      for (int g = 0; g < 3; ++g) s += FN[f * 3 + g] * I[g][d];
      nv += s * s;
    }}
    gn[NFQ * NN * 3 + q] = sqrt(nv) * det * FW[f * NFQ + q];
    for (int d = 0; d < 3; ++d) {{
      double s = 0.0;
      for (int a = 0; a < NN; ++a) s += FSV[(f * NFQ + q) * NN + a] * X[a * 3 + d];
      xq[q * 3 + d] = s;
    }}
  }}
}}
""")
    for k, fs in enumerate(fn_srcs):
        src.append(fs)
        src.append(f"""
#define KFN ukernel_face_{k}
extern "C" __global__ void __launch_bounds__(128) fem_uface_{k}(Params P) {{
  for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < P.n_items; e += (i64)gridDim.x * blockDim.x) {{
    const i64 cell = P.face_cells[e];
    const int f = P.face_ids[e];
    int nd[NN];
    double X[NN * 3];
    for (int a = 0; a < NN; ++a) {{
      nd[a] = P.conn[cell * NN + a];
      for (int d = 0; d < 3; ++d) X[a * 3 + d] = P.coords[(i64)nd[a] * 3 + d];
    }}
    double xq[NFQ * 3], gn[NFQ * NN * 3 + NFQ];
    face_geometry(X, f, xq, gn);
    const double* fsvp = FSV + (i64)f * NFQ * NN;
{_SCATTER}
  }}
}}
#undef KFN
""")
    return "".join(src)


# ---------------------------------------------------------------------------------------------
# tracing the reference's kernel signatures

def trace_cell(fn, nn, nq, vec, iv_shapes):
    """Trace fn(cell_sol_flat, x, cell_shape_grads, cell_JxW, cell_v_grads_JxW, *cell_internal_vars)
    (problem.py:289-294; cell_JxW shaped (num_vars, nq), cell_v_grads_JxW (nq, nn, 1, dim)).
    Returns (CUDA function source, per-cell internal-variable size)."""
    T = _Trace()
    _Trace.active = T
    try:
        u = _inputs("u", (nn * vec,))
        x = _inputs("ga", (nq, 3))
        g = _inputs("gb", (nq, nn, 3))
        jv = _inputs("gc", (nq + nq * nn * 3,))
        jxw = jv[:nq].reshape(1, nq)
        vg = jv[nq:].reshape(nq, nn, 1, 3)
        ivs, off = [], 0     # the internal variables, concatenated per cell in order
        for s in iv_shapes:
            k = int(np.prod(s))
            ivs.append(_inputs("iv", (k,), off).reshape(s) if k else np.zeros(s, dtype=object))
            off += k
        out = np.asarray(fn(u, x, g, jxw, vg, *ivs), dtype=object).reshape(-1)
    finally:
        _Trace.active = None
    if out.size != nn * vec:
        raise ValueError(f"universal kernel returned {out.size} values, expected num_nodes*vec = {nn * vec}")
    return emit_function("ukernel", list(out), _LEAVES, nn * vec), off


def trace_face(fn, nn, nfq, vec, k):
    """Trace fn(cell_sol_flat, x, face_shape_vals, face_shape_grads, face_nanson_scale)
    (problem.py:318-323; face_nanson_scale shaped (num_vars, nfq))."""
    T = _Trace()
    _Trace.active = T
    try:
        u = _inputs("u", (nn * vec,))
        x = _inputs("ga", (nfq, 3))
        fsv = _inputs("gb", (nfq, nn))
        gn = _inputs("gc", (nfq * nn * 3 + nfq,))
        fg = gn[:nfq * nn * 3].reshape(nfq, nn, 3)
        nanson = gn[nfq * nn * 3:].reshape(1, nfq)
        out = np.asarray(fn(u, x, fsv, fg, nanson), dtype=object).reshape(-1)
    finally:
        _Trace.active = None
    if out.size != nn * vec:
        raise ValueError(f"surface universal kernel returned {out.size} values, expected {nn * vec}")
    return emit_function(f"ukernel_face_{k}", list(out), _LEAVES, nn * vec)


# leaf kinds -> the generated function's parameters: u (dofs), ga / gb / gc (geometry: cell x,
# shape grads, [JxW | v_grads_JxW]; face x, face shape values, [face shape grads | Nanson]), iv
_LEAVES = {"u": "u", "ga": "ga", "gb": "gb", "gc": "gc", "iv": "iv"}


class CompiledKernels:
    """The problem's universal kernels, compiled for the current device."""

    def __init__(self, source, cell_iv, face_count):
        self.source = source
        self.cell_iv = cell_iv
        self.face_count = face_count
        h = C.c_void_p()
        call("fem_jit_load", source.encode(), C.byref(h))
        self.handle = h

    def launch(self, kernel, params, n_items, stream):
        call("fem_jit_launch", self.handle, kernel.encode(), C.byref(params), int(n_items), stream)


def params(**kw):
    """fem_jit_params_t with the given fields (device pointers as ints or None)."""
    P = _lib.FemJitParams()
    for k, v in kw.items():
        setattr(P, k, 0 if v is None else v)
    return P
