"""Built-in tensor maps (material laws) for get_tensor_map().

In the reference, get_tensor_map() returns an arbitrary JAX function that is
differentiated with jacfwd (jax_fem/problem.py:262-266).  Here the laws are
compiled CUDA device functions with hand-derived consistent tangents, so
get_tensor_map() returns one of these tagged objects:

  Laplace(k)                      flux = k grad u       (test_linear_poisson.py:15-17)
  LinearElastic(E, nu)            Hooke                 (test_linear_elasticity_cube.py:15-26)
  SIMPElastic(Emax, Emin, nu, p)  Hooke with E(theta)   (topology_optimization example, 3D)
  GeneralLinear(C)                sigma_I = C_IJ grad_J (any linear map)
  NeoHookean(E, nu, with_rho)     dpsi/dF               (test_hyper_elasticity.py:17-34)
  J2Plasticity(E, nu, sig0)       radial return         (test_plasticity.py:32-78)

A plain Python callable taking only u_grad is accepted if it is linear: it is
probed on the host with basis inputs and replaced by GeneralLinear (or by
Laplace / LinearElastic when it has that structure).  Any other callable raises
NotImplementedError -- there is no CPU evaluation path.
"""
import numpy as np
import torch

from . import _lib


class Material:
    kind = 0
    vec = 3
    n_qp_params = 0
    param_index = None      # index into internal_vars of the differentiable per-point parameter
    history = False
    linear = True           # tangent independent of u
    symmetric = True

    def consts(self):
        raise NotImplementedError

    def bind(self, internal_vars, num_cells, num_quads, device):
        """Return (qp_params tensor or None, history tensor or None) on the device (FP64, contiguous)."""
        return None, None

    def diff_vars(self):
        """Differentiable internal variables: [(index into internal_vars, 'qp' | 'sigma' | 'eps')]."""
        return [] if self.param_index is None else [(self.param_index, "qp")]


def _per_qp(t, num_cells, num_quads, device, name):
    t = torch.as_tensor(t, dtype=torch.float64, device=device)
    n = t.numel()
    if n == num_cells * num_quads:
        return t.reshape(-1).contiguous()
    if n == num_cells:
        return t.reshape(num_cells, 1).expand(num_cells, num_quads).reshape(-1).contiguous()
    raise ValueError(f"{name} must have num_cells*num_quads ({num_cells * num_quads}) or num_cells "
                     f"({num_cells}) entries, got shape {tuple(t.shape)}")


class Laplace(Material):
    kind = _lib.FEM_MAT_LAPLACE
    vec = 1

    def __init__(self, k=1.0):
        self.k = float(k)

    def consts(self):
        return [self.k]


class LinearElastic(Material):
    kind = _lib.FEM_MAT_LINEAR_ELASTIC

    def __init__(self, E, nu):
        self.E, self.nu = float(E), float(nu)

    def consts(self):
        return [self.E, self.nu]


class SIMPElastic(Material):
    """E(theta) = Emin + (Emax - Emin) theta^penal ; theta = internal_vars[0] per quad point."""
    kind = _lib.FEM_MAT_SIMP
    n_qp_params = 1
    param_index = 0

    def __init__(self, Emax=1.0, Emin=1e-3, nu=0.3, penal=3.0):
        self.Emax, self.Emin, self.nu, self.penal = float(Emax), float(Emin), float(nu), float(penal)

    def consts(self):
        return [self.Emax, self.Emin, self.nu, self.penal]

    def bind(self, internal_vars, num_cells, num_quads, device):
        if len(internal_vars) < 1:
            raise ValueError("SIMPElastic needs internal_vars = [theta] (set_params)")
        return _per_qp(internal_vars[0], num_cells, num_quads, device, "theta"), None


class GeneralLinear(Material):
    kind = _lib.FEM_MAT_GENERAL_LINEAR

    def __init__(self, C, vec):
        C = np.asarray(C, dtype=np.float64)
        m = vec * 3
        if C.shape != (m, m):
            raise ValueError(f"GeneralLinear needs a ({m},{m}) matrix")
        self.C, self.vec = C, vec
        self.symmetric = bool(np.allclose(C, C.T, rtol=1e-12, atol=1e-14 * np.abs(C).max()))

    def consts(self):
        return self.C.reshape(-1).tolist()


class NeoHookean(Material):
    """Compressible Neo-Hookean; with_rho=True reads internal_vars[0] = rho (E scale) and clamps J."""
    kind = _lib.FEM_MAT_NEO_HOOKEAN
    linear = False

    def __init__(self, E, nu, with_rho=False, clamp_J=None):
        self.E, self.nu = float(E), float(nu)
        self.with_rho = bool(with_rho)
        self.clamp = self.with_rho if clamp_J is None else bool(clamp_J)
        if self.with_rho:
            self.n_qp_params = 1
            self.param_index = 0

    def consts(self):
        return [self.E, self.nu, 1.0 if self.clamp else 0.0]

    def bind(self, internal_vars, num_cells, num_quads, device):
        if not self.with_rho:
            return None, None
        return _per_qp(internal_vars[0], num_cells, num_quads, device, "rho"), None


class J2Plasticity(Material):
    """Small-strain J2 radial return; internal_vars = [sigmas_old, epsilons_old(, scale)] with
    sigmas/epsilons shaped (num_cells, num_quads, 3, 3) and an optional E scale per point."""
    kind = _lib.FEM_MAT_J2
    linear = False
    history = True

    def __init__(self, E, nu, sig0, modulus_field=False):
        self.E, self.nu, self.sig0 = float(E), float(nu), float(sig0)
        self.modulus_field = bool(modulus_field)
        if self.modulus_field:
            self.n_qp_params = 1
            self.param_index = 2

    def consts(self):
        return [self.E, self.nu, self.sig0]

    def diff_vars(self):
        # the history (sigmas_old, epsilons_old) is differentiable too: gradients over load steps
        return [(0, "sigma"), (1, "eps")] + ([(2, "qp")] if self.modulus_field else [])

    def bind(self, internal_vars, num_cells, num_quads, device):
        if len(internal_vars) < 2:
            raise ValueError("J2Plasticity needs internal_vars = [sigmas_old, epsilons_old]")
        s = torch.as_tensor(internal_vars[0], dtype=torch.float64, device=device).reshape(num_cells, num_quads, 9)
        e = torch.as_tensor(internal_vars[1], dtype=torch.float64, device=device).reshape(num_cells, num_quads, 9)
        hist = torch.cat([s, e], dim=2).contiguous()
        qp = None
        if self.modulus_field:
            qp = _per_qp(internal_vars[2], num_cells, num_quads, device, "modulus scale")
        return qp, hist


def probe_tensor_map(fn, vec):
    """Turn a linear Python tensor map u_grad -> stress into a built-in material."""
    if isinstance(fn, Material):
        if fn.vec != vec:
            raise ValueError(f"material {type(fn).__name__} is for vec={fn.vec}, problem has vec={vec}")
        return fn
    try:
        import inspect
        nparams = len(inspect.signature(fn).parameters)
    except (TypeError, ValueError):
        nparams = 1
    if nparams != 1:
        raise NotImplementedError(
            "get_tensor_map() returned a Python function with internal variables; declare the law with a "
            "built-in material (SIMPElastic, NeoHookean, J2Plasticity, ...) -- there is no CPU fallback")
    m = vec * 3

    def f(G):
        return np.asarray(fn(np.asarray(G, dtype=np.float64).reshape(vec, 3)), dtype=np.float64).reshape(m)

    try:
        f0 = f(np.zeros(m))
        C = np.stack([f(np.eye(m)[J]) - f0 for J in range(m)], axis=1)
        rng = np.random.default_rng(1234)
        ok = np.allclose(f0, 0.0, atol=1e-12 * (np.abs(C).max() + 1.0))
        for _ in range(3):
            G = rng.standard_normal(m)
            ok = ok and np.allclose(f(G), C @ G, rtol=1e-10, atol=1e-10 * (np.abs(C).max() + 1.0))
            ok = ok and np.allclose(f(3.0 * G), 3.0 * (C @ G), rtol=1e-10, atol=1e-10 * (np.abs(C).max() + 1.0))
    except Exception as exc:  # noqa: BLE001
        raise NotImplementedError(f"could not evaluate the tensor map on the host for probing: {exc}") from exc
    if not ok:
        raise NotImplementedError(
            "get_tensor_map() returned a nonlinear Python function; declare it with a built-in material "
            "(NeoHookean, J2Plasticity, ...) -- there is no CPU fallback")
    scale = np.abs(C).max() if np.abs(C).max() > 0 else 1.0
    if vec == 1 and np.allclose(C, C[0, 0] * np.eye(3), atol=1e-13 * scale):
        return Laplace(C[0, 0])
    if vec == 3:
        lam, mu = C[0, 4], C[1, 1]
        iso = np.zeros((9, 9))
        for i in range(3):
            for j in range(3):
                for k in range(3):
                    for l in range(3):
                        iso[i * 3 + j, k * 3 + l] = lam * (i == j) * (k == l) + mu * ((i == k) * (j == l) + (i == l) * (j == k))
        if np.allclose(C, iso, atol=1e-13 * scale) and mu > 0:
            nu = lam / (2.0 * (lam + mu))
            E = mu * (3.0 * lam + 2.0 * mu) / (lam + mu)
            return LinearElastic(E, nu)
    return GeneralLinear(C, vec)
