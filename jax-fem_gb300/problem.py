"""Problem: the reference's weak-form front end on top of the GB300 engine.

Mirrors jax_fem/problem.py:15-556 for single-variable problems: the same
constructor arguments and subclass hooks (custom_init, get_tensor_map,
get_mass_map, get_surface_maps, set_params), the same attributes
(fes, boundary_inds_list, internal_vars, ...) and the same compute_residual /
newton_update entry points.  The per-cell kernels and assembly run in the
native library; get_tensor_map() must return a built-in material (or a linear
Python map, probed once).  Solution and parameter arrays are torch tensors.
"""
import numpy as np
import torch

from . import _lib
from .device import Engine
from .fe import FiniteElement, eval_pointwise
from .logger import logger
from .materials import probe_tensor_map


class Problem:
    """Single-variable FE problem (problem.py:15-128).

    Parameters follow the reference: mesh, vec, dim, ele_type='HEX8',
    quadrature_rule=None, quadrature_order=None, dirichlet_bc_info=None,
    location_fns=None, additional_info=()."""

    def __init__(self, mesh, vec, dim, ele_type="HEX8", quadrature_rule=None, quadrature_order=None,
                 dirichlet_bc_info=None, location_fns=None, additional_info=()):
        if isinstance(mesh, list):
            if len(mesh) != 1:
                raise NotImplementedError("multi-variable problems are not part of this build")
            mesh, vec, ele_type = mesh[0], _first(vec), _first(ele_type)
            quadrature_rule, quadrature_order = _first(quadrature_rule), _first(quadrature_order)
            dirichlet_bc_info = _first(dirichlet_bc_info)
        self.mesh = [mesh]
        self.vec = [vec]
        self.dim = dim
        self.ele_type = [ele_type]
        self.quadrature_rule = [quadrature_rule]
        self.quadrature_order = [quadrature_order]
        self.dirichlet_bc_info = [dirichlet_bc_info]
        self.location_fns = location_fns
        self.additional_info = additional_info
        self.num_vars = 1
        self.fes = [FiniteElement(mesh, vec, dim, ele_type, quadrature_rule, quadrature_order, dirichlet_bc_info)]
        fe = self.fes[0]
        self.cells_list = [fe.cells]
        self.num_cells = fe.num_cells
        self.boundary_inds_list = fe.get_boundary_conditions_inds(location_fns)
        self.offset = [0]
        self.num_total_dofs_all_vars = fe.num_total_dofs
        self._params_version = 0
        self._internal_vars = ()
        self.internal_vars_surfaces = [() for _ in range(len(self.boundary_inds_list))]
        self._engine = None
        self._body_force = None
        self._surface_tractions = []
        self.custom_init(*additional_info)
        self._engine = Engine(self)
        self._prepare_maps()

    # ---- internal variables: any assignment bumps a version (device copies refresh) ----
    @property
    def internal_vars(self):
        return self._internal_vars

    @internal_vars.setter
    def internal_vars(self, value):
        self._internal_vars = value
        self._params_version += 1

    # ---- hooks (subclasses override) ---------------------------------------------
    def custom_init(self, *args):
        """problem.py:184-187."""
        pass

    def set_params(self, params):
        """problem.py:493-556: subclasses set self.internal_vars from params (torch ops)."""
        raise NotImplementedError("Child class must implement this function!")

    # ---- set-up of u-independent maps (mass / surface), evaluated once ----------------
    def _prepare_maps(self):
        fe = self.fes[0]
        eng = self._engine
        if hasattr(self, "get_universal_kernel") or hasattr(self, "get_universal_kernels_surface"):
            raise NotImplementedError("universal kernels (user per-cell kernels) are not part of this build")
        n_surf = len(self.boundary_inds_list)
        if hasattr(self, "get_surface_maps"):
            maps = self.get_surface_maps()
            assert n_surf == len(maps)          # problem.py:340-346
        else:
            assert n_surf == 0, "Missing definitions for surface integral"
            maps = []
        if hasattr(self, "get_mass_map"):
            xq, _ = eng.quad_points()
            x = xq.reshape(-1, 3).cpu().numpy()
            self._body_force = _u_independent(self.get_mass_map(), x, fe.vec, "mass map")
        self._surface_tractions = []
        for bi, fn in zip(self.boundary_inds_list, maps):
            if len(bi) == 0:
                self._surface_tractions.append(None)
                continue
            xf, _ = eng.face_quad_points(bi)
            x = xf.reshape(-1, 3).cpu().numpy()
            h, coeffs = _surface_map_split(fn, x, fe.vec)
            self._surface_tractions.append(h)
            if coeffs is not None:
                eng.add_robin(bi, coeffs)
        eng.refresh_loads()

    def _resolve_material(self):
        if not hasattr(self, "get_tensor_map"):
            raise NotImplementedError("get_tensor_map() is required (laplace kernel, problem.py:283-287)")
        return probe_tensor_map(self.get_tensor_map(), self.fes[0].vec)

    # ---- reference entry points ------------------------------------------------------
    def unflatten_fn_sol_list(self, dofs):
        return [dofs.reshape(self.fes[0].num_total_nodes, self.fes[0].vec)]

    def compute_residual(self, sol_list):
        """problem.py:462-475: residual list without Dirichlet rows applied."""
        dofs = _flat(sol_list, self._engine.device)
        res = self._engine.residual(dofs, apply_bc=False)
        return self.unflatten_fn_sol_list(res)

    def newton_update(self, sol_list):
        """problem.py:477-491: residual list; the tangent (no Dirichlet rows applied) is kept
        on the device and returned by solver.get_A(problem) after zeroRows."""
        dofs = _flat(sol_list, self._engine.device)
        res = self._engine.residual(dofs, apply_bc=False)
        self._newton_point = dofs.clone()
        return self.unflatten_fn_sol_list(res)


def _first(x):
    return x[0] if isinstance(x, list) else x


def _flat(sol_list, device):
    if isinstance(sol_list, (list, tuple)):
        if len(sol_list) != 1:
            raise NotImplementedError("single-variable problems only")
        sol_list = sol_list[0]
    return torch.as_tensor(sol_list, dtype=torch.float64, device=device).reshape(-1).contiguous()


def _surface_map_split(fn, x, vec, max_degree=4):
    """Split a surface map t(u, x) into h(x) = t(0, x) at the face quadrature points and, when t
    depends on u, component-wise polynomial coefficients c[v][k] (k = 0..deg, c[v][0] = 0) with
    t_v(u, x) = h_v(x) + sum_k c[v][k] u_v^k, found by probing and verified on random u.  Other
    u-dependence raises NotImplementedError.  Returns (h flat, coeffs (vec, deg+1) or None)."""
    P = len(x)
    h = eval_pointwise(lambda u, xx: fn(u, xx), [np.zeros((P, vec)), x], (vec,)).reshape(P, vec)
    rng = np.random.default_rng(7)
    probe = rng.integers(0, P, size=min(P, 3))
    t = lambda u, p: np.asarray(fn(np.asarray(u, dtype=np.float64), x[p]), dtype=np.float64).reshape(vec)
    if all(np.allclose(t(rng.standard_normal(vec), p), h[p], rtol=1e-12, atol=1e-12 * (np.abs(h[p]).max() + 1.0))
           for p in probe):
        return h.reshape(-1), None
    samples = np.array([-1.0, -0.5, 0.5, 1.0, 1.5, 2.0])
    V = samples[:, None] ** np.arange(1, max_degree + 1)[None, :]
    coeffs = np.zeros((vec, max_degree + 1))
    for v in range(vec):
        fits = []
        for p in probe:
            rows = []
            for sv in samples:
                u = np.zeros(vec)
                u[v] = sv
                tv = t(u, p) - h[p]
                others = np.delete(tv, v)
                if not np.allclose(others, 0.0, atol=1e-12 * (np.abs(tv).max() + 1.0)):
                    raise NotImplementedError("u-dependent surface maps must act component-wise")
                rows.append(tv[v])
            c, *_ = np.linalg.lstsq(V, np.array(rows), rcond=None)
            fits.append(c)
        fits = np.array(fits)
        if not np.allclose(fits, fits[0], rtol=1e-9, atol=1e-12 * (np.abs(fits).max() + 1.0)):
            raise NotImplementedError("the u-dependent part of a surface map must not depend on x")
        coeffs[v, 1:] = fits[0]
    scale = np.abs(coeffs).max()
    if scale == 0.0:
        raise NotImplementedError("u-dependent surface maps must act component-wise")
    coeffs[np.abs(coeffs) <= 1e-13 * scale] = 0.0
    deg = max(int(np.nonzero(np.abs(coeffs).max(0))[0].max()), 1)
    coeffs = coeffs[:, :deg + 1]
    for p in probe:
        u = rng.uniform(-1.5, 1.5, vec)
        pred = h[p] + np.array([np.polyval(coeffs[v][::-1], u[v]) for v in range(vec)])
        if not np.allclose(t(u, p), pred, rtol=1e-9, atol=1e-11 * (np.abs(pred).max() + 1.0)):
            raise NotImplementedError("only component-wise polynomial u-dependence (degree <= 4) is built for "
                                      "surface maps")
    logger.debug("surface map: u-dependent part of degree %d", deg)
    return h.reshape(-1), coeffs


def _u_independent(fn, x, vec, what):
    """Evaluate map(u, x) at points with u = 0 and check that it does not depend on u."""
    P = len(x)
    u0 = np.zeros((P, vec))
    val = eval_pointwise(lambda u, xx: fn(u, xx), [u0, x], (vec,))
    rng = np.random.default_rng(7)
    probe = rng.integers(0, P, size=min(P, 4))
    for p in probe:
        alt = np.asarray(fn(rng.standard_normal(vec), x[p]), dtype=np.float64).reshape(vec)
        if not np.allclose(alt, val[p], rtol=1e-12, atol=1e-12 * (np.abs(val[p]).max() + 1.0)):
            raise NotImplementedError(f"{what} depends on u; only u-independent {what}s are built")
    logger.debug("%s evaluated at %d points", what, P)
    return val.reshape(-1)
