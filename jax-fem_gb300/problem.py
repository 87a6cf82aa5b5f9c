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
        n_surf = len(self.boundary_inds_list)
        if hasattr(self, "get_surface_maps"):
            maps = self.get_surface_maps()
            assert n_surf == len(maps)          # problem.py:340-346
        else:
            # surface terms may come from get_universal_kernels_surface alone (problem.py:305-332)
            assert n_surf == 0 or hasattr(self, "get_universal_kernels_surface"), \
                "Missing definitions for surface integral"
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
            if hasattr(self, "get_universal_kernel") or hasattr(self, "get_universal_kernels_surface"):
                # the physics is all in the universal kernels (problem.py:283-294 add no laplace term)
                return probe_tensor_map(lambda u_grad: 0.0 * u_grad, self.fes[0].vec)
            raise NotImplementedError("get_tensor_map() or get_universal_kernel() is required "
                                      "(problem.py:283-294)")
        return probe_tensor_map(self.get_tensor_map(), self.fes[0].vec)

    # ---- helpers the reference's universal kernels call (problem.py:86-92) -------------------
    def unflatten_fn_dof(self, dof_flat):
        """Cell dofs (num_nodes*vec,) -> [(num_nodes, vec)] (one variable)."""
        fe = self.fes[0]
        return [dof_flat.reshape(fe.num_nodes, fe.vec)]

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
    t_v(u, x) = h_v(x) + sum_k c[v][k] u_v^k.  Every probe is evaluated at every face quadrature
    point (one vectorised call where the map allows it), so u-dependence confined to part of the
    boundary is still seen.  Other u-dependence raises NotImplementedError.
    Returns (h flat, coeffs (vec, deg+1) or None)."""
    P = len(x)
    ev = lambda u: eval_pointwise(lambda uu, xx: fn(uu, xx), [u, x], (vec,)).reshape(P, vec)
    h = ev(np.zeros((P, vec)))
    rng = np.random.default_rng(7)
    tol = lambda ref: 1e-12 * (np.abs(ref).max(axis=-1, keepdims=True) + 1.0)
    if np.all(np.abs(ev(rng.standard_normal((P, vec))) - h) <= tol(h)):
        return h.reshape(-1), None
    samples = np.array([-1.0, -0.5, 0.5, 1.0, 1.5, 2.0])
    V = samples[:, None] ** np.arange(1, max_degree + 1)[None, :]
    coeffs = np.zeros((vec, max_degree + 1))
    for v in range(vec):
        rows = np.empty((len(samples), P))
        for k, sv in enumerate(samples):
            u = np.zeros((P, vec))
            u[:, v] = sv
            tv = ev(u) - h
            others = np.delete(tv, v, axis=1)
            if not np.all(np.abs(others) <= 1e-12 * (np.abs(tv).max(axis=1, keepdims=True) + 1.0)):
                raise NotImplementedError("u-dependent surface maps must act component-wise")
            rows[k] = tv[:, v]
        fits, *_ = np.linalg.lstsq(V, rows, rcond=None)          # (max_degree, P): one fit per point
        ref = fits[:, :1]
        if not np.all(np.abs(fits - ref) <= 1e-9 * np.abs(ref) + 1e-12 * (np.abs(fits).max() + 1.0)):
            raise NotImplementedError("the u-dependent part of a surface map must not depend on x")
        coeffs[v, 1:] = ref[:, 0]
    scale = np.abs(coeffs).max()
    if scale == 0.0:
        raise NotImplementedError("u-dependent surface maps must act component-wise")
    coeffs[np.abs(coeffs) <= 1e-13 * scale] = 0.0
    deg = max(int(np.nonzero(np.abs(coeffs).max(0))[0].max()), 1)
    coeffs = coeffs[:, :deg + 1]
    u = rng.uniform(-1.5, 1.5, (P, vec))
    pred = h + np.stack([np.polyval(coeffs[v][::-1], u[:, v]) for v in range(vec)], axis=1)
    if not np.all(np.abs(ev(u) - pred) <= 1e-9 * np.abs(pred) + 1e-11 * (np.abs(pred).max(axis=1, keepdims=True) + 1.0)):
        raise NotImplementedError("only component-wise polynomial u-dependence (degree <= 4) is built for "
                                  "surface maps")
    logger.debug("surface map: u-dependent part of degree %d", deg)
    return h.reshape(-1), coeffs


def _u_independent(fn, x, vec, what):
    """Evaluate map(u, x) at every point with u = 0 and check, again at every point, that a
    random u gives the same value (a map whose u-dependence is confined to part of the domain
    is refused, not integrated as a constant load)."""
    P = len(x)
    val = eval_pointwise(lambda u, xx: fn(u, xx), [np.zeros((P, vec)), x], (vec,)).reshape(P, vec)
    rng = np.random.default_rng(7)
    alt = eval_pointwise(lambda u, xx: fn(u, xx), [rng.standard_normal((P, vec)), x], (vec,)).reshape(P, vec)
    if not np.all(np.abs(alt - val) <= 1e-12 * np.abs(val) + 1e-12 * (np.abs(val).max(axis=1, keepdims=True) + 1.0)):
        raise NotImplementedError(f"{what} depends on u; only u-independent {what}s are built")
    logger.debug("%s evaluated at %d points", what, P)
    return val.reshape(-1)
