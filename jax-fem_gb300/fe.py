"""FiniteElement: per-variable element data, Dirichlet sets and boundary faces.

Mirrors jax_fem/fe.py:20-382.  Host-side set-up (evaluating the user's
location / value functions on mesh points) stays in numpy, as in the
reference; the geometric quantities the hot path needs are recomputed per
cell inside the CUDA kernels instead of being stored (fe.py:112-141 stores
(cells, quads, nodes, dim) arrays -- 1.5 GB in FP64 at 1M HEX8 cells).
The geometry accessors below are post-processing helpers evaluated on the
device with torch and are not used by the solver.
"""
import inspect

import numpy as np
import torch

from . import basis
from .logger import logger


def _nargs(fn):
    try:
        return fn.__code__.co_argcount
    except AttributeError:
        return len(inspect.signature(fn).parameters)


def eval_pointwise(fn, args, out_shape_tail=()):
    """Evaluate a user point function on P points.

    args: list of arrays shaped (P, ...).  The reference vmaps the function
    (fe.py:241-253); here we first try one vectorised call with the point axis
    last (so `point[0]` selects the x row of all points), verify it on a few
    points against per-point calls, and otherwise loop over points."""
    P = args[0].shape[0]
    if P == 0:
        return np.zeros((0,) + tuple(out_shape_tail))

    def single(p):
        return np.asarray(fn(*[a[p] for a in args]), dtype=np.float64)

    vec_res = None
    try:
        with np.errstate(all="ignore"):
            r = np.asarray(fn(*[np.moveaxis(a, 0, -1) for a in args]), dtype=np.float64)
        tail = tuple(out_shape_tail)
        if r.shape == tail + (P,):
            vec_res = np.moveaxis(r, -1, 0)
        elif r.shape == tail or (r.ndim == 0 and tail == ()):
            vec_res = np.broadcast_to(r, (P,) + tail).copy()
    except Exception:  # noqa: BLE001 -- any failure means "not vectorisable"
        vec_res = None
    if vec_res is not None:
        probe = np.unique(np.linspace(0, P - 1, min(P, 7)).astype(np.int64))
        ok = all(np.allclose(vec_res[p], single(p).reshape(vec_res[p].shape), rtol=1e-12, atol=1e-14)
                 for p in probe)
        if ok:
            return vec_res
    return np.stack([single(p).reshape(tuple(out_shape_tail)) for p in range(P)])


def _bc_values(fn, pts):
    """Dirichlet values value_fn(point) at the BC nodes (fe.py:241-253).  A value function that
    returns torch tensors (set_params closing over a parameter tensor, as in the reference's
    compute_gradients example) gives a torch FP64 tensor that keeps any graph, so the adjoint
    can send lam_b back to the parameter; otherwise a numpy array."""
    v0 = fn(pts[0])
    if torch.is_tensor(v0):
        try:   # one call with the point axis last, checked against per-point calls
            vv = fn(np.moveaxis(pts, 0, -1))
            vv = torch.as_tensor(vv, dtype=torch.float64)
            if vv.numel() == 1:
                vv = vv.reshape(1).expand(len(pts))
            elif vv.shape != (len(pts),):
                raise ValueError
            probe = np.unique(np.linspace(0, len(pts) - 1, min(len(pts), 5)).astype(np.int64))
            val = lambda t: float(torch.as_tensor(t).detach())   # compare values, leave the graph alone
            if not all(abs(val(vv[p]) - val(fn(pts[p]))) <= 1e-12 * (abs(val(vv[p])) + 1.0) for p in probe):
                raise ValueError
            return vv.to(torch.float64)
        except Exception:  # noqa: BLE001 -- per point
            return torch.stack([torch.as_tensor(fn(p), dtype=torch.float64).reshape(()) for p in pts])
    return np.asarray(eval_pointwise(fn, [pts]).reshape(-1), dtype=np.float64)


def eval_location(fn, points):
    n = _nargs(fn)
    if n == 1:
        return eval_pointwise(fn, [points]).astype(bool)
    if n == 2:
        return eval_pointwise(fn, [points, np.arange(len(points))]).astype(bool)
    raise ValueError(f"Wrong number of arguments for location_fn: must be 1 or 2, get {n}")


class FiniteElement:
    """One FE variable on a mesh (fe.py:20-110)."""

    def __init__(self, mesh, vec, dim, ele_type="HEX8", quadrature_rule=None, quadrature_order=None,
                 dirichlet_bc_info=None):
        if dim != 3:
            raise NotImplementedError("only dim=3 problems are built on GB300")
        if quadrature_rule not in (None, "default"):
            raise NotImplementedError("only the default quadrature rule is built")
        default_order, _ = basis.get_elements(ele_type)
        if quadrature_order not in (None, default_order):
            raise NotImplementedError(f"{ele_type}: only quadrature_order={default_order} is built")
        self.mesh = mesh
        self.vec = vec
        self.dim = dim
        self.ele_type = ele_type
        self.quadrature_rule = quadrature_rule
        self.quadrature_order = default_order
        self.dirichlet_bc_info = dirichlet_bc_info
        self.points = np.asarray(mesh.points, dtype=np.float64)
        self.cells = np.asarray(mesh.cells, dtype=np.int64)
        t = basis.element_tables(ele_type)
        self.shape_vals = t["shape_vals"]
        self.shape_grads_ref = t["shape_grads_ref"]
        self.quad_weights = t["quad_weights"]
        self.face_shape_vals = t["face_shape_vals"]
        self.face_shape_grads_ref = t["face_shape_grads_ref"]
        self.face_quad_weights = t["face_quad_weights"]
        self.face_normals = t["face_normals"]
        self.face_inds = t["face_inds"]
        self.elem_id = t["elem_id"]
        self.num_cells = len(self.cells)
        self.num_total_nodes = len(self.points)
        self.num_total_dofs = self.num_total_nodes * vec
        self.num_quads = self.shape_vals.shape[0]
        self.num_nodes = self.shape_vals.shape[1]
        self.num_faces = self.face_shape_vals.shape[0]
        self.num_face_quads = self.face_quad_weights.shape[1]
        if self.cells.shape[1] != self.num_nodes:
            raise ValueError(f"{ele_type} cells need {self.num_nodes} nodes, got {self.cells.shape[1]}")
        self.bc_version = 0
        self.node_inds_list, self.vec_inds_list, self.vals_list = self.Dirichlet_boundary_conditions(dirichlet_bc_info)
        logger.info("Solving a problem with %d cells, %dx%d = %d dofs.", self.num_cells, self.num_total_nodes, vec,
                    self.num_total_dofs)

    # ---- Dirichlet sets (fe.py:220-269) ---------------------------------------
    def Dirichlet_boundary_conditions(self, dirichlet_bc_info):
        node_inds_list, vec_inds_list, vals_list = [], [], []
        if dirichlet_bc_info is not None:
            location_fns, vecs, value_fns = dirichlet_bc_info
            assert len(location_fns) == len(value_fns) and len(value_fns) == len(vecs)
            for i in range(len(location_fns)):
                flags = eval_location(location_fns[i], self.points)
                node_inds = np.argwhere(flags).reshape(-1)
                vec_inds = np.ones_like(node_inds, dtype=np.int32) * vecs[i]
                values = _bc_values(value_fns[i], self.points[node_inds]) if len(node_inds) else np.zeros(0)
                node_inds_list.append(node_inds)
                vec_inds_list.append(vec_inds)
                vals_list.append(values)
        self.bc_version = getattr(self, "bc_version", 0) + 1
        return node_inds_list, vec_inds_list, vals_list

    def update_Dirichlet_boundary_conditions(self, dirichlet_bc_info):
        self.node_inds_list, self.vec_inds_list, self.vals_list = self.Dirichlet_boundary_conditions(dirichlet_bc_info)

    # ---- boundary faces (fe.py:271-322) ----------------------------------------
    def get_boundary_conditions_inds(self, location_fns):
        """(num_selected_faces, 2) arrays of (cell, local face) whose vertices all satisfy location_fn."""
        out = []
        if location_fns is None:
            return out
        cell_face_nodes = self.cells[:, self.face_inds]  # (C, nf, nfv)
        for fn in location_fns:
            flags = eval_location(fn, self.points)
            on = np.all(flags[cell_face_nodes], axis=2)
            out.append(np.argwhere(on))
        return out

    # ---- geometry helpers for post-processing (torch on the device) -------------
    def _dev(self, device):
        pts = torch.as_tensor(self.points, dtype=torch.float64, device=device)
        cells = torch.as_tensor(self.cells, dtype=torch.int64, device=device)
        return pts, cells

    def get_shape_grads(self, device="cuda"):
        """(num_cells, num_quads, num_nodes, dim) physical shape grads and (num_cells, num_quads) JxW."""
        pts, cells = self._dev(device)
        X = pts[cells]
        dN = torch.as_tensor(self.shape_grads_ref, device=device)
        J = torch.einsum("cnd,qne->cqde", X, dN)
        inv = torch.linalg.inv(J)
        grads = torch.einsum("qne,cqed->cqnd", dN, inv)
        jxw = torch.linalg.det(J) * torch.as_tensor(self.quad_weights, device=device)
        return grads, jxw

    def get_face_shape_grads(self, boundary_inds, device="cuda"):
        """fe.py:143-183: face shape grads (F, nfq, nn, dim) and Nanson scale (F, nfq)."""
        pts, cells = self._dev(device)
        b = torch.as_tensor(np.asarray(boundary_inds), dtype=torch.int64, device=device)
        X = pts[cells[b[:, 0]]]
        fg = torch.as_tensor(self.face_shape_grads_ref, device=device)[b[:, 1]]
        n = torch.as_tensor(self.face_normals, device=device)[b[:, 1]]
        J = torch.einsum("fnd,fqne->fqde", X, fg)
        inv = torch.linalg.inv(J)
        grads = torch.einsum("fqne,fqed->fqnd", fg, inv)
        nanson = torch.linalg.norm(torch.einsum("fe,fqed->fqd", n, inv), dim=-1)
        nanson = nanson * torch.linalg.det(J) * torch.as_tensor(self.face_quad_weights, device=device)[b[:, 1]]
        return grads, nanson

    def get_physical_quad_points(self, device="cuda"):
        pts, cells = self._dev(device)
        return torch.einsum("qn,cnd->cqd", torch.as_tensor(self.shape_vals, device=device), pts[cells])

    def get_physical_surface_quad_points(self, boundary_inds, device="cuda"):
        pts, cells = self._dev(device)
        b = torch.as_tensor(np.asarray(boundary_inds), dtype=torch.int64, device=device)
        fv = torch.as_tensor(self.face_shape_vals, device=device)[b[:, 1]]
        return torch.einsum("fqn,fnd->fqd", fv, pts[cells[b[:, 0]]])

    def convert_from_dof_to_quad(self, sol):
        """fe.py:324-341: (num_cells, num_quads, vec)."""
        cells = torch.as_tensor(self.cells, device=sol.device)
        return torch.einsum("cnv,qn->cqv", sol[cells], torch.as_tensor(self.shape_vals, device=sol.device))

    def sol_to_grad(self, sol):
        """fe.py:366-382: (num_cells, num_quads, vec, dim)."""
        grads, _ = self.get_shape_grads(sol.device)
        cells = torch.as_tensor(self.cells, device=sol.device)
        return torch.einsum("cnv,cqnd->cqvd", sol[cells], grads)
