"""Topology-optimisation update on the GPU, mirroring jax_fem/mma.py.

``optimize`` runs the reference's loop (mma.py:408-528): objective and constraint handles, the
sensitivity filter, and one MMA update per iteration.  The filter
(``compute_filter_kd_tree``, mma.py:27-57) is built on the GPU by ``fem_filter_build`` (a radius
search on a uniform grid of bins, which gives the k-d tree's weights: only neighbours closer than
rmin carry weight).  The MMA update (``MMA.mmasub``, mma.py:113-206, and ``subsolv``,
mma.py:209-405) runs as ``fem_mma_update``: per-variable work in CUDA kernels, the m-sized dual
variables on the host.  Arrays are torch tensors on the GPU (float64).
"""
import ctypes as C
import time

import numpy as np
import torch

from . import _lib
from ._lib import call, ptr
from .logger import logger

density_filtering = False       # mma.py:24
sensitivity_filtering = True    # mma.py:25
NUM_NBS = 20                    # mma.py:45


def _stream():
    return _lib.stream_handle()


class Filter:
    """Device filter matrix: nnb slots per row (cols -1 when unused), weights and row sums."""

    def __init__(self, cols, vals, hs, rmin):
        self.cols, self.vals, self.hs, self.rmin = cols, vals, hs, rmin
        self.n, self.nnb = cols.shape

    def apply(self, rows, rho=None, mode=0):
        """mode 0: H (rho g / max(1e-3, rho) / Hs) per row g; mode 1: H g / Hs."""
        g = torch.as_tensor(rows, dtype=torch.float64, device=self.cols.device).reshape(-1, self.n).contiguous()
        out = torch.empty_like(g)
        r = None if rho is None else torch.as_tensor(rho, dtype=torch.float64,
                                                     device=self.cols.device).reshape(-1).contiguous()
        call("fem_filter_apply", self.n, self.nnb, ptr(self.cols), ptr(self.vals), ptr(self.hs), ptr(r), ptr(g),
             g.shape[0], mode, ptr(out), _stream())
        return out


def _cell_volume(fe, chunk=1 << 22):
    """Sum of JxW over all cells (fe.JxW.sum() in mma.py:36): JxW = det J w_q by fem_quad_points
    on the device, in chunks of cells whose sums are added in order."""
    dev = torch.device("cuda", torch.cuda.current_device())
    coords = torch.as_tensor(np.asarray(fe.points), dtype=torch.float64, device=dev).contiguous()
    conn = torch.as_tensor(np.asarray(fe.cells), dtype=torch.int32, device=dev).contiguous()
    jxw = torch.empty(min(chunk, max(fe.num_cells, 1)) * fe.num_quads, dtype=torch.float64, device=dev)
    V = torch.zeros((), dtype=torch.float64, device=dev)
    for c0 in range(0, fe.num_cells, chunk):
        nc = min(chunk, fe.num_cells - c0)
        mesh = _lib.FemMesh(fe.elem_id, 1, fe.num_total_nodes, nc, coords.data_ptr(), conn[c0].data_ptr(), None,
                            None)
        call("fem_quad_points", C.byref(mesh), None, ptr(jxw), _stream())
        V += jxw[:nc * fe.num_quads].sum()
    return float(V)


def compute_filter_kd_tree(fe, num_nbs=NUM_NBS):
    """mma.py:27-57: returns (H, Hs) for the cells fe.flex_inds (all cells when unset), with
    rmin = 1.5 (V / num_cells)^(1/dim)."""
    flex = getattr(fe, "flex_inds", None)
    flex = np.arange(fe.num_cells) if flex is None else np.asarray(flex)
    centroids = np.mean(np.take(np.asarray(fe.points), np.asarray(fe.cells), axis=0), axis=1)[flex]
    V = _cell_volume(fe)
    rmin = 1.5 * (V / fe.num_cells) ** (1.0 / fe.dim)
    n = len(flex)
    dev = torch.device("cuda", torch.cuda.current_device())
    c = torch.as_tensor(np.ascontiguousarray(centroids), dtype=torch.float64, device=dev)
    cols = torch.empty(n, num_nbs, dtype=torch.int32, device=dev)
    vals = torch.empty(n, num_nbs, dtype=torch.float64, device=dev)
    hs = torch.empty(n, dtype=torch.float64, device=dev)
    nb = C.c_size_t()
    call("fem_filter_workspace", n, C.byref(nb))
    ws = torch.empty(nb.value, dtype=torch.uint8, device=dev)
    call("fem_filter_build", n, ptr(c), float(rmin), num_nbs, ptr(cols), ptr(vals), ptr(hs), ptr(ws), nb.value,
         _stream())
    H = Filter(cols, vals, hs, rmin)
    return H, hs


def applySensitivityFilter(ft, rho, dJ, dvc):
    """mma.py:59-62."""
    H = ft["H"]
    rho_f = torch.as_tensor(rho, dtype=torch.float64).reshape(-1)
    dJf = H.apply(torch.as_tensor(dJ).reshape(1, -1), rho_f, 0).reshape(dJ.shape)
    dvcf = H.apply(torch.as_tensor(dvc).reshape(dvc.shape[0], -1), rho_f, 0).reshape(dvc.shape)
    return dJf, dvcf


def applyDensityFilter(ft, rho):
    """mma.py:64-66."""
    return ft["H"].apply(torch.as_tensor(rho).reshape(1, -1), None, 1).reshape(rho.shape)


class MMA:
    """The reference's MMA driver object (mma.py:68-206): same setters and getters; ``mmasub``
    runs on the GPU.  Vectors are (n, 1) torch tensors; m-sized scalars may be numpy or torch."""

    def __init__(self):
        self.epoch = 0
        self.newton_steps = 0

    def resetMMACounter(self):
        self.epoch = 0

    def registerMMAIter(self, xval, xold1, xold2):
        self.epoch += 1
        self.xval, self.xold1, self.xold2 = xval, xold1, xold2

    def setNumConstraints(self, numConstraints):
        self.numConstraints = numConstraints

    def setNumDesignVariables(self, numDesVar):
        self.numDesignVariables = numDesVar

    def setMinandMaxBoundsForDesignVariables(self, xmin, xmax):
        self.xmin, self.xmax = xmin, xmax

    def setObjectiveWithGradient(self, obj, objGrad):
        self.objective, self.objectiveGradient = obj, objGrad

    def setConstraintWithGradient(self, cons, consGrad):
        self.constraint, self.consGrad = cons, consGrad

    def setScalingParams(self, zconst, zscale, ylinscale, yquadscale):
        self.zconst, self.zscale, self.ylinscale, self.yquadscale = zconst, zscale, ylinscale, yquadscale

    def setMoveLimit(self, movelim):
        self.moveLimit = movelim

    def setLowerAndUpperAsymptotes(self, low, upp):
        self.lowAsymp, self.upAsymp = low, upp

    def getOptimalValues(self):
        return self.xmma, None, None

    def getAsymptoteValues(self):
        return self.lowAsymp, self.upAsymp

    def mmasub(self, xval):
        m, n = self.numConstraints, self.numDesignVariables
        dev = torch.device("cuda", torch.cuda.current_device())
        d64 = lambda t: torch.as_tensor(t, dtype=torch.float64, device=dev).reshape(-1).contiguous()
        h64 = lambda t: np.ascontiguousarray(np.asarray(
            t.detach().cpu().numpy() if torch.is_tensor(t) else t, dtype=np.float64).reshape(-1))
        x = d64(xval)
        low, upp = d64(self.lowAsymp).clone(), d64(self.upAsymp).clone()
        dfdx = d64(self.consGrad)
        fval, a, c, d = (h64(v) for v in (self.constraint, self.zscale, self.ylinscale, self.yquadscale))
        key = (n, m)
        if getattr(self, "_ws_key", None) != key:
            nb = C.c_size_t()
            call("fem_mma_workspace", n, m, C.byref(nb))
            self._ws = torch.empty(nb.value, dtype=torch.uint8, device=dev)
            self._ws_key = key
        xmma = torch.empty_like(x)
        steps = C.c_int32()
        fp = lambda arr: arr.ctypes.data_as(C.POINTER(C.c_double))
        call("fem_mma_update", n, m, int(self.epoch), ptr(x), ptr(d64(self.xold1)), ptr(d64(self.xold2)), ptr(low),
             ptr(upp), ptr(d64(self.xmin)), ptr(d64(self.xmax)), float(self.moveLimit),
             ptr(d64(self.objectiveGradient)), fp(fval), ptr(dfdx), float(np.asarray(self.zconst).reshape(-1)[0]),
             fp(a), fp(c), fp(d), ptr(xmma), ptr(self._ws), self._ws.numel(), C.byref(steps), _stream())
        self.newton_steps = steps.value
        self.xmma = xmma.reshape(-1, 1)
        self.lowAsymp, self.upAsymp = low.reshape(-1, 1), upp.reshape(-1, 1)


def optimize(fe, rho_ini, optimizationParams, objectiveHandle, consHandle, numConstraints):
    """mma.py:408-528: TO by MMA with the sensitivity filter.  objectiveHandle(rho) -> (J, dJ),
    consHandle(rho, iter) -> (vc (m,), dvc (m, ...)); tensors or arrays; returns rho (torch, GPU)."""
    H, Hs = compute_filter_kd_tree(fe)
    ft = {"H": H, "Hs": Hs}
    dev = H.cols.device
    rho = torch.as_tensor(np.asarray(rho_ini) if not torch.is_tensor(rho_ini) else rho_ini,
                          dtype=torch.float64, device=dev)
    m = numConstraints
    n = rho.numel()
    mma = MMA()
    mma.setNumConstraints(m)
    mma.setNumDesignVariables(n)
    mma.setMinandMaxBoundsForDesignVariables(torch.zeros(n, 1, dtype=torch.float64, device=dev),
                                             torch.ones(n, 1, dtype=torch.float64, device=dev))
    xval = rho.reshape(-1, 1).clone()
    xold1, xold2 = xval.clone(), xval.clone()
    mma.registerMMAIter(xval, xold1, xold2)
    mma.setLowerAndUpperAsymptotes(torch.ones(n, 1, dtype=torch.float64, device=dev),
                                   torch.ones(n, 1, dtype=torch.float64, device=dev))
    mma.setScalingParams(1.0, np.zeros(m), 10000 * np.ones(m), np.zeros(m))
    mma.setMoveLimit(optimizationParams["movelimit"])
    loop = 0
    while loop < optimizationParams["maxIters"]:
        loop += 1
        logger.info("MMA solver...")
        rho_physical = applyDensityFilter(ft, rho) if density_filtering else rho
        J, dJ = objectiveHandle(rho_physical)
        vc, dvc = consHandle(rho_physical, loop)
        dJ = torch.as_tensor(dJ, dtype=torch.float64, device=dev).reshape(rho.shape)
        dvc = torch.as_tensor(dvc, dtype=torch.float64, device=dev).reshape((m,) + tuple(rho.shape))
        if sensitivity_filtering:
            dJ, dvc = applySensitivityFilter(ft, rho, dJ, dvc)
        t0 = time.time()
        mma.setObjectiveWithGradient(J, dJ.reshape(-1, 1))
        mma.setConstraintWithGradient(np.asarray(torch.as_tensor(vc).detach().cpu()).reshape(-1),
                                      dvc.reshape(m, -1))
        mma.mmasub(xval)
        xmma, _, _ = mma.getOptimalValues()
        xold2 = xold1.clone()
        xold1 = xval.clone()
        xval = xmma.clone()
        mma.registerMMAIter(xval, xold1, xold2)
        rho = xval.reshape(rho.shape)
        logger.info(f"MMA took {time.time() - t0} [s]")
        logger.info(f"Iter {loop:d}; J {float(J):.5f}; constraint {np.asarray(torch.as_tensor(vc).cpu())}\n\n\n")
    return rho
