"""Patch test of the oracle's elements (HEX8, TET10, TET4: shape functions, quadrature, geometry):
under an affine displacement the stress is constant, so the internal force at every interior node
vanishes and the forces sum to zero per component (partition of unity), on distorted meshes too.
Pins the oracle's element layer (jax_fem/basis.py, fe.py:112-141, problem.py:189-214) on the CPU."""
import numpy as np
import pytest
import torch

from oracle import fem as ofem, materials as omat


def _mesh(ele, n, rng):
    import jax_fem_gb300 as jf
    if ele == "HEX8":
        pts, cells = ofem.box_mesh(n, n, n, 1.0, 1.0, 1.0)
        nv = len(pts)
    else:
        m = jf.box_mesh_tet10(n, n, n, 1.0, 1.0, 1.0)
        pts, cells = m.points.copy(), m.cells_dict["tetra10"].copy()
        nv = (n + 1) ** 3
        if ele == "TET4":
            cells = cells[:, :4]
            pts = pts[:nv]
    pts = pts.copy()
    inner = np.all((pts[:nv] > 1e-9) & (pts[:nv] < 1 - 1e-9), axis=1)
    pts[:nv][inner] += 0.15 / n * rng.uniform(-1, 1, (int(inner.sum()), 3))   # distort interior vertices
    if ele == "TET10":   # keep edges straight: mid-edge nodes at the moved vertices' midpoints
        for a, b, m_ in ((0, 1, 4), (1, 2, 5), (0, 2, 6), (0, 3, 7), (1, 3, 8), (2, 3, 9)):
            pts[cells[:, m_]] = 0.5 * (pts[cells[:, a]] + pts[cells[:, b]])
    return pts, cells


@pytest.mark.parametrize("ele", ["HEX8", "TET10", "TET4"])
def test_patch_affine_displacement(ele):
    rng = np.random.default_rng(11)
    pts, cells = _mesh(ele, 3, rng)
    prob = ofem.OracleProblem(pts, cells, 3, ele_type=ele, tensor_map=omat.linear_elastic(10.0, 0.3))
    A = 0.01 * rng.standard_normal((3, 3))
    u = (pts @ A.T + np.array([0.1, -0.2, 0.3])).reshape(-1)
    r = prob.compute_residual(torch.from_numpy(u)).numpy().reshape(-1, 3)
    used = np.zeros(len(pts), dtype=bool)
    used[np.unique(cells)] = True
    interior = np.all((pts > 1e-9) & (pts < 1 - 1e-9), axis=1) & used
    scale = np.abs(r).max()
    assert scale > 0 and interior.sum() > 0
    assert np.abs(r[interior]).max() <= 1e-12 * scale
    assert np.abs(r.sum(axis=0)).max() <= 1e-12 * scale
