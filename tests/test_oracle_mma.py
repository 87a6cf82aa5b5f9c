"""CPU checks that pin the oracle's MMA and filter restatement (oracle/mma.py) with known answers:
the reference ships no MMA test, so the oracle is checked against a convex problem with an
analytic optimum and against the filter's closed-form weights on a uniform grid."""
import numpy as np
import pytest

from oracle import mma as omma


def _bisect_shift(t, vf):
    """x = clip(t - nu, 0, 1) with mean(x) = vf: the KKT point of min |x - t|^2, mean(x) <= vf."""
    lo, hi = -1.0, 2.0
    for _ in range(200):
        nu = 0.5 * (lo + hi)
        if np.clip(t - nu, 0, 1).mean() > vf:
            lo = nu
        else:
            hi = nu
    return np.clip(t - 0.5 * (lo + hi), 0, 1)


def test_oracle_mma_converges_to_kkt_point():
    """40 MMA iterations on min |x - t|^2 s.t. mean(x)/vf - 1 <= 0, 0 <= x <= 1 (n = 200) reach
    the analytic optimum to 1e-5, and the constraint is active to 1e-6."""
    rng = np.random.default_rng(0)
    n, vf = 200, 0.4
    t = rng.uniform(0.0, 1.2, n)
    x = np.full(n, 0.5)
    xold1, xold2 = x.copy(), x.copy()
    low, upp = np.ones(n), np.ones(n)
    xmin, xmax = np.zeros(n), np.ones(n)
    epoch = 1
    for _ in range(40):
        f0, df0 = np.sum((x - t) ** 2), 2 * (x - t)
        g = np.array([x.mean() / vf - 1.0])
        dg = np.full((1, n), 1.0 / (n * vf))
        xnew, low, upp = omma.mmasub(epoch, x, xold1, xold2, low, upp, xmin, xmax, 0.2, f0, df0, g, dg,
                                     1.0, np.zeros(1), 1e4 * np.ones(1), np.zeros(1))
        xold2, xold1, x = xold1, x, xnew
        epoch += 1
    ref = _bisect_shift(t, vf)
    err = np.abs(x - ref)
    assert np.median(err) < 1e-5 and err.max() < 1e-3
    assert abs(x.mean() / vf - 1.0) < 1e-5


@pytest.mark.parametrize("ele", ["HEX8", "TET4", "TET10"])
def test_oracle_cell_volume_tiles_the_box(ele):
    """The cells of a box mesh tile the box, so sum JxW = Lx Ly Lz: with the interior nodes moved
    for HEX8 (the 2x2x2 rule integrates det J of a trilinear map exactly) and TET4 (det J constant
    per cell), on the affine mesh for TET10; the jittered TET10 sum equals the oracle FE's JxW."""
    import jax_fem_gb300 as jf
    from jax_fem_gb300 import basis
    from oracle import fem as ofem
    nx, ny, nz, Lx, Ly, Lz = 5, 4, 3, 1.0, 0.8, 0.6
    if ele == "HEX8":
        m = jf.box_mesh(nx, ny, nz, Lx, Ly, Lz)
        pts, cells = np.array(m.points), np.asarray(m.cells_dict["hexahedron"])
    else:
        m = jf.box_mesh_tet10(nx, ny, nz, Lx, Ly, Lz)
        pts, cells = np.array(m.points), np.asarray(m.cells_dict["tetra10"])
        if ele == "TET4":
            nv = (nx + 1) * (ny + 1) * (nz + 1)
            pts, cells = pts[:nv], cells[:, :4]
    t = basis.element_tables(ele)
    box = Lx * Ly * Lz
    inner = np.all((pts > 1e-9) & (pts < np.array([Lx, Ly, Lz]) - 1e-9), axis=1)
    moved = pts.copy()
    moved[inner] += np.random.default_rng(3).uniform(-0.2, 0.2, (inner.sum(), 3)) * (Lx / nx)
    V = omma.cell_volume(pts if ele == "TET10" else moved, cells, t["shape_grads_ref"], t["quad_weights"])
    assert abs(V - box) <= 1e-14 * box, (ele, V)
    if ele == "TET10":
        Vm = omma.cell_volume(moved, cells, t["shape_grads_ref"], t["quad_weights"])
        Vo = ofem.OracleFE(moved, cells, 3, ele).JxW.sum()
        assert abs(Vm - Vo) <= 1e-14 * box


def test_oracle_filter_uniform_grid_weights():
    """On a uniform grid of unit cubes rmin = 1.5: an interior cell keeps itself (weight 1.5), its
    6 face neighbours (0.5) and 12 edge neighbours (1.5 - sqrt 2); corner neighbours (sqrt 3 > 1.5)
    carry no weight, so Hs = 1.5 + 3 + 12 (1.5 - sqrt 2)."""
    g = np.stack(np.meshgrid(np.arange(6), np.arange(5), np.arange(4), indexing="ij"), -1).reshape(-1, 3) + 0.5
    H, Hs, rmin = omma.filter_kd_tree(g.astype(float), volume=float(len(g)))
    assert abs(rmin - 1.5) < 1e-14
    i = np.where((g == [2.5, 2.5, 1.5]).all(1))[0][0]
    row = H.toarray()[i]
    w = np.sort(row[row > 0])[::-1]
    expect = np.sort(np.array([1.5] + [0.5] * 6 + [1.5 - np.sqrt(2)] * 12))[::-1]
    np.testing.assert_allclose(w, expect, rtol=0, atol=1e-14)
    assert abs(Hs[i] - expect.sum()) < 1e-13
