"""CPU checks that pin the oracle's MMA and filter restatement (oracle/mma.py) with known answers:
the reference ships no MMA test, so the oracle is checked against a convex problem with an
analytic optimum and against the filter's closed-form weights on a uniform grid."""
import numpy as np

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
