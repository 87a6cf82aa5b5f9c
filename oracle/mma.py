"""CPU restatement of jax-fem's MMA update and sensitivity filter (test infrastructure only).

Follows jax_fem/mma.py: the asymptote / move-limit / approximation set-up of ``MMA.mmasub``
(mma.py:113-206), the primal-dual interior-point ``subsolv`` (mma.py:209-405), the k-d tree
filter ``compute_filter_kd_tree`` (mma.py:27-57) and ``applySensitivityFilter`` (mma.py:59-62).
Vectors are flat numpy arrays: x-like (n,), constraint-like (m,), P/Q/dfdx (m, n).  Used by the
tests to check the GPU optimizer; never on the product path.
"""
import numpy as np
import scipy.sparse
import scipy.spatial

EPSIMIN = 1e-7      # mma.py:126
RAA0 = 1e-5         # mma.py:127
ALBEFA = 0.1        # mma.py:128
ASYINIT = 0.5       # mma.py:129
ASYINCR = 1.2       # mma.py:130
ASYDECR = 0.7       # mma.py:131


def asymptotes(it, xval, xold1, xold2, low, upp, xmin, xmax):
    """mma.py:136-155: initial asymptotes for it <= 2, then expanded / contracted by the sign
    of the last two moves and clamped to [x -/+ 10 (xmax-xmin), x -/+ 0.01 (xmax-xmin)]."""
    span = xmax - xmin
    if it <= 2:
        return xval - ASYINIT * span, xval + ASYINIT * span
    trend = (xval - xold1) * (xold1 - xold2)
    f = np.where(trend > 0, ASYINCR, np.where(trend < 0, ASYDECR, 1.0))
    lo = xval - f * (xold1 - low)
    up = xval + f * (upp - xold1)
    lo = np.minimum(np.maximum(lo, xval - 10 * span), xval - 0.01 * span)
    up = np.maximum(np.minimum(up, xval + 10 * span), xval + 0.01 * span)
    return lo, up


def approximation(xval, low, upp, xmin, xmax, move, df0dx, fval, dfdx):
    """mma.py:157-203: move-limited bounds alfa/beta and the convex approximation p0, q0, P, Q, b."""
    alfa = np.maximum(np.maximum(low + ALBEFA * (xval - low), xval - move * (xmax - xmin)), xmin)
    beta = np.minimum(np.minimum(upp - ALBEFA * (upp - xval), xval + move * (xmax - xmin)), xmax)
    inv_span = 1.0 / np.maximum(xmax - xmin, 1e-5)
    ux2 = (upp - xval) ** 2
    xl2 = (xval - low) ** 2
    pos, neg = np.maximum(df0dx, 0.0), np.maximum(-df0dx, 0.0)
    reg0 = 0.001 * (pos + neg) + RAA0 * inv_span
    p0 = (pos + reg0) * ux2
    q0 = (neg + reg0) * xl2
    Pp, Qn = np.maximum(dfdx, 0.0), np.maximum(-dfdx, 0.0)
    reg = 0.001 * (Pp + Qn) + RAA0 * inv_span[None, :]
    P = (Pp + reg) * ux2[None, :]
    Q = (Qn + reg) * xl2[None, :]
    b = P @ (1.0 / (upp - xval)) + Q @ (1.0 / (xval - low)) - fval
    return alfa, beta, p0, q0, P, Q, b


def _residual(st, epsi, low, upp, alfa, beta, p0, q0, P, Q, a0, a, b, c, d):
    x, y, z, lam, xsi, eta, mu, zet, s = st
    ux1, xl1 = upp - x, x - low
    plam = p0 + P.T @ lam
    qlam = q0 + Q.T @ lam
    gvec = P @ (1.0 / ux1) + Q @ (1.0 / xl1)
    parts = [plam / ux1 ** 2 - qlam / xl1 ** 2 - xsi + eta,      # rex
             c + d * y - mu - lam,                                # rey
             np.atleast_1d(a0 - zet - a @ lam),                   # rez
             gvec - a * z - y + s - b,                            # relam
             xsi * (x - alfa) - epsi,                             # rexsi
             eta * (beta - x) - epsi,                             # reeta
             mu * y - epsi,                                       # remu
             np.atleast_1d(zet * z - epsi),                       # rezet
             lam * s - epsi]                                      # res
    r = np.concatenate(parts)
    return np.sqrt(r @ r), np.abs(r).max()


def subsolv(m, n, low, upp, alfa, beta, p0, q0, P, Q, a0, a, b, c, d):
    """mma.py:209-405: the MMA subproblem by a primal-dual Newton method with a decreasing
    barrier epsi (x0.1 from 1 to 1e-7), at most 200 Newton steps per level and a halving line
    search on the residual norm (at most 50 halvings)."""
    epsi = 1.0
    x = 0.5 * (alfa + beta)
    y = np.ones(m)
    z = 1.0
    lam = np.ones(m)
    xsi = np.maximum(1.0 / (x - alfa), 1.0)
    eta = np.maximum(1.0 / (beta - x), 1.0)
    mu = np.maximum(np.ones(m), 0.5 * c)
    zet = 1.0
    s = np.ones(m)
    args = (low, upp, alfa, beta, p0, q0, P, Q, a0, a, b, c, d)
    while epsi > EPSIMIN:
        st = (x, y, z, lam, xsi, eta, mu, zet, s)
        rnorm, rmax = _residual(st, epsi, *args)
        newton = 0
        while rmax > 0.9 * epsi and newton < 200:
            newton += 1
            ux1, xl1 = upp - x, x - low
            plam = p0 + P.T @ lam
            qlam = q0 + Q.T @ lam
            gvec = P @ (1.0 / ux1) + Q @ (1.0 / xl1)
            GG = P / ux1 ** 2 - Q / xl1 ** 2
            dpsidx = plam / ux1 ** 2 - qlam / xl1 ** 2
            delx = dpsidx - epsi / (x - alfa) + epsi / (beta - x)
            dely = c + d * y - lam - epsi / y
            delz = a0 - a @ lam - epsi / z
            dellam = gvec - a * z - y - b + epsi / lam
            diagx = 2.0 * (plam / ux1 ** 3 + qlam / xl1 ** 3) + xsi / (x - alfa) + eta / (beta - x)
            diagy = d + mu / y
            diaglamyi = s / lam + 1.0 / diagy
            if m < n:
                blam = dellam + dely / diagy - GG @ (delx / diagx)
                Alam = np.diag(diaglamyi) + (GG / diagx) @ GG.T
                AA = np.zeros((m + 1, m + 1))
                AA[:m, :m] = Alam
                AA[:m, m] = a
                AA[m, :m] = a
                AA[m, m] = -zet / z
                sol = np.linalg.solve(AA, np.concatenate([blam, [delz]]))
                dlam, dz = sol[:m], sol[m]
                dx = -delx / diagx - (GG.T @ dlam) / diagx
            else:
                dellamyi = dellam + dely / diagy
                Axx = np.diag(diagx) + (GG.T / diaglamyi) @ GG
                azz = zet / z + a @ (a / diaglamyi)
                axz = -GG.T @ (a / diaglamyi)
                bx = delx + GG.T @ (dellamyi / diaglamyi)
                bz = delz - a @ (dellamyi / diaglamyi)
                AA = np.zeros((n + 1, n + 1))
                AA[:n, :n] = Axx
                AA[:n, n] = axz
                AA[n, :n] = axz
                AA[n, n] = azz
                sol = np.linalg.solve(AA, -np.concatenate([bx, [bz]]))
                dx, dz = sol[:n], sol[n]
                dlam = GG @ dx / diaglamyi - dz * (a / diaglamyi) + dellamyi / diaglamyi
            dy = -dely / diagy + dlam / diagy
            dxsi = -xsi + epsi / (x - alfa) - xsi * dx / (x - alfa)
            deta = -eta + epsi / (beta - x) + eta * dx / (beta - x)
            dmu = -mu + epsi / y - mu * dy / y
            dzet = -zet + epsi / z - zet * dz / z
            ds = -s + epsi / lam - s * dlam / lam
            xx = np.concatenate([y, [z], lam, xsi, eta, mu, [zet], s])
            dxx = np.concatenate([dy, [dz], dlam, dxsi, deta, dmu, [dzet], ds])
            stm = max(np.max(-1.01 * dxx / xx), np.max(-1.01 * dx / (x - alfa)),
                      np.max(1.01 * dx / (beta - x)), 1.0)
            steg = 1.0 / stm
            old = (x, y, z, lam, xsi, eta, mu, zet, s)
            step = (dx, dy, dz, dlam, dxsi, deta, dmu, dzet, ds)
            resinew = 2 * rnorm
            tries = 0
            while resinew > rnorm and tries < 50:
                tries += 1
                x, y, z, lam, xsi, eta, mu, zet, s = (o + steg * dd for o, dd in zip(old, step))
                resinew, rmax = _residual((x, y, z, lam, xsi, eta, mu, zet, s), epsi, *args)
                steg = steg / 2
            rnorm = resinew
            steg = 2 * steg
        epsi = 0.1 * epsi
    return x, y, z, lam, xsi, eta, mu, zet, s


def mmasub(it, xval, xold1, xold2, low, upp, xmin, xmax, move, f0val, df0dx, fval, dfdx, a0, a, c, d):
    """One MMA update (mma.py:113-206): returns (xmma, low, upp)."""
    m, n = dfdx.shape
    low, upp = asymptotes(it, xval, xold1, xold2, low, upp, xmin, xmax)
    alfa, beta, p0, q0, P, Q, b = approximation(xval, low, upp, xmin, xmax, move, df0dx, fval, dfdx)
    x = subsolv(m, n, low, upp, alfa, beta, p0, q0, P, Q, a0, a, b, c, d)[0]
    return x, low, upp


def cell_volume(points, cells, shape_grads_ref, quad_weights, chunk=1 << 18):
    """fe.JxW.sum() (mma.py:36), with JxW = det(J) w_q and J = sum_a x_a (x) dN_a/dxi (fe.py:112-141),
    per chunk of cells: J by one contraction over the cell's nodes, det J by the cofactor expansion
    along its first row."""
    dN = np.asarray(shape_grads_ref, dtype=np.float64)           # (nq, nn, 3)
    w = np.asarray(quad_weights, dtype=np.float64)
    V = 0.0
    for c0 in range(0, len(cells), chunk):
        X = np.asarray(points, dtype=np.float64)[np.asarray(cells)[c0:c0 + chunk]]   # (c, nn, 3)
        J = np.tensordot(X, dN, axes=([1], [1])).transpose(0, 2, 1, 3)               # (c, nq, 3, 3)
        det = (J[..., 0, 0] * (J[..., 1, 1] * J[..., 2, 2] - J[..., 1, 2] * J[..., 2, 1])
               - J[..., 0, 1] * (J[..., 1, 0] * J[..., 2, 2] - J[..., 1, 2] * J[..., 2, 0])
               + J[..., 0, 2] * (J[..., 1, 0] * J[..., 2, 1] - J[..., 1, 1] * J[..., 2, 0]))
        V += float((det * w).sum())
    return V


def filter_kd_tree(centroids, volume, dim=3, num_nbs=20):
    """mma.py:27-57: rmin = 1.5 (V / n_cells)^(1/dim); H[i, j] = max(rmin - |c_i - c_j|, 0) over
    the num_nbs nearest centroids of c_i; Hs = row sums.  Returns (H as scipy CSR, Hs)."""
    n = len(centroids)
    rmin = 1.5 * (volume / n) ** (1.0 / dim)
    tree = scipy.spatial.KDTree(centroids)
    dd, ii = tree.query(centroids, num_nbs)
    vals = np.where(rmin - dd > 0.0, rmin - dd, 0.0)
    H = scipy.sparse.csr_array((vals.reshape(-1), (np.repeat(np.arange(n), num_nbs), ii.reshape(-1))), shape=(n, n))
    return H, np.asarray(H.sum(1)).reshape(-1), rmin


def sensitivity_filter(H, Hs, rho, dJ, dvc):
    """mma.py:59-62: dJ <- H (rho dJ / max(1e-3, rho) / Hs), the same for each constraint row."""
    w = rho / np.maximum(1e-3, rho) / Hs
    return H @ (w * dJ), np.stack([H @ (w * g) for g in dvc])
