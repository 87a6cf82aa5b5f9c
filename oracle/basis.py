"""Element tables for the oracle (restates jax_fem/basis.py:19-250 without basix).

Reference cells are basix's: [0,1]^3 for the hexahedron, the unit simplex for
the tetrahedron.  Node order is meshio's (the mesh's own order); the reference
maps it onto basix order with `re_order` (basis.py:52-84) -- here the shape
functions are written directly in meshio order, which is the same thing.

Quadrature: basix's default rule (basis.py:127-138, 168) is Gauss-Jacobi for
the hexahedron/quadrilateral (order 2 -> 2 points per direction) and
Xiao-Gimbutas for simplices (order 2 -> the symmetric 4-point tetrahedron rule
and 3-point triangle rule).  Point order only matters for per-quadrature-point
parameters and is self-consistent throughout this repository.
"""
import numpy as np

# --- HEX8 -------------------------------------------------------------------
# meshio/VTK corner order: (0,0,0),(1,0,0),(1,1,0),(0,1,0),(0,0,1),(1,0,1),(1,1,1),(0,1,1)
HEX8_VERTS = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0],
                       [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]], dtype=np.float64)

# basix hexahedron facets (vertex lists in basix numbering, basis.py:217), mapped
# through re_order [0,1,3,2,4,5,7,6] (basis.py:53, reorder_inds basis.py:117-124).
# Facet f: z=0, y=0, x=0, x=1, y=1, z=1 with outward normals below.
HEX8_FACE_INDS = np.array([[0, 1, 3, 2], [0, 1, 4, 5], [0, 3, 4, 7],
                           [1, 2, 5, 6], [3, 2, 7, 6], [4, 5, 7, 6]], dtype=np.int64)
HEX8_FACE_NORMALS = np.array([[0, 0, -1], [0, -1, 0], [-1, 0, 0],
                              [1, 0, 0], [0, 1, 0], [0, 0, 1]], dtype=np.float64)


def gauss_1d(m):
    """Gauss-Legendre points/weights mapped to [0,1] (ascending)."""
    x, w = np.polynomial.legendre.leggauss(m)
    return 0.5 * (x + 1.0), 0.5 * w


def hex8_shape(xi):
    """Values (P,8) and reference gradients (P,8,3) of trilinear shape functions."""
    xi = np.atleast_2d(xi)
    V = HEX8_VERTS
    # 1D factors: vertex coord 0 -> (1 - x), 1 -> x
    f = np.where(V[None, :, :] > 0.5, xi[:, None, :], 1.0 - xi[:, None, :])  # (P,8,3)
    df = np.where(V[None, :, :] > 0.5, 1.0, -1.0) * np.ones_like(f)
    vals = f[:, :, 0] * f[:, :, 1] * f[:, :, 2]
    grads = np.stack([df[:, :, 0] * f[:, :, 1] * f[:, :, 2],
                      f[:, :, 0] * df[:, :, 1] * f[:, :, 2],
                      f[:, :, 0] * f[:, :, 1] * df[:, :, 2]], axis=-1)
    return vals, grads


def hex8_quadrature(order=2):
    m = (order + 2) // 2
    p, w = gauss_1d(m)
    pts = np.array([[p[i], p[j], p[k]] for i in range(m) for j in range(m) for k in range(m)])
    wts = np.array([w[i] * w[j] * w[k] for i in range(m) for j in range(m) for k in range(m)])
    return pts, wts


def quad_face_quadrature(order=2):
    m = (order + 2) // 2
    p, w = gauss_1d(m)
    pts = np.array([[p[i], p[j]] for i in range(m) for j in range(m)])
    wts = np.array([w[i] * w[j] for i in range(m) for j in range(m)])
    return pts, wts


# basix vertex lists of the hexahedron facets in basix numbering (used to map face points)
_HEX_BASIX_VERTS = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [1, 1, 0],
                             [0, 0, 1], [1, 0, 1], [0, 1, 1], [1, 1, 1]], dtype=np.float64)
_HEX_BASIX_FACETS = [[0, 1, 2, 3], [0, 1, 4, 5], [0, 2, 4, 6], [1, 3, 5, 7], [2, 3, 6, 7], [4, 5, 6, 7]]


def hex8_face_quadrature(order=2):
    """Face quad points on the reference hex (6, nfq, 3) and weights (6, nfq).

    Restates basis.py:210-238: the facet's P1 quadrilateral map applied to the
    facet vertices; weights scaled by the facet Jacobian (1 on the unit cube).
    """
    pts2, w2 = quad_face_quadrature(order)
    # P1 quadrilateral basis in basix order: (0,0),(1,0),(0,1),(1,1)
    s, t = pts2[:, 0], pts2[:, 1]
    q1 = np.stack([(1 - s) * (1 - t), s * (1 - t), (1 - s) * t, s * t], axis=1)
    fpts, fw = [], []
    for facet in _HEX_BASIX_FACETS:
        v = _HEX_BASIX_VERTS[facet]
        fpts.append(q1 @ v)
        J = np.stack([v[1] - v[0], v[2] - v[0]], axis=1)
        fw.append(w2 * np.linalg.norm(np.cross(J[:, 0], J[:, 1])))
    return np.stack(fpts), np.stack(fw)


# --- TET10 ------------------------------------------------------------------
# meshio order: vertices 0..3, then edge midpoints (0,1),(1,2),(0,2),(0,3),(1,3),(2,3)
TET10_EDGES = np.array([[0, 1], [1, 2], [0, 2], [0, 3], [1, 3], [2, 3]], dtype=np.int64)
# basix tetrahedron facets: facet i is opposite vertex i (basis.py:217)
TET_FACE_INDS = np.array([[1, 2, 3], [0, 2, 3], [0, 1, 3], [0, 1, 2]], dtype=np.int64)
TET_FACE_NORMALS = np.array([[1, 1, 1], [-1, 0, 0], [0, -1, 0], [0, 0, -1]], dtype=np.float64)
TET_FACE_NORMALS[0] /= np.sqrt(3.0)
TET_VERTS = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], dtype=np.float64)


def tet10_shape(xi):
    xi = np.atleast_2d(xi)
    L = np.stack([1 - xi.sum(1), xi[:, 0], xi[:, 1], xi[:, 2]], axis=1)  # barycentric (P,4)
    dL = np.array([[-1, -1, -1], [1, 0, 0], [0, 1, 0], [0, 0, 1]], dtype=np.float64)  # (4,3)
    vals = np.zeros((len(xi), 10))
    grads = np.zeros((len(xi), 10, 3))
    for i in range(4):
        vals[:, i] = L[:, i] * (2 * L[:, i] - 1)
        grads[:, i, :] = (4 * L[:, i] - 1)[:, None] * dL[i][None, :]
    for e, (a, b) in enumerate(TET10_EDGES):
        vals[:, 4 + e] = 4 * L[:, a] * L[:, b]
        grads[:, 4 + e, :] = 4 * (L[:, b][:, None] * dL[a][None, :] + L[:, a][:, None] * dL[b][None, :])
    return vals, grads


def tet4_shape(xi):
    """Linear tetrahedron (basis.py:55-60, degree 1): barycentric shape functions."""
    xi = np.atleast_2d(xi)
    vals = np.stack([1 - xi.sum(1), xi[:, 0], xi[:, 1], xi[:, 2]], axis=1)
    dL = np.array([[-1, -1, -1], [1, 0, 0], [0, 1, 0], [0, 0, 1]], dtype=np.float64)
    return vals, np.broadcast_to(dL, (len(xi), 4, 3)).copy()


def tet_quadrature(order=2):
    if order == 2:
        a, b = 0.5854101966249685, 0.1381966011250105
        pts = np.array([[b, b, b], [a, b, b], [b, a, b], [b, b, a]])
        return pts, np.full(4, 1.0 / 24.0)
    if order in (0, 1):
        return np.array([[0.25, 0.25, 0.25]]), np.array([1.0 / 6.0])
    raise NotImplementedError(f"tet quadrature order {order}")


def tri_quadrature(order=2):
    if order == 2:
        return np.array([[1 / 6, 1 / 6], [2 / 3, 1 / 6], [1 / 6, 2 / 3]]), np.full(3, 1.0 / 6.0)
    if order in (0, 1):
        return np.array([[1 / 3, 1 / 3]]), np.array([0.5])
    raise NotImplementedError(f"triangle quadrature order {order}")


def tet_face_quadrature(order=2):
    pts2, w2 = tri_quadrature(order)
    p1 = np.stack([1 - pts2.sum(1), pts2[:, 0], pts2[:, 1]], axis=1)
    fpts, fw = [], []
    for facet in TET_FACE_INDS:
        v = TET_VERTS[facet]
        fpts.append(p1 @ v)
        J = np.stack([v[1] - v[0], v[2] - v[0]], axis=1)
        fw.append(w2 * np.linalg.norm(np.cross(J[:, 0], J[:, 1])))
    return np.stack(fpts), np.stack(fw)


def element_tables(ele_type, quadrature_order=None):
    """Return dict with shape_vals (nq,nn), shape_grads_ref (nq,nn,3), quad_weights (nq,),
    face_shape_vals (nf,nfq,nn), face_shape_grads_ref (nf,nfq,nn,3), face_quad_weights (nf,nfq),
    face_normals (nf,3), face_inds (nf,nfv).  Mirrors basis.py:141-250."""
    if ele_type == "HEX8":
        order = 2 if quadrature_order is None else quadrature_order
        pts, w = hex8_quadrature(order)
        vals, grads = hex8_shape(pts)
        fpts, fw = hex8_face_quadrature(order)
        nf, nfq, _ = fpts.shape
        fv, fg = hex8_shape(fpts.reshape(-1, 3))
        face_inds, normals = HEX8_FACE_INDS, HEX8_FACE_NORMALS
    elif ele_type == "TET10":
        order = 2 if quadrature_order is None else quadrature_order
        pts, w = tet_quadrature(order)
        vals, grads = tet10_shape(pts)
        fpts, fw = tet_face_quadrature(order)
        nf, nfq, _ = fpts.shape
        fv, fg = tet10_shape(fpts.reshape(-1, 3))
        face_inds, normals = TET_FACE_INDS, TET_FACE_NORMALS
    elif ele_type == "TET4":
        order = 0 if quadrature_order is None else quadrature_order   # basis.py:59, one point
        pts, w = tet_quadrature(order)
        vals, grads = tet4_shape(pts)
        fpts, fw = tet_face_quadrature(order)
        nf, nfq, _ = fpts.shape
        fv, fg = tet4_shape(fpts.reshape(-1, 3))
        face_inds, normals = TET_FACE_INDS, TET_FACE_NORMALS
    else:
        raise NotImplementedError(ele_type)
    nn = vals.shape[1]
    return dict(shape_vals=vals, shape_grads_ref=grads, quad_weights=w,
                face_shape_vals=fv.reshape(nf, nfq, nn), face_shape_grads_ref=fg.reshape(nf, nfq, nn, 3),
                face_quad_weights=fw, face_normals=normals, face_inds=face_inds)
