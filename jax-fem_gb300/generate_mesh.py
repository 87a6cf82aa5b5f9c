"""Mesh container and structured mesh generators.

Mesh mirrors jax_fem/generate_mesh.py:13-55; box_mesh restates the structured
HEX8 generator of jax_fem/generate_mesh.py:151-189 (same node and cell order);
box_mesh_tet10 builds the Kuhn (6 tetrahedra per cube, all sharing the cube's
main diagonal) second-order tetrahedral mesh used for the TET10 workload.
gmsh-based generators of the reference are not part of this build.
"""
import numpy as np


class Mesh:
    """points (num_total_nodes, dim), cells (num_cells, num_nodes) in meshio order."""

    def __init__(self, points, cells, ele_type=None):
        self.points = np.asarray(points, dtype=np.float64)
        self.cells = np.asarray(cells)
        self.ele_type = ele_type


class _MeshioLike:
    """Stand-in for the meshio.Mesh the reference generators return."""

    def __init__(self, points, cells_dict):
        self.points = points
        self.cells_dict = cells_dict


def get_meshio_cell_type(ele_type):
    """jax_fem/generate_mesh.py:83-117 (types built here)."""
    table = {"HEX8": "hexahedron", "TET4": "tetra", "TET10": "tetra10"}
    if ele_type not in table:
        raise NotImplementedError(ele_type)
    return table[ele_type]


def box_mesh(Nx, Ny, Nz, domain_x, domain_y, domain_z):
    """Structured HEX8 mesh of [0,Lx]x[0,Ly]x[0,Lz] with Nx*Ny*Nz cells."""
    x = np.linspace(0, domain_x, Nx + 1)
    y = np.linspace(0, domain_y, Ny + 1)
    z = np.linspace(0, domain_z, Nz + 1)
    xv, yv, zv = np.meshgrid(x, y, z, indexing="ij")
    points = np.stack((xv, yv, zv), axis=3).reshape(-1, 3)
    ind = np.arange(len(points), dtype=np.int64).reshape(Nx + 1, Ny + 1, Nz + 1)
    corners = [ind[:-1, :-1, :-1], ind[1:, :-1, :-1], ind[1:, 1:, :-1], ind[:-1, 1:, :-1],
               ind[:-1, :-1, 1:], ind[1:, :-1, 1:], ind[1:, 1:, 1:], ind[:-1, 1:, 1:]]
    cells = np.stack(corners, axis=3).reshape(-1, 8)
    return _MeshioLike(points, {"hexahedron": cells})


def box_mesh_tet10(Nx, Ny, Nz, domain_x, domain_y, domain_z):
    """Kuhn-split TET10 mesh: each grid cube -> 6 tets sharing the (0,0,0)-(1,1,1) diagonal.

    Vertices are the grid points; edge midpoints are numbered after them
    (unique per edge).  Node order per cell is meshio's TET10 order."""
    gx, gy, gz = Nx + 1, Ny + 1, Nz + 1
    x = np.linspace(0, domain_x, gx)
    y = np.linspace(0, domain_y, gy)
    z = np.linspace(0, domain_z, gz)
    xv, yv, zv = np.meshgrid(x, y, z, indexing="ij")
    verts = np.stack((xv, yv, zv), axis=3).reshape(-1, 3)
    vid = np.arange(gx * gy * gz, dtype=np.int64).reshape(gx, gy, gz)
    # cube corner offsets in (i,j,k); Kuhn tets follow the 6 monotone paths 000 -> 111
    paths = [(0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0)]
    i, j, k = np.meshgrid(np.arange(Nx), np.arange(Ny), np.arange(Nz), indexing="ij")
    i, j, k = i.reshape(-1), j.reshape(-1), k.reshape(-1)
    tets = []
    for p in paths:
        c = np.zeros((len(i), 3), dtype=np.int64)
        pts = [vid[i, j, k]]
        for axis in p:
            c[:, axis] += 1
            pts.append(vid[i + c[:, 0], j + c[:, 1], k + c[:, 2]])
        tets.append(np.stack(pts, axis=1))
    tets = np.stack(tets, axis=1).reshape(-1, 4)
    # orient positively
    P = verts[tets]
    vol = np.einsum("ij,ij->i", np.cross(P[:, 1] - P[:, 0], P[:, 2] - P[:, 0]), P[:, 3] - P[:, 0])
    neg = vol < 0
    tets[neg] = tets[neg][:, [0, 2, 1, 3]]
    edges_local = np.array([[0, 1], [1, 2], [0, 2], [0, 3], [1, 3], [2, 3]])
    e = tets[:, edges_local]  # (T, 6, 2)
    e_sorted = np.sort(e, axis=2).reshape(-1, 2)
    key = e_sorted[:, 0] * len(verts) + e_sorted[:, 1]
    uniq, inv = np.unique(key, return_inverse=True)
    mids_a, mids_b = uniq // len(verts), uniq % len(verts)
    mid_pts = 0.5 * (verts[mids_a] + verts[mids_b])
    points = np.concatenate([verts, mid_pts])
    cells = np.concatenate([tets, len(verts) + inv.reshape(-1, 6)], axis=1)
    return _MeshioLike(points, {"tetra10": cells})
