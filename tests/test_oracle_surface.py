"""CPU checks that pin the oracle's face kernel for u-dependent surface maps (jax_fem/problem.py:
238-259, the Robin pattern of applications/robin_bc/example.py:64-80) independently of the GPU."""
import numpy as np
import torch

from oracle import fem as ofem, materials as omat


def _laplace(n, surface_maps, locs):
    pts, cells = ofem.box_mesh(n, n, n, 1.0, 1.0, 1.0)
    left = lambda p: np.isclose(p[0], 0.0, atol=1e-5)
    bc = [[left], [0], [lambda p: 0.0]]
    return ofem.OracleProblem(pts, cells, 1, dirichlet_bc_info=bc, location_fns=locs, tensor_map=omat.laplace(),
                              surface_maps=surface_maps), pts


def test_linear_robin_face_matrix_is_the_face_mass_matrix():
    """A spring map k u on the face x = 1 adds k * int N_a N_b dS to the tangent: symmetric,
    entries summing to k * area, row sums equal to k times the lumped face weights of a uniform
    bilinear grid (h^2 inside, h^2/2 on edges, h^2/4 at corners), and nothing off the face."""
    n, k = 3, 7.0
    right = lambda p: np.isclose(p[0], 1.0, atol=1e-5)
    robin, pts = _laplace(n, [lambda u, x: k * u], [right])
    plain, _ = _laplace(n, [lambda u, x: 0.0 * u], [right])
    u = torch.from_numpy(np.random.default_rng(1).uniform(0.1, 1.0, len(pts)))
    robin.newton_update(u)
    plain.newton_update(u)
    D = (ofem.assemble_petsc(robin) - ofem.assemble_petsc(plain)).toarray()
    assert np.abs(D - D.T).max() <= 1e-14 * k
    assert abs(D.sum() - k * 1.0) <= 1e-12 * k
    h = 1.0 / n
    on_face = np.isclose(pts[:, 0], 1.0)
    on_edge_y = np.isclose(pts[:, 1], 0.0) | np.isclose(pts[:, 1], 1.0)
    on_edge_z = np.isclose(pts[:, 2], 0.0) | np.isclose(pts[:, 2], 1.0)
    lumped = np.where(on_face, h * h / (2.0 ** (on_edge_y.astype(int) + on_edge_z.astype(int))), 0.0)
    np.testing.assert_allclose(D.sum(axis=1), k * lumped, rtol=0, atol=1e-13 * k)
    assert np.abs(D[~on_face]).max() == 0.0 and np.abs(D[:, ~on_face]).max() == 0.0


def test_robin_residual_is_the_map_integrated_against_shape_functions():
    """For t(u) = 5 u^2 on x = 1 and u = c constant, the face residual is 5 c^2 int N_a dS: the
    lumped weights times 5 c^2 (the residual convention R = ... + int t(u) N_a dS)."""
    n, c = 2, 0.6
    right = lambda p: np.isclose(p[0], 1.0, atol=1e-5)
    robin, pts = _laplace(n, [lambda u, x: 5.0 * u ** 2], [right])
    plain, _ = _laplace(n, [lambda u, x: 0.0 * u], [right])
    u = torch.full((len(pts),), c, dtype=torch.float64)
    r = robin.compute_residual(u).numpy() - plain.compute_residual(u).numpy()
    h = 1.0 / n
    on_face = np.isclose(pts[:, 0], 1.0)
    edges = (np.isclose(pts[:, 1], 0.0) | np.isclose(pts[:, 1], 1.0)).astype(int) + \
        (np.isclose(pts[:, 2], 0.0) | np.isclose(pts[:, 2], 1.0)).astype(int)
    lumped = np.where(on_face, h * h / 2.0 ** edges, 0.0)
    np.testing.assert_allclose(r, 5.0 * c * c * lumped, rtol=0, atol=1e-14)
