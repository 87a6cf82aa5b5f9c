"""Problem definitions shared by the tests: the reference's FEniCSx regression cases
(tests/benchmarks/*/test_*.py) written once for the GB300 API and once for the oracle."""
import numpy as np
import torch

import jax_fem_gb300 as jf
from oracle import fem as ofem, materials as omat

H = 10.0


def _x0(p):
    return np.isclose(p[0], 0.0, atol=1e-5)


def _x1(p):
    return np.isclose(p[0], 1.0, atol=1e-5)


def _bottom(p):
    return np.isclose(p[2], 0.0, atol=1e-5)


def _top(p):
    return np.isclose(p[2], H, atol=1e-5)


def cube_elasticity(g):
    """test_linear_elasticity_cube.py:15-72: E=70e3, nu=0.3, u=1 at x=0, body -(0,10,10), surface -(10,0,0)."""
    one = lambda p: 1.0
    bc = [[_x0] * 3, [0, 1, 2], [one] * 3]

    class P(jf.Problem):
        def get_tensor_map(self):
            def stress(u_grad):
                E, nu = 70e3, 0.3
                mu = E / (2. * (1. + nu))
                lmbda = E * nu / ((1 + nu) * (1 - 2 * nu))
                eps = 0.5 * (u_grad + u_grad.T)
                return lmbda * np.trace(eps) * np.eye(3) + 2 * mu * eps
            return stress

        def get_mass_map(self):
            return lambda u, x: -np.array([0., 10., 10.])

        def get_surface_maps(self):
            return [lambda u, x: -np.array([10., 0., 0.])]

    mesh = jf.Mesh(g["points"], g["cells"])
    prob = P(mesh, vec=3, dim=3, dirichlet_bc_info=bc, location_fns=[_x1])
    oprob = ofem.OracleProblem(g["points"], g["cells"], 3, dirichlet_bc_info=bc, location_fns=[_x1],
                               tensor_map=omat.linear_elastic(70e3, 0.3),
                               mass_map=lambda u, x: -torch.tensor([0., 10., 10.]),
                               surface_maps=[lambda u, x: -torch.tensor([10., 0., 0.])])
    return prob, oprob


def poisson(g):
    """test_linear_poisson.py:15-55."""
    bc = [[_x0, _x1], [0, 0], [lambda p: 0., lambda p: 1.]]

    class P(jf.Problem):
        def get_tensor_map(self):
            return lambda x: x

    mesh = jf.Mesh(g["points"], g["cells"])
    prob = P(mesh, vec=1, dim=3, dirichlet_bc_info=bc)
    oprob = ofem.OracleProblem(g["points"], g["cells"], 1, dirichlet_bc_info=bc, tensor_map=omat.laplace())
    return prob, oprob


def cylinder_elasticity(g):
    """test_linear_elasticity_cylinder.py:15-112."""
    zero = lambda p: 0.0
    bc = [[_bottom] * 3, [0, 1, 2], [zero] * 3]

    class P(jf.Problem):
        def get_tensor_map(self):
            return jf.LinearElastic(70e3, 0.3)

        def get_mass_map(self):
            return lambda u, x: -np.array([1e3 * x[0], 2e3 * x[1], 3e3 * x[2]])

        def get_surface_maps(self):
            return [lambda u, x: -np.array([1e3 * x[0] ** 2 + 1e3 * x[1] ** 2, 0. * x[0], 0. * x[0]])]

    mesh = jf.Mesh(g["points"], g["cells"])
    prob = P(mesh, vec=3, dim=3, dirichlet_bc_info=bc, location_fns=[_top])
    oprob = ofem.OracleProblem(g["points"], g["cells"], 3, dirichlet_bc_info=bc, location_fns=[_top],
                               tensor_map=omat.linear_elastic(70e3, 0.3),
                               mass_map=lambda u, x: -torch.stack([1e3 * x[0], 2e3 * x[1], 3e3 * x[2]]),
                               surface_maps=[lambda u, x: -torch.stack([1e3 * x[0] ** 2 + 1e3 * x[1] ** 2,
                                                                         0 * x[0], 0 * x[0]])])
    return prob, oprob


def hyperelastic(g):
    """test_hyper_elasticity.py:15-109: E=1e3, nu=0.3, bottom fixed, top u_z=1."""
    zero = lambda p: 0.0
    bc = [[_bottom] * 3 + [_top] * 3, [0, 1, 2, 0, 1, 2], [zero] * 5 + [lambda p: 1.0]]

    class P(jf.Problem):
        def get_tensor_map(self):
            return jf.NeoHookean(1e3, 0.3)

    mesh = jf.Mesh(g["points"], g["cells"])
    prob = P(mesh, vec=3, dim=3, dirichlet_bc_info=bc)
    oprob = ofem.OracleProblem(g["points"], g["cells"], 3, dirichlet_bc_info=bc,
                               tensor_map=omat.neo_hookean(1e3, 0.3))
    return prob, oprob, bc


def plasticity(g):
    """test_plasticity.py:16-137: J2, E=70e3, nu=0.3, sig0=250, top u_z = disps[k]."""
    zero = lambda p: 0.0
    disps = g["disps"]
    bc = [[_bottom] * 3 + [_top] * 3, [0, 1, 2, 0, 1, 2], [zero] * 5 + [lambda p, d=disps[0]: d]]

    class P(jf.Problem):
        def custom_init(self):
            fe = self.fes[0]
            self.sigmas_old = torch.zeros((fe.num_cells, fe.num_quads, 3, 3), dtype=torch.float64, device="cuda")
            self.epsilons_old = torch.zeros_like(self.sigmas_old)
            self.internal_vars = [self.sigmas_old, self.epsilons_old]

        def get_tensor_map(self):
            return jf.J2Plasticity(70e3, 0.3, 250.0)

        def update_stress_strain(self, sol):
            self.sigmas_old, self.epsilons_old = self._engine.j2_update(sol.reshape(-1))
            self.internal_vars = [self.sigmas_old, self.epsilons_old]

        def compute_avg_stress(self):
            _, jxw = self._engine.quad_points()
            s = (self.sigmas_old * jxw[:, :, None, None]).sum((0, 1))
            return s / jxw.sum()

    mesh = jf.Mesh(g["points"], g["cells"])
    prob = P(mesh, vec=3, dim=3, dirichlet_bc_info=bc)
    return prob, bc, disps


def simp_box(nx, ny, nz, L=(2.0, 1.0, 0.5), seed=0, theta=None, load=1.0):
    """SIMP cantilever: clamped x=0, traction on x=Lx face (surface map (0, 0, load)),
    theta = 0.5 + U(-0.05, 0.05)."""
    Lx, Ly, Lz = L
    m = jf.box_mesh(nx, ny, nz, Lx, Ly, Lz)
    points, cells = m.points, m.cells_dict["hexahedron"]
    left = lambda p: np.isclose(p[0], 0.0, atol=1e-5)
    right = lambda p: np.isclose(p[0], Lx, atol=1e-5)
    zero = lambda p: 0.0
    bc = [[left] * 3, [0, 1, 2], [zero] * 3]

    class P(jf.Problem):
        def get_tensor_map(self):
            return jf.SIMPElastic(1.0, 1e-3, 0.3, 3.0)

        def get_surface_maps(self):
            return [lambda u, x: np.array([0.0, 0.0, load])]

        def set_params(self, params):
            self.internal_vars = [params[:, None, :].expand(-1, 8, -1)]

    prob = P(jf.Mesh(points, cells), vec=3, dim=3, dirichlet_bc_info=bc, location_fns=[right])
    oprob = ofem.OracleProblem(points, cells, 3, dirichlet_bc_info=bc, location_fns=[right],
                               tensor_map=omat.simp_elastic(1.0, 1e-3, 0.3, 3.0),
                               surface_maps=[lambda u, x: torch.tensor([0.0, 0.0, load])])
    if theta is None:
        rng = np.random.default_rng(seed)
        theta = 0.5 + rng.uniform(-0.05, 0.05, size=(len(cells), 1))
    return prob, oprob, theta


def oracle_set_params(oprob, p):
    return [p[:, None, :].expand(-1, 8, -1)]
