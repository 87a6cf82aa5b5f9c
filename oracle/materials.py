"""Per-quadrature-point tensor maps of the reference's built-in physics, in torch (CPU, float64).

Each map acts on a single point (vmapped by the caller), exactly like the
reference's user functions.  Sources:
  Laplace / heat          tests/benchmarks/linear_poisson/test_linear_poisson.py:15-17
  linear elasticity       tests/benchmarks/linear_elasticity_cube/test_linear_elasticity_cube.py:15-26
  SIMP (3D isotropic)     docs/source/learn/topology_optimization/example.ipynb cell 9 (E law), 3D Hooke
  Neo-Hookean             tests/benchmarks/hyperelasticity/test_hyper_elasticity.py:15-34,
                          applications/scalability/hyperelastic3d_common.py:45-70 (rho scaling, J clamp)
  J2 small strain         tests/benchmarks/plasticity/test_plasticity.py:32-78
"""
import torch


def lame(E, nu):
    mu = E / (2.0 * (1.0 + nu))
    lmbda = E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu))
    return lmbda, mu


def laplace():
    return lambda u_grad: u_grad


def linear_elastic(E, nu):
    lmbda, mu = lame(E, nu)

    def stress(u_grad):
        eps = 0.5 * (u_grad + u_grad.T)
        return lmbda * torch.trace(eps) * torch.eye(3, dtype=u_grad.dtype) + 2.0 * mu * eps
    return stress


def simp_modulus(theta, Emax, Emin, penal):
    return Emin + (Emax - Emin) * theta ** penal


def simp_elastic(Emax, Emin, nu, penal):
    """stress(u_grad, theta) with theta shaped (1,) per quad point."""
    def stress(u_grad, theta):
        E = simp_modulus(theta[0], Emax, Emin, penal)
        lmbda, mu = lame(E, nu)
        eps = 0.5 * (u_grad + u_grad.T)
        return lmbda * torch.trace(eps) * torch.eye(3, dtype=u_grad.dtype) + 2.0 * mu * eps
    return stress


def det3(F):
    """3x3 determinant by cofactor expansion (AD-friendly at any order)."""
    return (F[0, 0] * (F[1, 1] * F[2, 2] - F[1, 2] * F[2, 1])
            - F[0, 1] * (F[1, 0] * F[2, 2] - F[1, 2] * F[2, 0])
            + F[0, 2] * (F[1, 0] * F[2, 1] - F[1, 1] * F[2, 0]))


def neo_hookean(E, nu, with_rho=False):
    """First Piola-Kirchhoff stress of psi = mu/2 (J^{-2/3} I1 - 3) + kappa/2 (J-1)^2."""
    def psi(F, scale):
        Ee = E * scale
        mu = Ee / (2.0 * (1.0 + nu))
        kappa = Ee / (3.0 * (1.0 - 2.0 * nu))
        J = det3(F)
        if with_rho:
            J = torch.clamp(J, min=1e-14)
        Jinv = J ** (-2.0 / 3.0)
        I1 = torch.trace(F.T @ F)
        return (mu / 2.0) * (Jinv * I1 - 3.0) + (kappa / 2.0) * (J - 1.0) ** 2

    P_fn = torch.func.grad(psi, argnums=0)
    if with_rho:
        def first_pk(u_grad, rho):
            return P_fn(u_grad + torch.eye(3, dtype=u_grad.dtype), rho[0] if rho.ndim else rho)
    else:
        def first_pk(u_grad):
            return P_fn(u_grad + torch.eye(3, dtype=u_grad.dtype), torch.ones((), dtype=u_grad.dtype))
    return first_pk


def j2_maps(E, nu, sig0, mu_field=False):
    """(strain, stress_return_map) following test_plasticity.py:33-65.

    With mu_field=True the return map takes an extra per-point factor s (shape (1,))
    scaling E (so the shear modulus mu = s * mu0)."""
    def safe_sqrt(x):
        return torch.where(x > 0.0, torch.sqrt(torch.where(x > 0.0, x, torch.ones_like(x))), torch.zeros_like(x))

    def safe_divide(x, y):
        return torch.where(y == 0.0, torch.zeros_like(x), x / torch.where(y == 0.0, torch.ones_like(y), y))

    def strain(u_grad):
        return 0.5 * (u_grad + u_grad.T)

    def stress(eps, scale):
        lmbda, mu = lame(E * scale, nu)
        return lmbda * torch.trace(eps) * torch.eye(3, dtype=eps.dtype) + 2.0 * mu * eps

    def rmap(u_grad, sigma_old, epsilon_old, scale):
        eps_crt = strain(u_grad)
        eps_inc = eps_crt - epsilon_old
        sigma_trial = stress(eps_inc, scale) + sigma_old
        s_dev = sigma_trial - (1.0 / 3.0) * torch.trace(sigma_trial) * torch.eye(3, dtype=u_grad.dtype)
        s_norm = safe_sqrt(1.5 * torch.sum(s_dev * s_dev))
        f_yield = s_norm - sig0
        f_plus = torch.where(f_yield > 0.0, f_yield, torch.zeros_like(f_yield))
        return sigma_trial - safe_divide(f_plus * s_dev, s_norm)

    if mu_field:
        def stress_return_map(u_grad, sigma_old, epsilon_old, s):
            return rmap(u_grad, sigma_old, epsilon_old, s[0])
    else:
        def stress_return_map(u_grad, sigma_old, epsilon_old):
            return rmap(u_grad, sigma_old, epsilon_old, torch.ones((), dtype=u_grad.dtype))
    return strain, stress_return_map
