// Material-point laws of the reference's built-in physics with hand-derived
// consistent tangents (the reference differentiates them with jax.jacfwd,
// jax_fem/problem.py:262-266; here dP/dF is written out once per law).
//
//   LAPLACE         S = k grad u                      test_linear_poisson.py:15-17
//   LINEAR_ELASTIC  S = lam tr(eps) I + 2 mu eps      test_linear_elasticity_cube.py:15-26
//   SIMP            same with E = Emin + (Emax-Emin) theta^p   (topology_optimization example)
//   GENERAL_LINEAR  S_I = C_IJ grad_J   (any linear tensor map, probed on the host)
//   NEO_HOOKEAN     P = dpsi/dF, psi = mu/2 (J^-2/3 I1 - 3) + kappa/2 (J-1)^2
//                   test_hyper_elasticity.py:17-34; optional rho scaling and J clamp
//                   from applications/scalability/hyperelastic3d_common.py:53-60
//   J2              small-strain radial return         test_plasticity.py:32-65
//
// Tangent kinds: TAN_SCALAR (K_ab = t0 ga.gb), TAN_ISO (lam, mu), TAN_FULL
// ((vec*3)^2 entries A[(i,j),(k,l)] = dS_ij / d grad_kl).
#pragma once

#include <cmath>

namespace fem {

enum { TAN_SCALAR = 0, TAN_ISO = 1, TAN_FULL = 2 };

struct MatConsts {
  double c[96];
  int n;
  int clamp;   // NEO_HOOKEAN J clamp flag
};

template <typename T>
__device__ __forceinline__ void lame(T E, T nu, T& lam, T& mu) {
  mu = E / (T(2) * (T(1) + nu));
  lam = E * nu / ((T(1) + nu) * (T(1) - T(2) * nu));
}

template <int MAT, int VEC>
struct MatTraits;

template <> struct MatTraits<FEM_MAT_LAPLACE, 1> { static constexpr int TAN = TAN_SCALAR, NTAN = 1; };
template <> struct MatTraits<FEM_MAT_LINEAR_ELASTIC, 3> { static constexpr int TAN = TAN_ISO, NTAN = 2; };
template <> struct MatTraits<FEM_MAT_SIMP, 3> { static constexpr int TAN = TAN_ISO, NTAN = 2; };
template <> struct MatTraits<FEM_MAT_GENERAL_LINEAR, 1> { static constexpr int TAN = TAN_FULL, NTAN = 9; };
template <> struct MatTraits<FEM_MAT_GENERAL_LINEAR, 3> { static constexpr int TAN = TAN_FULL, NTAN = 81; };
template <> struct MatTraits<FEM_MAT_NEO_HOOKEAN, 3> { static constexpr int TAN = TAN_FULL, NTAN = 81; };
template <> struct MatTraits<FEM_MAT_J2, 3> { static constexpr int TAN = TAN_FULL, NTAN = 81; };

// Evaluate stress S (VEC x 3, row-major) and optionally the tangent.
// qp: this point's parameters (may be null), hist: 18 history values (J2).
template <int MAT, int VEC, typename T>
struct Material;

template <typename T>
struct Material<FEM_MAT_LAPLACE, 1, T> {
  __device__ static void eval(const T g[3], const MatConsts& mc, const double*, const double*,
                              T S[3], T* tan, bool want_tan) {
    const T k = T(mc.c[0]);
    for (int d = 0; d < 3; ++d) S[d] = k * g[d];
    if (want_tan) tan[0] = k;
  }
  __device__ static void dparam(const T*, const MatConsts&, const double*, const double*, T*) {}
};

template <typename T>
__device__ __forceinline__ void iso_stress(const T g[9], T lam, T mu, T S[9]) {
  const T tr = g[0] + g[4] + g[8];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) S[i * 3 + j] = mu * (g[i * 3 + j] + g[j * 3 + i]) + (i == j ? lam * tr : T(0));
}

template <typename T>
struct Material<FEM_MAT_LINEAR_ELASTIC, 3, T> {
  __device__ static void eval(const T g[9], const MatConsts& mc, const double*, const double*,
                              T S[9], T* tan, bool want_tan) {
    T lam, mu;
    lame<T>(T(mc.c[0]), T(mc.c[1]), lam, mu);
    iso_stress(g, lam, mu, S);
    if (want_tan) { tan[0] = lam; tan[1] = mu; }
  }
  // lam / mu = 2 nu / (1 - 2 nu): the same at every point
  __device__ static T lam_over_mu(const MatConsts& mc) { return T(2) * T(mc.c[1]) / (T(1) - T(2) * T(mc.c[1])); }
  __device__ static void dparam(const T*, const MatConsts&, const double*, const double*, T*) {}
};

// SIMP: E(theta) = Emin + (Emax - Emin) theta^p ; consts [Emax, Emin, nu, penal]
template <typename T>
struct Material<FEM_MAT_SIMP, 3, T> {
  __device__ static T modulus(T th, const MatConsts& mc) {
    const T p = T(mc.c[3]);
    const T tp = (mc.c[3] == 3.0) ? th * th * th : pow(th, p);
    return T(mc.c[1]) + (T(mc.c[0]) - T(mc.c[1])) * tp;
  }
  __device__ static T dmodulus(T th, const MatConsts& mc) {
    const T p = T(mc.c[3]);
    const T tp1 = (mc.c[3] == 3.0) ? th * th : pow(th, p - T(1));
    return (T(mc.c[0]) - T(mc.c[1])) * p * tp1;
  }
  __device__ static void eval(const T g[9], const MatConsts& mc, const double* qp, const double*,
                              T S[9], T* tan, bool want_tan) {
    const T E = modulus(T(qp[0]), mc);
    T lam, mu;
    lame<T>(E, T(mc.c[2]), lam, mu);
    iso_stress(g, lam, mu, S);
    if (want_tan) { tan[0] = lam; tan[1] = mu; }
  }
  // lam / mu = 2 nu / (1 - 2 nu): only E varies with theta
  __device__ static T lam_over_mu(const MatConsts& mc) { return T(2) * T(mc.c[2]) / (T(1) - T(2) * T(mc.c[2])); }
  // dS/dtheta
  __device__ static void dparam(const T g[9], const MatConsts& mc, const double* qp, const double*, T dS[9]) {
    const T dE = dmodulus(T(qp[0]), mc);
    T lam, mu;
    lame<T>(dE, T(mc.c[2]), lam, mu);
    iso_stress(g, lam, mu, dS);
  }
};

template <int VEC, typename T>
struct Material<FEM_MAT_GENERAL_LINEAR, VEC, T> {
  static constexpr int M = VEC * 3;
  __device__ static void eval(const T g[M], const MatConsts& mc, const double*, const double*,
                              T S[M], T* tan, bool want_tan) {
    for (int I = 0; I < M; ++I) {
      T s = T(0);
      for (int J = 0; J < M; ++J) s += T(mc.c[I * M + J]) * g[J];
      S[I] = s;
    }
    if (want_tan)
      for (int k = 0; k < M * M; ++k) tan[k] = T(mc.c[k]);
  }
  __device__ static void dparam(const T*, const MatConsts&, const double*, const double*, T*) {}
};

// Neo-Hookean: P = c1 (F - I1/3 H) + kappa J (J-1) H,  H = F^-T, c1 = mu J^-2/3.
// A_ijkl = c1 [d_ik d_jl - 2/3 (H_kl F_ij + F_kl H_ij) + 2/9 I1 H_ij H_kl + I1/3 H_kj H_il]
//        + kappa [(2J-1) J H_ij H_kl - J (J-1) H_kj H_il]
// consts [E, nu, clampJ]; optional qp param rho scales E.
template <typename T>
struct Material<FEM_MAT_NEO_HOOKEAN, 3, T> {
  __device__ static void eval(const T g[9], const MatConsts& mc, const double* qp, const double*,
                              T S[9], T* tan, bool want_tan) {
    T E = T(mc.c[0]);
    if (qp) E *= T(qp[0]);
    const T nu = T(mc.c[1]);
    const T mu = E / (T(2) * (T(1) + nu));
    const T kappa = E / (T(3) * (T(1) - T(2) * nu));
    T F[3][3];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) F[i][j] = g[i * 3 + j] + (i == j ? T(1) : T(0));
    T J = det3<T>(F);
    bool clamped = false;
    if (mc.clamp && J < T(1e-14)) { J = T(1e-14); clamped = true; }
    T Fi[3][3];
    inv3<T>(F, det3<T>(F), Fi);
    T H[3][3];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) H[i][j] = Fi[j][i];
    T I1 = T(0);
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) I1 += F[i][j] * F[i][j];
    const T cb = cbrt(J);
    const T c1 = mu / (cb * cb);
    if (clamped) {
      // J = max(det F, 1e-14) is constant below the clamp: P = c1 F, A = c1 I
      for (int k = 0; k < 9; ++k) S[k] = c1 * g[k] + ((k == 0 || k == 4 || k == 8) ? c1 : T(0));
      if (want_tan)
        for (int k = 0; k < 81; ++k) tan[k] = (k / 9 == k % 9) ? c1 : T(0);
      return;
    }
    const T c2 = kappa * J * (J - T(1));
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) S[i * 3 + j] = c1 * (F[i][j] - I1 / T(3) * H[i][j]) + c2 * H[i][j];
    if (!want_tan) return;
    const T k1 = kappa * (T(2) * J - T(1)) * J;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j)
        for (int k = 0; k < 3; ++k)
          for (int l = 0; l < 3; ++l) {
            const T a = c1 * ((i == k && j == l ? T(1) : T(0)) - T(2) / T(3) * (H[k][l] * F[i][j] + F[k][l] * H[i][j]) +
                              T(2) / T(9) * I1 * H[i][j] * H[k][l] + I1 / T(3) * H[k][j] * H[i][l]) +
                        k1 * H[i][j] * H[k][l] - c2 * H[k][j] * H[i][l];
            tan[(i * 3 + j) * 9 + k * 3 + l] = a;
          }
  }
  // dP/drho = P(rho = 1)
  __device__ static void dparam(const T g[9], const MatConsts& mc, const double*, const double*, T dS[9]) {
    eval(g, mc, nullptr, nullptr, dS, nullptr, false);
  }
};

// J2 small strain, perfect plasticity (radial return); consts [E, nu, sig0];
// history sigma_old(9) | eps_old(9); optional qp param s scaling E.
// Plastic tangent: A = C - beta*mu*(I4s2 - 2/3 I(x)I) - gamma s(x)s,
// beta = 1 - sig0/q, gamma = 3 mu sig0 / q^3, I4s2_ijkl = d_ik d_jl + d_il d_jk.
template <typename T>
struct Material<FEM_MAT_J2, 3, T> {
  struct State {
    T lam, mu, sig_tr[9], s[9], q, deps[9];
    bool plastic;
  };
  __device__ static void trial(const T g[9], const MatConsts& mc, const double* qp, const double* hist, State& st) {
    T E = T(mc.c[0]);
    if (qp) E *= T(qp[0]);
    lame<T>(E, T(mc.c[1]), st.lam, st.mu);
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        const T e = T(0.5) * (g[i * 3 + j] + g[j * 3 + i]);
        st.deps[i * 3 + j] = e - (hist ? T(hist[9 + i * 3 + j]) : T(0));
      }
    const T tr = st.deps[0] + st.deps[4] + st.deps[8];
    for (int k = 0; k < 9; ++k)
      st.sig_tr[k] = T(2) * st.mu * st.deps[k] + (hist ? T(hist[k]) : T(0));
    st.sig_tr[0] += st.lam * tr; st.sig_tr[4] += st.lam * tr; st.sig_tr[8] += st.lam * tr;
    const T p = (st.sig_tr[0] + st.sig_tr[4] + st.sig_tr[8]) / T(3);
    T ss = T(0);
    for (int k = 0; k < 9; ++k) {
      st.s[k] = st.sig_tr[k] - ((k == 0 || k == 4 || k == 8) ? p : T(0));
      ss += st.s[k] * st.s[k];
    }
    const T x = T(1.5) * ss;
    st.q = x > T(0) ? sqrt(x) : T(0);
    st.plastic = (st.q - T(mc.c[2])) > T(0);
  }
  __device__ static void eval(const T g[9], const MatConsts& mc, const double* qp, const double* hist,
                              T S[9], T* tan, bool want_tan) {
    State st;
    trial(g, mc, qp, hist, st);
    const T sig0 = T(mc.c[2]);
    const T beta = st.plastic ? (T(1) - sig0 / st.q) : T(0);
    for (int k = 0; k < 9; ++k) S[k] = st.sig_tr[k] - beta * st.s[k];
    if (!want_tan) return;
    const T gam = st.plastic ? T(3) * st.mu * sig0 / (st.q * st.q * st.q) : T(0);
    const T bm = beta * st.mu;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j)
        for (int k = 0; k < 3; ++k)
          for (int l = 0; l < 3; ++l) {
            const T dij = i == j ? T(1) : T(0), dkl = k == l ? T(1) : T(0);
            const T i4 = (i == k && j == l ? T(1) : T(0)) + (i == l && j == k ? T(1) : T(0));
            tan[(i * 3 + j) * 9 + k * 3 + l] = st.lam * dij * dkl + st.mu * i4 - bm * (i4 - T(2) / T(3) * dij * dkl) -
                                               gam * st.s[i * 3 + j] * st.s[k * 3 + l];
          }
  }
  // d sigma / d s for the E-scale parameter s (history held fixed)
  __device__ static void dparam(const T g[9], const MatConsts& mc, const double* qp, const double* hist, T dS[9]) {
    State st;
    trial(g, mc, qp, hist, st);
    const T scale = qp ? T(qp[0]) : T(1);
    const T lam0 = st.lam / scale, mu0 = st.mu / scale;
    const T tr = st.deps[0] + st.deps[4] + st.deps[8];
    T dtr[9];
    for (int k = 0; k < 9; ++k) dtr[k] = T(2) * mu0 * st.deps[k] + ((k == 0 || k == 4 || k == 8) ? lam0 * tr : T(0));
    if (!st.plastic) {
      for (int k = 0; k < 9; ++k) dS[k] = dtr[k];
      return;
    }
    const T sig0 = T(mc.c[2]);
    const T beta = T(1) - sig0 / st.q;
    const T trd = tr / T(3);
    T sde = T(0);
    for (int k = 0; k < 9; ++k) sde += st.s[k] * st.deps[k];
    const T gam = T(3) * mu0 * sig0 / (st.q * st.q * st.q);
    for (int k = 0; k < 9; ++k) {
      const T dev = st.deps[k] - ((k == 0 || k == 4 || k == 8) ? trd : T(0));
      dS[k] = dtr[k] - beta * T(2) * mu0 * dev - gam * sde * st.s[k];
    }
  }
  // Reverse mode through the return map and the history update (test_plasticity.py:54-78).
  // Given cotangents gs of sigma_new (9) and ge of eps_new = sym(g) (9), returns the cotangent W
  // of g = grad u (9), of sigma_old (dso), eps_old (deo) and of the E scale (dsc).
  // sigma depends on sigma_tr only, with D = d sigma / d sigma_tr
  //   = (1 - beta) I + (beta / 3) I(x)I - (3 sig0 / (2 q^3)) s(x)s   (identity when elastic),
  // and sigma_tr = C : (sym(g) - eps_old) + sigma_old.
  __device__ static void hist_vjp(const T g[9], const MatConsts& mc, const double* qp, const double* hist,
                                  const T gs[9], const T ge[9], T W[9], T dso[9], T deo[9], T& dsc) {
    State st;
    trial(g, mc, qp, hist, st);
    T z[9];
    if (st.plastic) {
      const T sig0 = T(mc.c[2]);
      const T beta = T(1) - sig0 / st.q;
      const T c3 = T(1.5) * sig0 / (st.q * st.q * st.q);
      const T trg = gs[0] + gs[4] + gs[8];
      T gss = T(0);
      for (int k = 0; k < 9; ++k) gss += gs[k] * st.s[k];
      for (int k = 0; k < 9; ++k)
        z[k] = (T(1) - beta) * gs[k] + ((k == 0 || k == 4 || k == 8) ? beta * trg / T(3) : T(0)) - c3 * gss * st.s[k];
    } else {
      for (int k = 0; k < 9; ++k) z[k] = gs[k];
    }
    // y = C^T : z on the 9 components of deps (deps_ij = sym(g)_ij - eps_old_ij)
    const T trz = z[0] + z[4] + z[8];
    T y[9];
    for (int k = 0; k < 9; ++k) y[k] = T(2) * st.mu * z[k] + ((k == 0 || k == 4 || k == 8) ? st.lam * trz : T(0));
    for (int k = 0; k < 9; ++k) {
      dso[k] = z[k];
      deo[k] = -y[k];
    }
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j)
        W[i * 3 + j] = T(0.5) * (y[i * 3 + j] + y[j * 3 + i]) + T(0.5) * (ge[i * 3 + j] + ge[j * 3 + i]);
    T dS[9];
    dparam(g, mc, qp, hist, dS);
    dsc = T(0);
    for (int k = 0; k < 9; ++k) dsc += gs[k] * dS[k];
  }
};

}  // namespace fem
