// Method of Moving Asymptotes on the GPU (jax_fem/mma.py): the asymptote / approximation set-up
// of MMA.mmasub (mma.py:113-206) and the primal-dual interior-point subsolv (mma.py:209-405),
// plus the k-d tree sensitivity / density filter (mma.py:27-66) as a grid-hashed radius search.
//
// Design: every per-variable quantity (x, xsi, eta and their Newton directions, the convex
// approximation p0, q0, P, Q, the bounds alfa / beta) lives in a caller workspace on the GPU
// and is touched by four grid-stride kernels (set-up, residual, Newton system, direction) that
// also produce per-CTA partial sums / maxima.  A one-CTA kernel reduces the partials in a fixed
// order (deterministic), and the host holds the m-sized dual variables (y, z, lambda, mu, zeta,
// s), solves the (m+1)x(m+1) reduced Newton system and runs the step-length logic.  m <= 4.
#include <cmath>
#include <vector>

#include "fem_common.cuh"

namespace fem {

constexpr int MMA_THREADS = 256;
constexpr int MMA_MAXM = 4;
constexpr int MMA_MAX_BLOCKS = 2048;
constexpr int MMA_MAXK = 64;   // partial-sum slots per CTA

// Small per-call scalars passed by value.
struct MmaScal {
  double lam[MMA_MAXM];
  double dlam[MMA_MAXM];
  double epsi;
  double steg;
};

// Block reduction of KS sums followed by KM maxima into partials[blockIdx.x * (KS + KM) + k].
template <int KS, int KM>
__device__ __forceinline__ void mma_block_store(double (&v)[KS + KM > 0 ? KS + KM : 1], double* partials) {
  constexpr int K = KS + KM;
  constexpr int W = MMA_THREADS / 32;
  __shared__ double sh[K > 0 ? K : 1][W];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < K; ++k) {
    double t = v[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const double u = __shfl_xor_sync(0xffffffffu, t, o);
      t = k < KS ? t + u : fmax(t, u);
    }
    if (lane == 0) sh[k][warp] = t;
  }
  __syncthreads();
  if (threadIdx.x < K) {
    const int k = threadIdx.x;
    double acc = sh[k][0];
    for (int w = 1; w < W; ++w) acc = k < KS ? acc + sh[k][w] : fmax(acc, sh[k][w]);
    partials[(size_t)blockIdx.x * K + k] = acc;
  }
}

// One CTA: out[k] = sum (k < ks) or max (k >= ks) over the nb blocks' partials, fixed order.
__global__ void mma_reduce_kernel(const double* __restrict__ partials, int nb, int ks, int km, double* out) {
  __shared__ double sh[MMA_THREADS];
  const int K = ks + km;
  for (int k = 0; k < K; ++k) {
    const bool is_sum = k < ks;
    double acc = is_sum ? 0.0 : -INFINITY;
    for (int b = threadIdx.x; b < nb; b += blockDim.x) {
      const double v = partials[(size_t)b * K + k];
      acc = is_sum ? acc + v : fmax(acc, v);
    }
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
      if (threadIdx.x < s) sh[threadIdx.x] = is_sum ? sh[threadIdx.x] + sh[threadIdx.x + s]
                                                    : fmax(sh[threadIdx.x], sh[threadIdx.x + s]);
      __syncthreads();
    }
    if (threadIdx.x == 0) out[k] = sh[0];
    __syncthreads();
  }
}

#define MMA_LOOP(i, n) \
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < (n); i += (int64_t)gridDim.x * blockDim.x)

// Asymptotes (mma.py:136-155), bounds alfa/beta (mma.py:157-166), p0, q0, P, Q (mma.py:168-197),
// the partial sums of b = P/(upp - x) + Q/(x - low) (mma.py:199) and subsolv's starting point
// (mma.py:214-224).
template <int M>
__global__ void __launch_bounds__(MMA_THREADS)
mma_setup_kernel(int64_t n, int iter, const double* __restrict__ xval, const double* __restrict__ xold1,
                 const double* __restrict__ xold2, double* __restrict__ low, double* __restrict__ upp,
                 const double* __restrict__ xmin, const double* __restrict__ xmax, double move,
                 const double* __restrict__ df0dx, const double* __restrict__ dfdx, double* __restrict__ alfa,
                 double* __restrict__ beta, double* __restrict__ p0, double* __restrict__ q0, double* __restrict__ P,
                 double* __restrict__ Q, double* __restrict__ x, double* __restrict__ xsi, double* __restrict__ eta,
                 double* partials) {
  double v[M];
#pragma unroll
  for (int j = 0; j < M; ++j) v[j] = 0.0;
  MMA_LOOP(i, n) {
    const double xv = xval[i], span = xmax[i] - xmin[i];
    double lo, up;
    if (iter <= 2) {
      lo = xv - 0.5 * span;
      up = xv + 0.5 * span;
    } else {
      const double x1 = xold1[i];
      const double trend = (xv - x1) * (x1 - xold2[i]);
      const double f = trend > 0.0 ? 1.2 : (trend < 0.0 ? 0.7 : 1.0);
      lo = xv - f * (x1 - low[i]);
      up = xv + f * (upp[i] - x1);
      lo = fmin(fmax(lo, xv - 10.0 * span), xv - 0.01 * span);
      up = fmax(fmin(up, xv + 10.0 * span), xv + 0.01 * span);
    }
    low[i] = lo;
    upp[i] = up;
    const double al = fmax(fmax(lo + 0.1 * (xv - lo), xv - move * span), xmin[i]);
    const double be = fmin(fmin(up - 0.1 * (up - xv), xv + move * span), xmax[i]);
    alfa[i] = al;
    beta[i] = be;
    const double inv_span = 1.0 / fmax(span, 1e-5);
    const double ux1 = up - xv, xl1 = xv - lo;
    const double ux2 = ux1 * ux1, xl2 = xl1 * xl1;
    const double g = df0dx[i];
    const double pos = fmax(g, 0.0), neg = fmax(-g, 0.0);
    const double reg = 0.001 * (pos + neg) + 1e-5 * inv_span;
    p0[i] = (pos + reg) * ux2;
    q0[i] = (neg + reg) * xl2;
#pragma unroll
    for (int j = 0; j < M; ++j) {
      const double gj = dfdx[(int64_t)j * n + i];
      const double pj = fmax(gj, 0.0), qj = fmax(-gj, 0.0);
      const double rj = 0.001 * (pj + qj) + 1e-5 * inv_span;
      const double Pj = (pj + rj) * ux2, Qj = (qj + rj) * xl2;
      P[(int64_t)j * n + i] = Pj;
      Q[(int64_t)j * n + i] = Qj;
      v[j] += Pj / ux1 + Qj / xl1;
    }
    const double x0 = 0.5 * (al + be);
    x[i] = x0;
    xsi[i] = fmax(1.0 / (x0 - al), 1.0);
    eta[i] = fmax(1.0 / (be - x0), 1.0);
  }
  mma_block_store<M, 0>(v, partials);
}

// Per-variable residual parts (mma.py:225-251 / 366-388): sums of rex^2, rexsi^2, reeta^2 and
// gvec_j, and the max of their absolute values.  With trial != 0 the state is first set to
// old + steg * direction (the line search's trial point).
template <int M>
__global__ void __launch_bounds__(MMA_THREADS)
mma_residual_kernel(int64_t n, int trial, MmaScal sc, const double* __restrict__ low, const double* __restrict__ upp,
                    const double* __restrict__ alfa, const double* __restrict__ beta, const double* __restrict__ p0,
                    const double* __restrict__ q0, const double* __restrict__ P, const double* __restrict__ Q,
                    double* __restrict__ x, double* __restrict__ xsi, double* __restrict__ eta,
                    const double* __restrict__ xo, const double* __restrict__ xsio, const double* __restrict__ etao,
                    const double* __restrict__ dx, const double* __restrict__ dxsi, const double* __restrict__ deta,
                    double* partials) {
  double v[M + 4];
#pragma unroll
  for (int k = 0; k < M + 3; ++k) v[k] = 0.0;
  v[M + 3] = 0.0;
  MMA_LOOP(i, n) {
    double xv, xs, et;
    if (trial) {
      xv = xo[i] + sc.steg * dx[i];
      xs = xsio[i] + sc.steg * dxsi[i];
      et = etao[i] + sc.steg * deta[i];
      x[i] = xv;
      xsi[i] = xs;
      eta[i] = et;
    } else {
      xv = x[i];
      xs = xsi[i];
      et = eta[i];
    }
    const double ux1 = upp[i] - xv, xl1 = xv - low[i];
    double plam = p0[i], qlam = q0[i];
#pragma unroll
    for (int j = 0; j < M; ++j) {
      const double Pj = P[(int64_t)j * n + i], Qj = Q[(int64_t)j * n + i];
      plam += Pj * sc.lam[j];
      qlam += Qj * sc.lam[j];
      v[3 + j] += Pj / ux1 + Qj / xl1;
    }
    const double rex = plam / (ux1 * ux1) - qlam / (xl1 * xl1) - xs + et;
    const double rexsi = xs * (xv - alfa[i]) - sc.epsi;
    const double reeta = et * (beta[i] - xv) - sc.epsi;
    v[0] += rex * rex;
    v[1] += rexsi * rexsi;
    v[2] += reeta * reeta;
    v[M + 3] = fmax(v[M + 3], fmax(fabs(rex), fmax(fabs(rexsi), fabs(reeta))));
  }
  mma_block_store<M + 3, 1>(v, partials);
}

// Newton system parts (mma.py:257-299, m < n branch): stores delx, diagx and sums gvec_j,
// (GG (delx / diagx))_j and Alam_jk = sum GG_j GG_k / diagx (k >= j).
template <int M>
__global__ void __launch_bounds__(MMA_THREADS)
mma_newton_kernel(int64_t n, MmaScal sc, const double* __restrict__ low, const double* __restrict__ upp,
                  const double* __restrict__ alfa, const double* __restrict__ beta, const double* __restrict__ p0,
                  const double* __restrict__ q0, const double* __restrict__ P, const double* __restrict__ Q,
                  const double* __restrict__ x, const double* __restrict__ xsi, const double* __restrict__ eta,
                  double* __restrict__ delx, double* __restrict__ diagx, double* partials) {
  constexpr int NA = M * (M + 1) / 2;
  double v[2 * M + NA];
#pragma unroll
  for (int k = 0; k < 2 * M + NA; ++k) v[k] = 0.0;
  MMA_LOOP(i, n) {
    const double xv = x[i];
    const double ux1 = upp[i] - xv, xl1 = xv - low[i];
    const double ux2 = ux1 * ux1, xl2 = xl1 * xl1;
    const double xa = xv - alfa[i], bx = beta[i] - xv;
    double plam = p0[i], qlam = q0[i], gg[M];
#pragma unroll
    for (int j = 0; j < M; ++j) {
      const double Pj = P[(int64_t)j * n + i], Qj = Q[(int64_t)j * n + i];
      plam += Pj * sc.lam[j];
      qlam += Qj * sc.lam[j];
      v[j] += Pj / ux1 + Qj / xl1;
      gg[j] = Pj / ux2 - Qj / xl2;
    }
    const double dl = plam / ux2 - qlam / xl2 - sc.epsi / xa + sc.epsi / bx;
    const double dg = 2.0 * (plam / (ux1 * ux2) + qlam / (xl1 * xl2)) + xsi[i] / xa + eta[i] / bx;
    delx[i] = dl;
    diagx[i] = dg;
    const double r = dl / dg;
    int k = 2 * M;
#pragma unroll
    for (int j = 0; j < M; ++j) {
      v[M + j] += gg[j] * r;
#pragma unroll
      for (int l = j; l < M; ++l) v[k++] += gg[j] * gg[l] / dg;
    }
  }
  mma_block_store<2 * M + NA, 0>(v, partials);
}

// Newton directions dx, dxsi, deta (mma.py:300-329), a copy of the state as the line search's
// origin, and the largest step ratio over the per-variable entries (mma.py:330-339).
template <int M>
__global__ void __launch_bounds__(MMA_THREADS)
mma_direction_kernel(int64_t n, MmaScal sc, const double* __restrict__ low, const double* __restrict__ upp,
                     const double* __restrict__ alfa, const double* __restrict__ beta, const double* __restrict__ P,
                     const double* __restrict__ Q, const double* __restrict__ x, const double* __restrict__ xsi,
                     const double* __restrict__ eta, const double* __restrict__ delx, const double* __restrict__ diagx,
                     double* __restrict__ dx, double* __restrict__ dxsi, double* __restrict__ deta,
                     double* __restrict__ xo, double* __restrict__ xsio, double* __restrict__ etao, double* partials) {
  double v[1] = {-INFINITY};
  MMA_LOOP(i, n) {
    const double xv = x[i], xs = xsi[i], et = eta[i];
    const double ux1 = upp[i] - xv, xl1 = xv - low[i];
    const double ux2 = ux1 * ux1, xl2 = xl1 * xl1;
    const double xa = xv - alfa[i], bx = beta[i] - xv;
    double gl = 0.0;
#pragma unroll
    for (int j = 0; j < M; ++j)
      gl += (P[(int64_t)j * n + i] / ux2 - Q[(int64_t)j * n + i] / xl2) * sc.dlam[j];
    const double dg = diagx[i];
    const double d = -delx[i] / dg - gl / dg;
    const double ds = -xs + sc.epsi / xa - xs * d / xa;
    const double de = -et + sc.epsi / bx + et * d / bx;
    dx[i] = d;
    dxsi[i] = ds;
    deta[i] = de;
    xo[i] = xv;
    xsio[i] = xs;
    etao[i] = et;
    v[0] = fmax(v[0], fmax(fmax(-1.01 * ds / xs, -1.01 * de / et), fmax(-1.01 * d / xa, 1.01 * d / bx)));
  }
  mma_block_store<0, 1>(v, partials);
}

// ---- host driver --------------------------------------------------------------------
static size_t mma_al(size_t b) { return (b + 255) & ~size_t(255); }

static size_t mma_ws_bytes(int64_t n, int m) {
  return mma_al(sizeof(double) * (size_t)n) * (size_t)(15 + 2 * m) +
         mma_al(sizeof(double) * (size_t)MMA_MAX_BLOCKS * MMA_MAXK) + mma_al(sizeof(double) * MMA_MAXK);
}

// Dense (k x k) solve by Gaussian elimination with partial pivoting; false if singular.
static bool small_solve(std::vector<double>& A, std::vector<double>& b, int k) {
  for (int c = 0; c < k; ++c) {
    int piv = c;
    for (int r = c + 1; r < k; ++r)
      if (std::fabs(A[r * k + c]) > std::fabs(A[piv * k + c])) piv = r;
    if (A[piv * k + c] == 0.0) return false;
    if (piv != c) {
      for (int j = 0; j < k; ++j) std::swap(A[c * k + j], A[piv * k + j]);
      std::swap(b[c], b[piv]);
    }
    for (int r = c + 1; r < k; ++r) {
      const double f = A[r * k + c] / A[c * k + c];
      for (int j = c; j < k; ++j) A[r * k + j] -= f * A[c * k + j];
      b[r] -= f * b[c];
    }
  }
  for (int r = k - 1; r >= 0; --r) {
    double acc = b[r];
    for (int j = r + 1; j < k; ++j) acc -= A[r * k + j] * b[j];
    b[r] = acc / A[r * k + r];
  }
  return true;
}

struct MmaArrays {
  double *alfa, *beta, *p0, *q0, *x, *xsi, *eta, *xo, *xsio, *etao, *dx, *dxsi, *deta, *delx, *diagx, *P, *Q;
  double *partials, *red;
};

static MmaArrays mma_carve(void* ws, int64_t n, int m) {
  char* p = static_cast<char*>(ws);
  const size_t vb = mma_al(sizeof(double) * (size_t)n);
  MmaArrays a;
  double** one[] = {&a.alfa, &a.beta, &a.p0, &a.q0, &a.x, &a.xsi, &a.eta, &a.xo, &a.xsio, &a.etao,
                    &a.dx, &a.dxsi, &a.deta, &a.delx, &a.diagx};
  for (double** q : one) { *q = reinterpret_cast<double*>(p); p += vb; }
  a.P = reinterpret_cast<double*>(p); p += vb * m;
  a.Q = reinterpret_cast<double*>(p); p += vb * m;
  a.partials = reinterpret_cast<double*>(p); p += mma_al(sizeof(double) * (size_t)MMA_MAX_BLOCKS * MMA_MAXK);
  a.red = reinterpret_cast<double*>(p);
  return a;
}

template <int M>
static int mma_update_impl(int64_t n, int iter, const double* xval, const double* xold1, const double* xold2,
                           double* low, double* upp, const double* xmin, const double* xmax, double move,
                           const double* df0dx, const double* fval, const double* dfdx, double a0, const double* a,
                           const double* c, const double* d, double* xmma, void* ws, int32_t* newton_steps,
                           cudaStream_t s) {
  const MmaArrays w = mma_carve(ws, n, M);
  int g = grid_for(n, MMA_THREADS, 8);
  if (g > MMA_MAX_BLOCKS) g = MMA_MAX_BLOCKS;
  double host[MMA_MAXK];
  auto reduce = [&](int ks, int km) -> int {
    mma_reduce_kernel<<<1, MMA_THREADS, 0, s>>>(w.partials, g, ks, km, w.red);
    note_launches(1);
    FEM_CUDA(cudaMemcpyAsync(host, w.red, sizeof(double) * (ks + km), cudaMemcpyDeviceToHost, s));
    FEM_CUDA(cudaStreamSynchronize(s));
    return check_launch("mma kernels");
  };
  mma_setup_kernel<M><<<g, MMA_THREADS, 0, s>>>(n, iter, xval, xold1, xold2, low, upp, xmin, xmax, move, df0dx, dfdx,
                                                w.alfa, w.beta, w.p0, w.q0, w.P, w.Q, w.x, w.xsi, w.eta, w.partials);
  note_launches(1);
  int rc = reduce(M, 0);
  if (rc) return rc;
  double b[M];
  for (int j = 0; j < M; ++j) b[j] = host[j] - fval[j];
  // dual variables of subsolv (mma.py:216-224)
  double y[M], lam[M], mu[M], sv[M], z = 1.0, zet = 1.0;
  for (int j = 0; j < M; ++j) { y[j] = 1.0; lam[j] = 1.0; mu[j] = std::fmax(1.0, 0.5 * c[j]); sv[j] = 1.0; }
  MmaScal sc{};
  int total_newton = 0;
  // residual norm and max of the full KKT residual: per-variable parts from the GPU, the rest here
  auto residual = [&](int trial, double steg, double epsi, const double* yv, double zv, const double* lv,
                      const double* muv, double zetv, const double* sv_, double& rnorm, double& rmax) -> int {
    for (int j = 0; j < M; ++j) sc.lam[j] = lv[j];
    sc.epsi = epsi;
    sc.steg = steg;
    mma_residual_kernel<M><<<g, MMA_THREADS, 0, s>>>(n, trial, sc, low, upp, w.alfa, w.beta, w.p0, w.q0, w.P, w.Q,
                                                     w.x, w.xsi, w.eta, w.xo, w.xsio, w.etao, w.dx, w.dxsi, w.deta,
                                                     w.partials);
    note_launches(1);
    const int r2 = reduce(M + 3, 1);
    if (r2) return r2;
    double ss = host[0] + host[1] + host[2], mx = host[M + 3];
    double al = 0.0;
    for (int j = 0; j < M; ++j) al += a[j] * lv[j];
    auto acc = [&](double r) { ss += r * r; mx = std::fmax(mx, std::fabs(r)); };
    for (int j = 0; j < M; ++j) acc(c[j] + d[j] * yv[j] - muv[j] - lv[j]);          // rey
    acc(a0 - zetv - al);                                                               // rez
    for (int j = 0; j < M; ++j) acc(host[3 + j] - a[j] * zv - yv[j] + sv_[j] - b[j]);  // relam
    for (int j = 0; j < M; ++j) acc(muv[j] * yv[j] - epsi);                            // remu
    acc(zetv * zv - epsi);                                                             // rezet
    for (int j = 0; j < M; ++j) acc(lv[j] * sv_[j] - epsi);                            // res
    rnorm = std::sqrt(ss);
    rmax = mx;
    return FEM_OK;
  };
  double epsi = 1.0;
  while (epsi > 1e-7) {
    double rnorm, rmax;
    rc = residual(0, 0.0, epsi, y, z, lam, mu, zet, sv, rnorm, rmax);
    if (rc) return rc;
    int it = 0;
    while (rmax > 0.9 * epsi && it < 200) {
      ++it;
      ++total_newton;
      for (int j = 0; j < M; ++j) sc.lam[j] = lam[j];
      sc.epsi = epsi;
      mma_newton_kernel<M><<<g, MMA_THREADS, 0, s>>>(n, sc, low, upp, w.alfa, w.beta, w.p0, w.q0, w.P, w.Q, w.x,
                                                     w.xsi, w.eta, w.delx, w.diagx, w.partials);
      note_launches(1);
      constexpr int NA = M * (M + 1) / 2;
      rc = reduce(2 * M + NA, 0);
      if (rc) return rc;
      double al = 0.0;
      for (int j = 0; j < M; ++j) al += a[j] * lam[j];
      double dely[M], dellam[M], diagy[M], dly[M];
      const double delz = a0 - al - epsi / z;
      std::vector<double> AA((M + 1) * (M + 1), 0.0), rhs(M + 1, 0.0);
      int k = 2 * M;
      for (int j = 0; j < M; ++j)
        for (int l = j; l < M; ++l) {
          AA[j * (M + 1) + l] = host[k];
          AA[l * (M + 1) + j] = host[k];
          ++k;
        }
      for (int j = 0; j < M; ++j) {
        dely[j] = c[j] + d[j] * y[j] - lam[j] - epsi / y[j];
        dellam[j] = host[j] - a[j] * z - y[j] - b[j] + epsi / lam[j];
        diagy[j] = d[j] + mu[j] / y[j];
        dly[j] = sv[j] / lam[j] + 1.0 / diagy[j];
        AA[j * (M + 1) + j] += dly[j];
        AA[j * (M + 1) + M] = a[j];
        AA[M * (M + 1) + j] = a[j];
        rhs[j] = dellam[j] + dely[j] / diagy[j] - host[M + j];
      }
      AA[M * (M + 1) + M] = -zet / z;
      rhs[M] = delz;
      if (!small_solve(AA, rhs, M + 1)) return fail(FEM_ERR_DEVICE, "MMA: singular reduced Newton system");
      double dlam[M], dy[M], dmu[M], ds[M];
      const double dz = rhs[M];
      double stm = 1.0;
      for (int j = 0; j < M; ++j) {
        dlam[j] = rhs[j];
        dy[j] = -dely[j] / diagy[j] + dlam[j] / diagy[j];
        dmu[j] = -mu[j] + epsi / y[j] - mu[j] * dy[j] / y[j];
        ds[j] = -sv[j] + epsi / lam[j] - sv[j] * dlam[j] / lam[j];
        stm = std::fmax(stm, std::fmax(std::fmax(-1.01 * dy[j] / y[j], -1.01 * dlam[j] / lam[j]),
                                       std::fmax(-1.01 * dmu[j] / mu[j], -1.01 * ds[j] / sv[j])));
      }
      const double dzet = -zet + epsi / z - zet * dz / z;
      stm = std::fmax(stm, std::fmax(-1.01 * dz / z, -1.01 * dzet / zet));
      for (int j = 0; j < M; ++j) sc.dlam[j] = dlam[j];
      mma_direction_kernel<M><<<g, MMA_THREADS, 0, s>>>(n, sc, low, upp, w.alfa, w.beta, w.P, w.Q, w.x, w.xsi, w.eta,
                                                        w.delx, w.diagx, w.dx, w.dxsi, w.deta, w.xo, w.xsio, w.etao,
                                                        w.partials);
      note_launches(1);
      rc = reduce(0, 1);
      if (rc) return rc;
      stm = std::fmax(stm, host[0]);
      double steg = 1.0 / stm;
      double yo[M], lamo[M], muo[M], so[M];
      for (int j = 0; j < M; ++j) { yo[j] = y[j]; lamo[j] = lam[j]; muo[j] = mu[j]; so[j] = sv[j]; }
      const double zo = z, zeto = zet;
      double resinew = 2.0 * rnorm;
      int tries = 0;
      while (resinew > rnorm && tries < 50) {
        ++tries;
        for (int j = 0; j < M; ++j) {
          y[j] = yo[j] + steg * dy[j];
          lam[j] = lamo[j] + steg * dlam[j];
          mu[j] = muo[j] + steg * dmu[j];
          sv[j] = so[j] + steg * ds[j];
        }
        z = zo + steg * dz;
        zet = zeto + steg * dzet;
        rc = residual(1, steg, epsi, y, z, lam, mu, zet, sv, resinew, rmax);
        if (rc) return rc;
        steg *= 0.5;
      }
      rnorm = resinew;
    }
    epsi *= 0.1;
  }
  FEM_CUDA(cudaMemcpyAsync(xmma, w.x, sizeof(double) * (size_t)n, cudaMemcpyDeviceToDevice, s));
  if (newton_steps) *newton_steps = total_newton;
  return FEM_OK;
}

}  // namespace fem

using namespace fem;

extern "C" int fem_mma_workspace(int64_t n, int32_t m, size_t* bytes) {
  FEM_REQUIRE(bytes && n > 0 && m >= 1 && m <= MMA_MAXM, "need n > 0 and 1 <= m <= 4");
  *bytes = mma_ws_bytes(n, m);
  return FEM_OK;
}

extern "C" int fem_mma_update(int64_t n, int32_t m, int32_t iter, const double* xval, const double* xold1,
                              const double* xold2, double* low, double* upp, const double* xmin, const double* xmax,
                              double move, const double* df0dx, const double* fval, const double* dfdx, double a0,
                              const double* a, const double* c, const double* d, double* xmma, void* ws,
                              size_t ws_bytes, int32_t* newton_steps, void* stream) {
  FEM_REQUIRE(n > m && m >= 1 && m <= MMA_MAXM, "need 1 <= m <= 4 and n > m");
  FEM_REQUIRE(xval && xold1 && xold2 && low && upp && xmin && xmax && df0dx && dfdx && xmma && ws, "NULL argument");
  FEM_REQUIRE(fval && a && c && d, "NULL host argument (fval, a, c, d)");
  FEM_REQUIRE(ws_bytes >= mma_ws_bytes(n, m), "workspace too small");
  cudaStream_t s = as_stream(stream);
  switch (m) {
    case 1: return mma_update_impl<1>(n, iter, xval, xold1, xold2, low, upp, xmin, xmax, move, df0dx, fval, dfdx, a0, a, c, d, xmma, ws, newton_steps, s);
    case 2: return mma_update_impl<2>(n, iter, xval, xold1, xold2, low, upp, xmin, xmax, move, df0dx, fval, dfdx, a0, a, c, d, xmma, ws, newton_steps, s);
    case 3: return mma_update_impl<3>(n, iter, xval, xold1, xold2, low, upp, xmin, xmax, move, df0dx, fval, dfdx, a0, a, c, d, xmma, ws, newton_steps, s);
    default: return mma_update_impl<4>(n, iter, xval, xold1, xold2, low, upp, xmin, xmax, move, df0dx, fval, dfdx, a0, a, c, d, xmma, ws, newton_steps, s);
  }
}

// ---- sensitivity / density filter (mma.py:27-66) --------------------------------------
// H[i, j] = max(rmin - |c_i - c_j|, 0) over the nnb nearest centroids of c_i, Hs = row sums.
// Only neighbours closer than rmin carry weight, so the search is a radius search on a uniform
// grid of bins no smaller than rmin (27 neighbouring bins), keeping the nnb nearest by
// (distance, index).  Rows are stored ELL-style: nnb slots per row, unused slots col = -1.
namespace fem {

constexpr int FILTER_MAX_NB = 32;

__global__ void filter_bbox_kernel(int64_t n, const double* __restrict__ c, double* partials) {
  double v[6] = {-INFINITY, -INFINITY, -INFINITY, -INFINITY, -INFINITY, -INFINITY};
  MMA_LOOP(i, n) {
    for (int d = 0; d < 3; ++d) {
      v[d] = fmax(v[d], -c[i * 3 + d]);
      v[3 + d] = fmax(v[3 + d], c[i * 3 + d]);
    }
  }
  mma_block_store<0, 6>(v, partials);
}

struct BinGrid {
  double lo[3];
  double h;
  int nb[3];
};

__device__ __forceinline__ int bin_coord(double x, double lo, double h, int nb) {
  int b = (int)floor((x - lo) / h);
  return b < 0 ? 0 : (b >= nb ? nb - 1 : b);
}

__global__ void filter_count_kernel(int64_t n, const double* __restrict__ c, BinGrid g, int* __restrict__ cnt,
                                    int* __restrict__ bin_of) {
  MMA_LOOP(i, n) {
    const int bx = bin_coord(c[i * 3], g.lo[0], g.h, g.nb[0]);
    const int by = bin_coord(c[i * 3 + 1], g.lo[1], g.h, g.nb[1]);
    const int bz = bin_coord(c[i * 3 + 2], g.lo[2], g.h, g.nb[2]);
    const int b = (bx * g.nb[1] + by) * g.nb[2] + bz;
    bin_of[i] = b;
    atomicAdd(cnt + b, 1);
  }
}

// Exclusive scan of nb ints by one CTA (set-up only): contiguous chunks per thread.
__global__ void filter_scan_kernel(const int* __restrict__ cnt, int nb, int* __restrict__ start,
                                   int* __restrict__ cursor) {
  __shared__ int part[1024];
  const int t = threadIdx.x, T = blockDim.x;
  const int chunk = (nb + T - 1) / T;
  const int b0 = t * chunk, b1 = min(nb, b0 + chunk);
  int s = 0;
  for (int b = b0; b < b1; ++b) s += cnt[b];
  part[t] = s;
  __syncthreads();
  if (t == 0) {
    int acc = 0;
    for (int k = 0; k < T; ++k) { const int v = part[k]; part[k] = acc; acc += v; }
    start[nb] = acc;
  }
  __syncthreads();
  int acc = part[t];
  for (int b = b0; b < b1; ++b) { start[b] = acc; cursor[b] = acc; acc += cnt[b]; }
}

__global__ void filter_fill_kernel(int64_t n, const int* __restrict__ bin_of, int* __restrict__ cursor,
                                   int* __restrict__ order) {
  MMA_LOOP(i, n) order[atomicAdd(cursor + bin_of[i], 1)] = (int)i;
}

__global__ void filter_query_kernel(int64_t n, const double* __restrict__ c, BinGrid g, double rmin, int nnb,
                                    const int* __restrict__ start, const int* __restrict__ order,
                                    const int* __restrict__ bin_of, int* __restrict__ cols,
                                    double* __restrict__ vals, double* __restrict__ hs) {
  MMA_LOOP(i, n) {
    double bd[FILTER_MAX_NB];
    int bj[FILTER_MAX_NB];
    int cntk = 0;
    const double xi = c[i * 3], yi = c[i * 3 + 1], zi = c[i * 3 + 2];
    const int b = bin_of[i];
    const int bz = b % g.nb[2], by = (b / g.nb[2]) % g.nb[1], bx = b / (g.nb[2] * g.nb[1]);
    for (int ox = -1; ox <= 1; ++ox) {
      const int X = bx + ox;
      if (X < 0 || X >= g.nb[0]) continue;
      for (int oy = -1; oy <= 1; ++oy) {
        const int Y = by + oy;
        if (Y < 0 || Y >= g.nb[1]) continue;
        for (int oz = -1; oz <= 1; ++oz) {
          const int Z = bz + oz;
          if (Z < 0 || Z >= g.nb[2]) continue;
          const int nbin = (X * g.nb[1] + Y) * g.nb[2] + Z;
          for (int p = start[nbin]; p < start[nbin + 1]; ++p) {
            const int j = order[p];
            const double dx = c[(int64_t)j * 3] - xi, dy = c[(int64_t)j * 3 + 1] - yi, dz = c[(int64_t)j * 3 + 2] - zi;
            const double d = sqrt(dx * dx + dy * dy + dz * dz);
            if (!(d < rmin)) continue;
            // insert (d, j) into the sorted list of the nnb nearest
            if (cntk == nnb && (d > bd[cntk - 1] || (d == bd[cntk - 1] && j > bj[cntk - 1]))) continue;
            int q = cntk < nnb ? cntk++ : nnb - 1;
            while (q > 0 && (bd[q - 1] > d || (bd[q - 1] == d && bj[q - 1] > j))) {
              bd[q] = bd[q - 1];
              bj[q] = bj[q - 1];
              --q;
            }
            bd[q] = d;
            bj[q] = j;
          }
        }
      }
    }
    double sum = 0.0;
    for (int k = 0; k < nnb; ++k) {
      if (k < cntk) {
        const double wv = rmin - bd[k];
        cols[i * nnb + k] = bj[k];
        vals[i * nnb + k] = wv;
        sum += wv;
      } else {
        cols[i * nnb + k] = -1;
        vals[i * nnb + k] = 0.0;
      }
    }
    hs[i] = sum;
  }
}

// mode 0 (sensitivity, mma.py:59-62): out_r[i] = sum_k H[i,k] rho_c g_r[c] / max(1e-3, rho_c) / Hs[c]
// mode 1 (density, mma.py:64-66):     out_r[i] = sum_k H[i,k] g_r[c] / Hs[i]
__global__ void filter_apply_kernel(int64_t n, int nnb, const int* __restrict__ cols, const double* __restrict__ vals,
                                    const double* __restrict__ hs, const double* __restrict__ rho,
                                    const double* __restrict__ g, int nr, int mode, double* __restrict__ out) {
  MMA_LOOP(i, n) {
    for (int r = 0; r < nr; ++r) {
      const double* gr = g + (int64_t)r * n;
      double acc = 0.0;
      for (int k = 0; k < nnb; ++k) {
        const int cidx = cols[i * nnb + k];
        if (cidx < 0) continue;
        const double wv = vals[i * nnb + k];
        if (mode == 0) {
          const double rc = rho[cidx];
          acc += wv * (rc * gr[cidx] / fmax(1e-3, rc) / hs[cidx]);
        } else {
          acc += wv * gr[cidx];
        }
      }
      out[(int64_t)r * n + i] = mode == 0 ? acc : acc / hs[i];
    }
  }
}

static size_t filter_ws_bytes(int64_t n) {
  const size_t nbmax = (size_t)(4 * n + 64);
  return mma_al(sizeof(int) * (nbmax + 1)) * 3 + mma_al(sizeof(int) * (size_t)n) * 2 +
         mma_al(sizeof(double) * (size_t)MMA_MAX_BLOCKS * 6) + mma_al(sizeof(double) * 8);
}

}  // namespace fem

extern "C" int fem_filter_workspace(int64_t n, size_t* bytes) {
  FEM_REQUIRE(bytes && n > 0, "bad arguments");
  *bytes = filter_ws_bytes(n);
  return FEM_OK;
}

extern "C" int fem_filter_build(int64_t n, const double* centroids, double rmin, int32_t nnb, int32_t* cols,
                                double* vals, double* hs, void* ws, size_t ws_bytes, void* stream) {
  FEM_REQUIRE(n > 0 && centroids && cols && vals && hs && ws, "NULL argument");
  FEM_REQUIRE(nnb >= 1 && nnb <= FILTER_MAX_NB, "nnb must be in 1..32");
  FEM_REQUIRE(rmin > 0.0 && std::isfinite(rmin), "rmin must be positive");
  FEM_REQUIRE(n < ((int64_t)1 << 29), "filter supports < 2^29 design cells");
  FEM_REQUIRE(ws_bytes >= filter_ws_bytes(n), "workspace too small");
  cudaStream_t s = as_stream(stream);
  const size_t nbmax = (size_t)(4 * n + 64);
  char* p = static_cast<char*>(ws);
  int* cnt = reinterpret_cast<int*>(p); p += mma_al(sizeof(int) * (nbmax + 1));
  int* start = reinterpret_cast<int*>(p); p += mma_al(sizeof(int) * (nbmax + 1));
  int* cursor = reinterpret_cast<int*>(p); p += mma_al(sizeof(int) * (nbmax + 1));
  int* order = reinterpret_cast<int*>(p); p += mma_al(sizeof(int) * (size_t)n);
  int* bin_of = reinterpret_cast<int*>(p); p += mma_al(sizeof(int) * (size_t)n);
  double* partials = reinterpret_cast<double*>(p); p += mma_al(sizeof(double) * (size_t)MMA_MAX_BLOCKS * 6);
  double* red = reinterpret_cast<double*>(p);
  int gsz = grid_for(n, MMA_THREADS, 8);
  if (gsz > MMA_MAX_BLOCKS) gsz = MMA_MAX_BLOCKS;
  filter_bbox_kernel<<<gsz, MMA_THREADS, 0, s>>>(n, centroids, partials);
  mma_reduce_kernel<<<1, MMA_THREADS, 0, s>>>(partials, gsz, 0, 6, red);
  note_launches(2);
  double bb[6];
  FEM_CUDA(cudaMemcpyAsync(bb, red, sizeof(bb), cudaMemcpyDeviceToHost, s));
  FEM_CUDA(cudaStreamSynchronize(s));
  int rc = check_launch("filter bbox");
  if (rc) return rc;
  BinGrid g;
  g.h = rmin;
  for (int d = 0; d < 3; ++d) g.lo[d] = -bb[d];
  for (;;) {
    size_t B = 1;
    for (int d = 0; d < 3; ++d) {
      g.nb[d] = (int)std::floor((bb[3 + d] + bb[d]) / g.h) + 1;
      B *= (size_t)g.nb[d];
    }
    if (B <= nbmax) break;
    g.h *= 1.26;  // coarser bins keep the 27-bin neighbourhood valid (bin size >= rmin)
  }
  const int B = g.nb[0] * g.nb[1] * g.nb[2];
  FEM_CUDA(cudaMemsetAsync(cnt, 0, sizeof(int) * (size_t)B, s));
  filter_count_kernel<<<gsz, MMA_THREADS, 0, s>>>(n, centroids, g, cnt, bin_of);
  filter_scan_kernel<<<1, 1024, 0, s>>>(cnt, B, start, cursor);
  filter_fill_kernel<<<gsz, MMA_THREADS, 0, s>>>(n, bin_of, cursor, order);
  filter_query_kernel<<<gsz, MMA_THREADS, 0, s>>>(n, centroids, g, rmin, nnb, start, order, bin_of, cols, vals, hs);
  note_launches(4);
  return check_launch("filter build");
}

extern "C" int fem_filter_apply(int64_t n, int32_t nnb, const int32_t* cols, const double* vals, const double* hs,
                                const double* rho, const double* g, int32_t nr, int32_t mode, double* out,
                                void* stream) {
  FEM_REQUIRE(n > 0 && cols && vals && hs && g && out && nr >= 1, "NULL argument");
  FEM_REQUIRE(mode == 0 || mode == 1, "mode must be 0 (sensitivity) or 1 (density)");
  FEM_REQUIRE(mode == 1 || rho, "sensitivity filtering needs rho");
  FEM_REQUIRE(nnb >= 1 && nnb <= FILTER_MAX_NB, "nnb must be in 1..32");
  cudaStream_t s = as_stream(stream);
  filter_apply_kernel<<<grid_for(n, MMA_THREADS, 8), MMA_THREADS, 0, s>>>(n, nnb, cols, vals, hs, rho, g, nr, mode,
                                                                           out);
  note_launches(1);
  return check_launch("filter apply");
}
