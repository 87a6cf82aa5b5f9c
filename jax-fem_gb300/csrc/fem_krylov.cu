// Sparse linear algebra on the node-block CSR: SpMV, Dirichlet row handling,
// Jacobi / block-Jacobi preconditioners, PCG and BiCGStab.
//
// Matrix layout: values in scalar CSR order (row-major, columns sorted); the
// column indices are implicit in the node-block structure -- every node row
// i owns nb_i block columns block_cols[block_ptr[i]..] and each of its vec
// scalar rows holds vec*nb_i consecutive values.  SpMV therefore streams the
// values once and reads one 4-byte block column per vec*vec values instead of
// one per value (the reference's BCOO stores two 8-byte indices per value).
//
// Solvers run as a host loop of stream-ordered kernels.  Every kernel starts by
// reading the control block's `done` word and returns at once when it is set;
// FP64 dot products are reduced per CTA and finished by the last CTA (atomic
// ticket), which also performs the scalar recurrences (alpha, beta, omega,
// convergence test), so the iteration stops on the device at exactly the
// first iteration meeting the criterion.  The host polls `done` every CHUNK
// iterations; no kernel ever waits on another.
#include <cmath>

#include "fem_common.cuh"
#include "fem_elements.cuh"

namespace fem {

constexpr int VTHREADS = 256;      // vector kernels
constexpr int SPMV_THREADS = 256;  // 8 warps = 8 node rows per CTA
constexpr int MAX_PARTIAL_BLOCKS = 8192;
constexpr int CHUNK = 16;

struct KCtl {
  double rho, rho_prev, alpha, beta, omega, thresh2, rr, bb, d0, d1, ss;
  long long iter, maxiter;
  int done, status, exit_early, pad;
  unsigned int ticket[4];
};

enum { FIN_NONE = 0, FIN_PCG_INIT, FIN_PCG_ALPHA, FIN_PCG_UPDATE, FIN_BICG_INIT, FIN_BICG_ALPHA, FIN_BICG_S,
       FIN_BICG_OMEGA, FIN_BICG_UPDATE, FIN_DOT };

__device__ __forceinline__ bool finite(double v) { return isfinite(v); }

// Scalar recurrences run by the last CTA of a reducing kernel.
__device__ void finalize(KCtl* C, int op, const double (&d)[3], double* dot_out) {
  switch (op) {
    case FIN_PCG_INIT:  // d = (r.z, r.r, b.b)
      C->rho = d[0];
      C->rr = d[1];
      C->bb = d[2];
      C->iter = 0;
      C->status = FEM_SOLVE_CONVERGED;
      C->thresh2 = fmax(C->thresh2 * d[2], C->d1);  // thresh2 held rtol^2, d1 held atol^2
      if (!finite(d[0]) || !finite(d[1])) { C->status = FEM_SOLVE_NAN; C->done = 1; }
      else if (d[1] <= C->thresh2) C->done = 1;
      else if (C->maxiter <= 0) { C->status = FEM_SOLVE_MAXITER; C->done = 1; }
      break;
    case FIN_PCG_ALPHA:  // d0 = p.q
      C->d0 = d[0];
      if (!(d[0] > 0.0) || !finite(d[0])) { C->status = finite(d[0]) ? FEM_SOLVE_BREAKDOWN : FEM_SOLVE_NAN; C->done = 1; }
      else C->alpha = C->rho / d[0];
      break;
    case FIN_PCG_UPDATE: {  // d = (r.z, r.r)
      C->iter += 1;
      C->rr = d[1];
      if (!finite(d[0]) || !finite(d[1])) { C->status = FEM_SOLVE_NAN; C->done = 1; break; }
      if (d[1] <= C->thresh2) { C->status = FEM_SOLVE_CONVERGED; C->done = 1; break; }
      if (C->iter >= C->maxiter) { C->status = FEM_SOLVE_MAXITER; C->done = 1; break; }
      C->beta = d[0] / C->rho;
      C->rho = d[0];
      break;
    }
    case FIN_BICG_INIT:  // d = (r.r, b.b, rhat.r); jax: atol2 = max(tol^2 b.b, atol^2)
      C->rr = d[0];
      C->bb = d[1];
      C->thresh2 = fmax(C->thresh2 * d[1], C->d1);
      C->rho_prev = 1.0; C->alpha = 1.0; C->omega = 1.0;
      C->rho = d[2];
      C->iter = 0;
      C->status = FEM_SOLVE_CONVERGED;
      if (!finite(d[0])) { C->status = FEM_SOLVE_NAN; C->done = 1; }
      else if (d[0] <= C->thresh2) C->done = 1;
      else if (C->maxiter <= 0) { C->status = FEM_SOLVE_MAXITER; C->done = 1; }
      else if (C->rho == 0.0) { C->status = FEM_SOLVE_BREAKDOWN; C->done = 1; }
      else C->beta = C->rho / C->rho_prev * C->alpha / C->omega;
      break;
    case FIN_BICG_ALPHA:  // d0 = rhat.q
      C->alpha = C->rho / d[0];
      if (!finite(C->alpha)) { C->status = FEM_SOLVE_BREAKDOWN; C->done = 1; }
      break;
    case FIN_BICG_S:  // d0 = s.s
      C->ss = d[0];
      C->exit_early = (d[0] < C->thresh2) ? 1 : 0;
      break;
    case FIN_BICG_OMEGA:  // d = (t.s, t.t)
      C->omega = d[0] / d[1];
      if (C->exit_early) C->omega = 0.0;
      break;
    case FIN_BICG_UPDATE: {  // d = (r.r, rhat.r)
      C->iter += 1;
      C->rr = d[0];
      if (!finite(d[0])) { C->status = FEM_SOLVE_NAN; C->done = 1; break; }
      if (!C->exit_early && (C->omega == 0.0 || C->alpha == 0.0)) { C->status = FEM_SOLVE_BREAKDOWN; C->done = 1; break; }
      if (d[0] <= C->thresh2) { C->status = FEM_SOLVE_CONVERGED; C->done = 1; break; }
      if (C->iter >= C->maxiter) { C->status = FEM_SOLVE_MAXITER; C->done = 1; break; }
      C->rho_prev = C->rho;
      C->rho = d[1];
      if (C->rho == 0.0) { C->status = FEM_SOLVE_BREAKDOWN; C->done = 1; break; }
      C->beta = C->rho / C->rho_prev * C->alpha / C->omega;
      break;
    }
    case FIN_DOT:
      *dot_out = d[0];
      break;
    default:
      break;
  }
}

// Per-CTA partial sums of up to 3 dots, last CTA finalizes.
template <int ND>
__device__ __forceinline__ void reduce_and_finalize(double (&v)[3], KCtl* C, int op, double* partials,
                                                    unsigned* ticket, double* dot_out) {
  __shared__ double sh[3 * 32];
  double w[ND];
#pragma unroll
  for (int k = 0; k < ND; ++k) w[k] = v[k];
  block_sum<ND>(w, sh);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < ND; ++k) partials[(size_t)blockIdx.x * 3 + k] = w[k];
  }
  if (last_block_ticket(ticket)) {
    double tot[3] = {0, 0, 0};
    // partials are strided by 3: each thread sums a block-ordered subset, then a fixed tree
    double acc[ND];
#pragma unroll
    for (int k = 0; k < ND; ++k) acc[k] = 0.0;
    for (unsigned b = threadIdx.x; b < gridDim.x; b += blockDim.x) {
      const volatile double* p = partials + (size_t)b * 3;
#pragma unroll
      for (int k = 0; k < ND; ++k) acc[k] += p[k];
    }
    block_sum<ND>(acc, sh);
    if (threadIdx.x == 0) {
#pragma unroll
      for (int k = 0; k < ND; ++k) tot[k] = acc[k];
      finalize(C, op, tot, dot_out);
    }
  }
}

// ---- SpMV (warp per node row, lane per block column) -------------------------
// y = A x; optional fused dots d0 = a.y, d1 = y.y and last-CTA finalize op.
template <int VEC, typename T, int ND>
__global__ void __launch_bounds__(SPMV_THREADS) spmv_kernel(int64_t n_nodes, const int64_t* __restrict__ bp,
                                                            const int32_t* __restrict__ bcols,
                                                            const T* __restrict__ vals, const T* __restrict__ x,
                                                            T* __restrict__ y, const T* __restrict__ a, KCtl* C,
                                                            int op, double* partials, int ticket_id) {
  if (C && C->done) return;
  const int lane = threadIdx.x & 31;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  double dv[3] = {0.0, 0.0, 0.0};
  for (int64_t i = warp; i < n_nodes; i += nwarps) {
    const int64_t b0 = bp[i];
    const int nb = (int)(bp[i + 1] - b0);
    const T* vrow = vals + (int64_t)VEC * VEC * b0;
    T acc[VEC];
#pragma unroll
    for (int r = 0; r < VEC; ++r) acc[r] = T(0);
    for (int k = lane; k < nb; k += 32) {
      const int64_t col = bcols[b0 + k];
      T xv[VEC];
#pragma unroll
      for (int d = 0; d < VEC; ++d) xv[d] = __ldg(x + VEC * col + d);
#pragma unroll
      for (int r = 0; r < VEC; ++r) {
        const T* vr = vrow + (int64_t)r * VEC * nb + VEC * k;
#pragma unroll
        for (int d = 0; d < VEC; ++d) acc[r] += __ldcs(vr + d) * xv[d];
      }
    }
#pragma unroll
    for (int r = 0; r < VEC; ++r) acc[r] = warp_sum(acc[r]);
    if (lane < VEC) {
      T out = acc[0];
#pragma unroll
      for (int r = 1; r < VEC; ++r)
        if (lane == r) out = acc[r];
      const int64_t row = (int64_t)VEC * i + lane;
      y[row] = out;
      if constexpr (ND >= 1) dv[0] += double(a[row]) * double(out);
      if constexpr (ND >= 2) dv[1] += double(out) * double(out);
    }
  }
  if constexpr (ND > 0) reduce_and_finalize<ND>(dv, C, op, partials, C->ticket + ticket_id, nullptr);
}

// ---- vector kernels (thread per node) ----------------------------------------
template <int VEC, typename T, int PC>
__device__ __forceinline__ void precond(const T* pc, int64_t i, const T (&r)[VEC], T (&z)[VEC]) {
  if constexpr (PC == FEM_PC_NONE) {
#pragma unroll
    for (int c = 0; c < VEC; ++c) z[c] = r[c];
  } else if constexpr (PC == FEM_PC_JACOBI) {
#pragma unroll
    for (int c = 0; c < VEC; ++c) z[c] = pc[VEC * i + c] * r[c];
  } else {
    const T* B = pc + (int64_t)VEC * VEC * i;
#pragma unroll
    for (int c = 0; c < VEC; ++c) {
      T s = T(0);
#pragma unroll
      for (int d = 0; d < VEC; ++d) s += B[c * VEC + d] * r[d];
      z[c] = s;
    }
  }
}

#define GRID_STRIDE_NODES(i, n) \
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < (n); i += (int64_t)gridDim.x * blockDim.x)

// r = b - Ax (Ax in q), z = M r, p = z ; dots (r.z, r.r, b.b)
template <int VEC, typename T, int PC>
__global__ void pcg_init_kernel(int64_t n_nodes, const T* b, const T* q, T* r, T* z, T* p, const T* pc, KCtl* C,
                                double* partials) {
  double dv[3] = {0, 0, 0};
  GRID_STRIDE_NODES(i, n_nodes) {
    T rv[VEC], zv[VEC];
#pragma unroll
    for (int c = 0; c < VEC; ++c) {
      const T bv = b[VEC * i + c];
      rv[c] = bv - q[VEC * i + c];
      dv[2] += double(bv) * double(bv);
    }
    precond<VEC, T, PC>(pc, i, rv, zv);
#pragma unroll
    for (int c = 0; c < VEC; ++c) {
      r[VEC * i + c] = rv[c];
      z[VEC * i + c] = zv[c];
      p[VEC * i + c] = zv[c];
      dv[0] += double(rv[c]) * double(zv[c]);
      dv[1] += double(rv[c]) * double(rv[c]);
    }
  }
  reduce_and_finalize<3>(dv, C, FIN_PCG_INIT, partials, C->ticket + 1, nullptr);
}

// x += alpha p ; r -= alpha q ; z = M r ; dots (r.z, r.r)
template <int VEC, typename T, int PC>
__global__ void pcg_update_kernel(int64_t n_nodes, T* x, T* r, T* z, const T* p, const T* q, const T* pc, KCtl* C,
                                  double* partials) {
  if (C->done) return;
  const T alpha = T(C->alpha);
  double dv[3] = {0, 0, 0};
  GRID_STRIDE_NODES(i, n_nodes) {
    T rv[VEC], zv[VEC];
#pragma unroll
    for (int c = 0; c < VEC; ++c) {
      const int64_t k = VEC * i + c;
      x[k] += alpha * p[k];
      rv[c] = r[k] - alpha * q[k];
      r[k] = rv[c];
    }
    precond<VEC, T, PC>(pc, i, rv, zv);
#pragma unroll
    for (int c = 0; c < VEC; ++c) {
      z[VEC * i + c] = zv[c];
      dv[0] += double(rv[c]) * double(zv[c]);
      dv[1] += double(rv[c]) * double(rv[c]);
    }
  }
  reduce_and_finalize<2>(dv, C, FIN_PCG_UPDATE, partials, C->ticket + 1, nullptr);
}

template <typename T>
__global__ void pcg_direction_kernel(int64_t n, T* p, const T* z, const KCtl* C) {
  if (C->done) return;
  const T beta = T(C->beta);
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
    p[k] = z[k] + beta * p[k];
}

// BiCGStab (jax.scipy.sparse.linalg.bicgstab iteration).
// init: r = b - Ax (Ax in q), rhat = r, p = r, q = r ; dots (r.r, b.b, rhat.r)
template <typename T>
__global__ void bicg_init_kernel(int64_t n, const T* b, T* q, T* r, T* rhat, T* p, KCtl* C, double* partials) {
  double dv[3] = {0, 0, 0};
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    const T rv = b[k] - q[k];
    r[k] = rv; rhat[k] = rv; p[k] = rv; q[k] = rv;
    dv[0] += double(rv) * double(rv);
    dv[1] += double(b[k]) * double(b[k]);
  }
  dv[2] = dv[0];
  reduce_and_finalize<3>(dv, C, FIN_BICG_INIT, partials, C->ticket + 1, nullptr);
}

// p = r + beta (p - omega q) ; phat = M p
template <int VEC, typename T, int PC>
__global__ void bicg_p_kernel(int64_t n_nodes, const T* r, T* p, const T* q, T* phat, const T* pc, const KCtl* C) {
  if (C->done) return;
  const T beta = T(C->beta), omega = T(C->omega);
  GRID_STRIDE_NODES(i, n_nodes) {
    T pv[VEC], ph[VEC];
#pragma unroll
    for (int c = 0; c < VEC; ++c) {
      const int64_t k = VEC * i + c;
      pv[c] = r[k] + beta * (p[k] - omega * q[k]);
      p[k] = pv[c];
    }
    precond<VEC, T, PC>(pc, i, pv, ph);
#pragma unroll
    for (int c = 0; c < VEC; ++c) phat[VEC * i + c] = ph[c];
  }
}

// s = r - alpha q ; shat = M s ; dot (s.s)
template <int VEC, typename T, int PC>
__global__ void bicg_s_kernel(int64_t n_nodes, const T* r, const T* q, T* s, T* shat, const T* pc, KCtl* C,
                              double* partials) {
  if (C->done) return;
  const T alpha = T(C->alpha);
  double dv[3] = {0, 0, 0};
  GRID_STRIDE_NODES(i, n_nodes) {
    T sv[VEC], sh[VEC];
#pragma unroll
    for (int c = 0; c < VEC; ++c) {
      const int64_t k = VEC * i + c;
      sv[c] = r[k] - alpha * q[k];
      s[k] = sv[c];
      dv[0] += double(sv[c]) * double(sv[c]);
    }
    precond<VEC, T, PC>(pc, i, sv, sh);
#pragma unroll
    for (int c = 0; c < VEC; ++c) shat[VEC * i + c] = sh[c];
  }
  reduce_and_finalize<1>(dv, C, FIN_BICG_S, partials, C->ticket + 1, nullptr);
}

// x += alpha phat (+ omega shat) ; r = s (- omega t) ; dots (r.r, rhat.r)
template <typename T>
__global__ void bicg_update_kernel(int64_t n, T* x, T* r, const T* rhat, const T* phat, const T* s, const T* shat,
                                   const T* t, KCtl* C, double* partials) {
  if (C->done) return;
  const T alpha = T(C->alpha), omega = T(C->omega);
  const bool early = C->exit_early != 0;
  double dv[3] = {0, 0, 0};
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    T rv;
    if (early) {
      x[k] += alpha * phat[k];
      rv = s[k];
    } else {
      x[k] += alpha * phat[k] + omega * shat[k];
      rv = s[k] - omega * t[k];
    }
    r[k] = rv;
    dv[0] += double(rv) * double(rv);
    dv[1] += double(rhat[k]) * double(rv);
  }
  reduce_and_finalize<2>(dv, C, FIN_BICG_UPDATE, partials, C->ticket + 1, nullptr);
}

template <typename T>
__global__ void dot_kernel(int64_t n, const T* x, const T* y, KCtl* C, double* partials, double* out) {
  double dv[3] = {0, 0, 0};
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
    dv[0] += double(x[k]) * double(y[k]);
  reduce_and_finalize<1>(dv, C, FIN_DOT, partials, C->ticket + 2, out);
}

__global__ void init_ctl_kernel(KCtl* C, double thresh2_rel, double atol2, long long maxiter) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    C->done = 0; C->status = 0; C->exit_early = 0;
    C->thresh2 = thresh2_rel; C->d1 = atol2; C->maxiter = maxiter; C->iter = 0;
    C->ticket[0] = C->ticket[1] = C->ticket[2] = C->ticket[3] = 0;
  }
}

// ---- Dirichlet rows, preconditioner setup, helpers ---------------------------
template <typename T>
__global__ void zero_rows_kernel(int vec, const int64_t* bp, const int64_t* indptr, const int64_t* diag, T* vals,
                                 const int32_t* rows, int64_t n_rows, T dval) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n_rows; k += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = rows[k];
    const int64_t i = r / vec;
    const int64_t len = (int64_t)vec * (bp[i + 1] - bp[i]);
    T* v = vals + indptr[r];
    for (int64_t j = 0; j < len; ++j) v[j] = T(0);
    vals[diag[r]] = dval;
  }
}

__global__ void apply_bc_vec_kernel(double* res, const double* dofs, const int32_t* rows, const double* values,
                                    int64_t n, double scale) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = rows[k];
    res[r] = dofs[r] - values[k] * scale;
  }
}

template <int VEC, typename T>
__global__ void precond_setup_kernel(int64_t n_nodes, const int64_t* bp, const int32_t* bcols, const T* vals,
                                     int kind, T* pc) {
  GRID_STRIDE_NODES(i, n_nodes) {
    const int64_t b0 = bp[i];
    const int nb = (int)(bp[i + 1] - b0);
    int kd = 0;
    for (int k = 0; k < nb; ++k)
      if (bcols[b0 + k] == i) { kd = k; break; }
    double B[VEC][VEC];
    for (int r = 0; r < VEC; ++r)
      for (int c = 0; c < VEC; ++c) B[r][c] = double(vals[(int64_t)VEC * VEC * b0 + (int64_t)r * VEC * nb + VEC * kd + c]);
    if (kind == FEM_PC_JACOBI) {
      for (int r = 0; r < VEC; ++r) pc[VEC * i + r] = T(1.0 / B[r][r]);
    } else {
      if constexpr (VEC == 1) {
        pc[i] = T(1.0 / B[0][0]);
      } else {
        double Bi[3][3];
        inv3<double>(B, det3<double>(B), Bi);
        for (int r = 0; r < 3; ++r)
          for (int c = 0; c < 3; ++c) pc[9 * i + r * 3 + c] = T(Bi[r][c]);
      }
    }
  }
}

__global__ void cast_kernel(const double* src, float* dst, int64_t n, const uint8_t* mask) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
    dst[k] = (mask && mask[k]) ? 0.0f : (float)src[k];
}

__global__ void axpy_kernel(double alpha, const float* x, double* y, int64_t n) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
    y[k] += alpha * (double)x[k];
}

// ---- workspace ----------------------------------------------------------------
static size_t al(size_t x) { return (x + 255) & ~size_t(255); }

struct KWs {
  KCtl* ctl;
  double* partials;
  char* vecs;
  size_t vec_bytes;
};

static size_t krylov_ws_bytes(int64_t n_dofs, int precision) {
  const size_t es = precision == FEM_F32 ? 4 : 8;
  return al(sizeof(KCtl)) + al(sizeof(double) * 3 * MAX_PARTIAL_BLOCKS) + 8 * al(es * (size_t)n_dofs);
}

static KWs carve(void* ws, int64_t n_dofs, int precision) {
  const size_t es = precision == FEM_F32 ? 4 : 8;
  char* p = static_cast<char*>(ws);
  KWs w;
  w.ctl = reinterpret_cast<KCtl*>(p); p += al(sizeof(KCtl));
  w.partials = reinterpret_cast<double*>(p); p += al(sizeof(double) * 3 * MAX_PARTIAL_BLOCKS);
  w.vecs = p;
  w.vec_bytes = al(es * (size_t)n_dofs);
  return w;
}

static int vec_grid(int64_t n) {
  int g = grid_for(n, VTHREADS, 4);
  return g > MAX_PARTIAL_BLOCKS ? MAX_PARTIAL_BLOCKS : g;
}

static int spmv_grid(int64_t n_nodes) {
  int g = grid_for(n_nodes * 32, SPMV_THREADS, 8);
  return g > MAX_PARTIAL_BLOCKS ? MAX_PARTIAL_BLOCKS : g;
}

template <int VEC, typename T>
static void launch_spmv(const fem_pattern_t* pat, int64_t n_nodes, const T* vals, const T* x, T* y, const T* a,
                        KCtl* C, int op, double* partials, int nd, cudaStream_t s) {
  const int g = spmv_grid(n_nodes);
  if (nd == 0)
    spmv_kernel<VEC, T, 0><<<g, SPMV_THREADS, 0, s>>>(n_nodes, pat->block_ptr, pat->block_cols, vals, x, y, a, C, op,
                                                      partials, 0);
  else if (nd == 1)
    spmv_kernel<VEC, T, 1><<<g, SPMV_THREADS, 0, s>>>(n_nodes, pat->block_ptr, pat->block_cols, vals, x, y, a, C, op,
                                                      partials, 0);
  else
    spmv_kernel<VEC, T, 2><<<g, SPMV_THREADS, 0, s>>>(n_nodes, pat->block_ptr, pat->block_cols, vals, x, y, a, C, op,
                                                      partials, 0);
  note_launches(1);
}

static int poll(KCtl* C, cudaStream_t s, KCtl* host) {
  FEM_CUDA(cudaMemcpyAsync(host, C, sizeof(KCtl), cudaMemcpyDeviceToHost, s));
  FEM_CUDA(cudaStreamSynchronize(s));
  return FEM_OK;
}

template <int VEC, typename T, int PC>
static int pcg_impl(const fem_pattern_t* pat, int64_t n_nodes, const T* vals, const T* pc, const T* b, T* x,
                    double rtol, double atol, int64_t maxiter, void* ws, int64_t* iters, double* rnorm,
                    int32_t* status, cudaStream_t s) {
  const int64_t n = n_nodes * VEC;
  KWs w = carve(ws, n, sizeof(T) == 4 ? FEM_F32 : FEM_F64);
  T* r = reinterpret_cast<T*>(w.vecs);
  T* z = reinterpret_cast<T*>(w.vecs + w.vec_bytes);
  T* p = reinterpret_cast<T*>(w.vecs + 2 * w.vec_bytes);
  T* q = reinterpret_cast<T*>(w.vecs + 3 * w.vec_bytes);
  KCtl* C = w.ctl;
  init_ctl_kernel<<<1, 32, 0, s>>>(C, rtol * rtol, atol * atol, (long long)maxiter);
  note_launches(1);
  launch_spmv<VEC, T>(pat, n_nodes, vals, x, q, nullptr, nullptr, FIN_NONE, nullptr, 0, s);
  pcg_init_kernel<VEC, T, PC><<<vec_grid(n_nodes), VTHREADS, 0, s>>>(n_nodes, b, q, r, z, p, pc, C, w.partials);
  note_launches(1);
  int rc = check_launch("pcg init");
  if (rc) return rc;
  KCtl h;
  int64_t launched = 0;
  while (true) {
    rc = poll(C, s, &h);
    if (rc) return rc;
    if (h.done || launched >= maxiter) break;
    for (int k = 0; k < CHUNK && launched < maxiter; ++k, ++launched) {
      launch_spmv<VEC, T>(pat, n_nodes, vals, p, q, p, C, FIN_PCG_ALPHA, w.partials, 1, s);
      pcg_update_kernel<VEC, T, PC><<<vec_grid(n_nodes), VTHREADS, 0, s>>>(n_nodes, x, r, z, p, q, pc, C, w.partials);
      note_launches(1);
      pcg_direction_kernel<T><<<vec_grid(n), VTHREADS, 0, s>>>(n, p, z, C);
      note_launches(1);
    }
    rc = check_launch("pcg iteration");
    if (rc) return rc;
  }
  if (iters) *iters = h.iter;
  if (rnorm) *rnorm = std::sqrt(h.rr);
  if (status) *status = h.done ? h.status : FEM_SOLVE_MAXITER;
  return FEM_OK;
}

template <int VEC, typename T, int PC>
static int bicg_impl(const fem_pattern_t* pat, int64_t n_nodes, const T* vals, const T* pc, const T* b, T* x,
                     double tol, double atol, int64_t maxiter, void* ws, int64_t* iters, double* rnorm,
                     int32_t* status, cudaStream_t s) {
  const int64_t n = n_nodes * VEC;
  KWs w = carve(ws, n, sizeof(T) == 4 ? FEM_F32 : FEM_F64);
  T* v[8];
  for (int k = 0; k < 8; ++k) v[k] = reinterpret_cast<T*>(w.vecs + k * w.vec_bytes);
  T *r = v[0], *rhat = v[1], *p = v[2], *phat = v[3], *q = v[4], *sv = v[5], *shat = v[6], *t = v[7];
  KCtl* C = w.ctl;
  init_ctl_kernel<<<1, 32, 0, s>>>(C, tol * tol, atol * atol, (long long)maxiter);
  note_launches(1);
  launch_spmv<VEC, T>(pat, n_nodes, vals, x, q, nullptr, nullptr, FIN_NONE, nullptr, 0, s);
  bicg_init_kernel<T><<<vec_grid(n), VTHREADS, 0, s>>>(n, b, q, r, rhat, p, C, w.partials);
  note_launches(1);
  int rc = check_launch("bicgstab init");
  if (rc) return rc;
  KCtl h;
  int64_t launched = 0;
  while (true) {
    rc = poll(C, s, &h);
    if (rc) return rc;
    if (h.done || launched >= maxiter) break;
    for (int k = 0; k < CHUNK && launched < maxiter; ++k, ++launched) {
      bicg_p_kernel<VEC, T, PC><<<vec_grid(n_nodes), VTHREADS, 0, s>>>(n_nodes, r, p, q, phat, pc, C);
      note_launches(1);
      launch_spmv<VEC, T>(pat, n_nodes, vals, phat, q, rhat, C, FIN_BICG_ALPHA, w.partials, 1, s);
      bicg_s_kernel<VEC, T, PC><<<vec_grid(n_nodes), VTHREADS, 0, s>>>(n_nodes, r, q, sv, shat, pc, C, w.partials);
      note_launches(1);
      launch_spmv<VEC, T>(pat, n_nodes, vals, shat, t, sv, C, FIN_BICG_OMEGA, w.partials, 2, s);
      bicg_update_kernel<T><<<vec_grid(n), VTHREADS, 0, s>>>(n, x, r, rhat, phat, sv, shat, t, C, w.partials);
      note_launches(1);
    }
    rc = check_launch("bicgstab iteration");
    if (rc) return rc;
  }
  if (iters) *iters = h.iter;
  if (rnorm) *rnorm = std::sqrt(h.rr);
  if (status) *status = h.done ? h.status : FEM_SOLVE_MAXITER;
  return FEM_OK;
}

}  // namespace fem

using namespace fem;

static int check_pat(const fem_pattern_t* pat, int64_t n_nodes, int32_t vec, int32_t precision) {
  FEM_REQUIRE(pat && pat->block_ptr && pat->block_cols, "pattern NULL");
  FEM_REQUIRE(n_nodes > 0, "n_nodes must be positive");
  FEM_REQUIRE(vec == 1 || vec == 3, "vec must be 1 or 3");
  FEM_REQUIRE(precision == FEM_F32 || precision == FEM_F64, "bad precision");
  return FEM_OK;
}

extern "C" int fem_spmv(const fem_pattern_t* pat, int64_t n_nodes, int32_t vec, int32_t precision, const void* vals,
                        const void* x, void* y, void* stream) {
  int rc = check_pat(pat, n_nodes, vec, precision);
  if (rc) return rc;
  FEM_REQUIRE(vals && x && y, "NULL vector");
  cudaStream_t s = as_stream(stream);
  if (precision == FEM_F32) {
    if (vec == 3) launch_spmv<3, float>(pat, n_nodes, (const float*)vals, (const float*)x, (float*)y, nullptr, nullptr, 0, nullptr, 0, s);
    else launch_spmv<1, float>(pat, n_nodes, (const float*)vals, (const float*)x, (float*)y, nullptr, nullptr, 0, nullptr, 0, s);
  } else {
    if (vec == 3) launch_spmv<3, double>(pat, n_nodes, (const double*)vals, (const double*)x, (double*)y, nullptr, nullptr, 0, nullptr, 0, s);
    else launch_spmv<1, double>(pat, n_nodes, (const double*)vals, (const double*)x, (double*)y, nullptr, nullptr, 0, nullptr, 0, s);
  }
  return check_launch("spmv");
}

extern "C" int fem_zero_rows(const fem_pattern_t* pat, int32_t vec, int32_t precision, void* vals, const int32_t* rows,
                             int64_t n_rows, double diag_value, void* stream) {
  FEM_REQUIRE(pat && pat->block_ptr && pat->indptr && pat->diag && vals, "pattern/vals NULL");
  FEM_REQUIRE(vec == 1 || vec == 3, "vec must be 1 or 3");
  FEM_REQUIRE(n_rows >= 0 && (n_rows == 0 || rows), "rows NULL");
  if (n_rows == 0) return FEM_OK;
  cudaStream_t s = as_stream(stream);
  if (precision == FEM_F32)
    zero_rows_kernel<float><<<grid_for(n_rows, 128), 128, 0, s>>>(vec, pat->block_ptr, pat->indptr, pat->diag,
                                                                  (float*)vals, rows, n_rows, (float)diag_value);
  else
    zero_rows_kernel<double><<<grid_for(n_rows, 128), 128, 0, s>>>(vec, pat->block_ptr, pat->indptr, pat->diag,
                                                                   (double*)vals, rows, n_rows, diag_value);
  note_launches(1);
  return check_launch("zero_rows");
}

extern "C" int fem_apply_bc_vec(double* res, const double* dofs, const int32_t* rows, const double* values,
                                int64_t n_rows, double scale, void* stream) {
  FEM_REQUIRE(n_rows >= 0, "n_rows < 0");
  if (n_rows == 0) return FEM_OK;
  FEM_REQUIRE(res && dofs && rows && values, "NULL argument");
  apply_bc_vec_kernel<<<grid_for(n_rows, 256), 256, 0, as_stream(stream)>>>(res, dofs, rows, values, n_rows, scale);
  note_launches(1);
  return check_launch("apply_bc_vec");
}

extern "C" int fem_precond_setup(const fem_pattern_t* pat, int64_t n_nodes, int32_t vec, int32_t precision,
                                 const void* vals, int32_t pc_kind, void* pc, void* stream) {
  int rc = check_pat(pat, n_nodes, vec, precision);
  if (rc) return rc;
  FEM_REQUIRE(pc_kind == FEM_PC_JACOBI || pc_kind == FEM_PC_BJACOBI, "pc_kind must be JACOBI or BJACOBI");
  FEM_REQUIRE(vals && pc, "NULL argument");
  cudaStream_t s = as_stream(stream);
  const int g = grid_for(n_nodes, 256);
  if (precision == FEM_F32) {
    if (vec == 3) precond_setup_kernel<3, float><<<g, 256, 0, s>>>(n_nodes, pat->block_ptr, pat->block_cols, (const float*)vals, pc_kind, (float*)pc);
    else precond_setup_kernel<1, float><<<g, 256, 0, s>>>(n_nodes, pat->block_ptr, pat->block_cols, (const float*)vals, pc_kind, (float*)pc);
  } else {
    if (vec == 3) precond_setup_kernel<3, double><<<g, 256, 0, s>>>(n_nodes, pat->block_ptr, pat->block_cols, (const double*)vals, pc_kind, (double*)pc);
    else precond_setup_kernel<1, double><<<g, 256, 0, s>>>(n_nodes, pat->block_ptr, pat->block_cols, (const double*)vals, pc_kind, (double*)pc);
  }
  note_launches(1);
  return check_launch("precond_setup");
}

extern "C" int fem_krylov_workspace(int64_t n_dofs, int32_t precision, size_t* bytes) {
  FEM_REQUIRE(bytes && n_dofs >= 0, "bad arguments");
  FEM_REQUIRE(precision == FEM_F32 || precision == FEM_F64, "bad precision");
  *bytes = krylov_ws_bytes(n_dofs, precision);
  return FEM_OK;
}

template <typename T>
static int solve_dispatch(bool bicg, const fem_pattern_t* pat, int64_t n_nodes, int vec, const void* vals, int pc_kind,
                          const void* pc, const void* b, void* x, double rtol, double atol, int64_t maxiter, void* ws,
                          int64_t* it, double* rn, int32_t* st, cudaStream_t s) {
  const T* V = (const T*)vals;
  const T* P = (const T*)pc;
  const T* B = (const T*)b;
  T* X = (T*)x;
#define FEM_SOLVE_CASE(VEC, PC)                                                                          \
  if (vec == VEC && pc_kind == PC)                                                                       \
    return bicg ? bicg_impl<VEC, T, PC>(pat, n_nodes, V, P, B, X, rtol, atol, maxiter, ws, it, rn, st, s) \
                : pcg_impl<VEC, T, PC>(pat, n_nodes, V, P, B, X, rtol, atol, maxiter, ws, it, rn, st, s);
  FEM_SOLVE_CASE(3, FEM_PC_NONE)
  FEM_SOLVE_CASE(3, FEM_PC_JACOBI)
  FEM_SOLVE_CASE(3, FEM_PC_BJACOBI)
  FEM_SOLVE_CASE(1, FEM_PC_NONE)
  FEM_SOLVE_CASE(1, FEM_PC_JACOBI)
  FEM_SOLVE_CASE(1, FEM_PC_BJACOBI)
#undef FEM_SOLVE_CASE
  return fail(FEM_ERR_ARG, "bad vec / preconditioner");
}

static int krylov_entry(bool bicg, const fem_pattern_t* pat, int64_t n_nodes, int32_t vec, int32_t precision,
                        const void* vals, int32_t pc_kind, const void* pc, const void* b, void* x, double rtol,
                        double atol, int64_t maxiter, void* ws, size_t ws_bytes, int64_t* iterations, double* res_norm,
                        int32_t* status, void* stream) {
  int rc = check_pat(pat, n_nodes, vec, precision);
  if (rc) return rc;
  FEM_REQUIRE(vals && b && x && ws, "NULL argument");
  FEM_REQUIRE(pc_kind == FEM_PC_NONE || pc, "preconditioner data NULL");
  FEM_REQUIRE(pc_kind >= FEM_PC_NONE && pc_kind <= FEM_PC_BJACOBI, "bad pc_kind");
  FEM_REQUIRE(rtol >= 0 && atol >= 0 && maxiter >= 0, "tolerances / maxiter must be non-negative");
  FEM_REQUIRE(ws_bytes >= krylov_ws_bytes(n_nodes * vec, precision), "krylov workspace too small");
  cudaStream_t s = as_stream(stream);
  if (precision == FEM_F32)
    return solve_dispatch<float>(bicg, pat, n_nodes, vec, vals, pc_kind, pc, b, x, rtol, atol, maxiter, ws, iterations,
                                 res_norm, status, s);
  return solve_dispatch<double>(bicg, pat, n_nodes, vec, vals, pc_kind, pc, b, x, rtol, atol, maxiter, ws, iterations,
                                res_norm, status, s);
}

extern "C" int fem_pcg(const fem_pattern_t* pat, int64_t n_nodes, int32_t vec, int32_t precision, const void* vals,
                       int32_t pc_kind, const void* pc, const void* b, void* x, double rtol, double atol,
                       int64_t maxiter, void* ws, size_t ws_bytes, int64_t* iterations, double* res_norm,
                       int32_t* status, void* stream) {
  return krylov_entry(false, pat, n_nodes, vec, precision, vals, pc_kind, pc, b, x, rtol, atol, maxiter, ws, ws_bytes,
                      iterations, res_norm, status, stream);
}

extern "C" int fem_bicgstab(const fem_pattern_t* pat, int64_t n_nodes, int32_t vec, int32_t precision,
                            const void* vals, int32_t pc_kind, const void* pc, const void* b, void* x, double tol,
                            double atol, int64_t maxiter, void* ws, size_t ws_bytes, int64_t* iterations,
                            double* res_norm, int32_t* status, void* stream) {
  return krylov_entry(true, pat, n_nodes, vec, precision, vals, pc_kind, pc, b, x, tol, atol, maxiter, ws, ws_bytes,
                      iterations, res_norm, status, stream);
}

extern "C" int fem_cast_f64_f32(const double* src, float* dst, int64_t n, const uint8_t* mask, void* stream) {
  FEM_REQUIRE(n >= 0 && (n == 0 || (src && dst)), "NULL argument");
  if (n == 0) return FEM_OK;
  cast_kernel<<<grid_for(n, 256), 256, 0, as_stream(stream)>>>(src, dst, n, mask);
  return check_launch("cast");
}

extern "C" int fem_axpy_f32_f64(double alpha, const float* x, double* y, int64_t n, void* stream) {
  FEM_REQUIRE(n >= 0 && (n == 0 || (x && y)), "NULL argument");
  if (n == 0) return FEM_OK;
  axpy_kernel<<<grid_for(n, 256), 256, 0, as_stream(stream)>>>(alpha, x, y, n);
  return check_launch("axpy");
}

extern "C" int fem_dot(int32_t precision, const void* x, const void* y, int64_t n, double* out, void* ws,
                       size_t ws_bytes, void* stream) {
  FEM_REQUIRE(x && y && out && ws && n >= 0, "NULL argument");
  FEM_REQUIRE(ws_bytes >= al(sizeof(KCtl)) + al(sizeof(double) * 3 * MAX_PARTIAL_BLOCKS), "workspace too small");
  cudaStream_t s = as_stream(stream);
  KWs w = carve(ws, 0, FEM_F64);
  init_ctl_kernel<<<1, 32, 0, s>>>(w.ctl, 0.0, 0.0, 0);
  note_launches(1);
  const int g = vec_grid(n > 0 ? n : 1);
  if (precision == FEM_F32)
    dot_kernel<float><<<g, VTHREADS, 0, s>>>(n, (const float*)x, (const float*)y, w.ctl, w.partials, out);
  else
    dot_kernel<double><<<g, VTHREADS, 0, s>>>(n, (const double*)x, (const double*)y, w.ctl, w.partials, out);
  note_launches(1);
  return check_launch("dot");
}
