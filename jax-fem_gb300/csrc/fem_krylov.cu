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
#include <mutex>
#include <type_traits>

#include "fem_common.cuh"
#include "fem_df.cuh"
#include "fem_elements.cuh"

namespace fem {

constexpr int VTHREADS = 256;      // vector kernels
constexpr int SPMV_THREADS = 256;  // 8 warps = 8 node rows per CTA
constexpr int MAX_PARTIAL_BLOCKS = 8192;
// Iterations launched between two host polls of the control block (one replayed graph per chunk)
#ifndef FEM_CHUNK
#define FEM_CHUNK 16
#endif
constexpr int CHUNK = FEM_CHUNK;

struct KCtl {
  double rho, rho_prev, alpha, beta, omega, thresh2, rr, bb, d0, d1, ss;
  double rmax2, delta2, rr_true, check2;   // reliable-update PCG
  long long iter, maxiter;
  int done, status, exit_early, fault;   // fault: a bounded device wait ran out
  unsigned int ticket[4];
  float alpha_h, alpha_l, beta_h, beta_l;   // alpha, beta as float pairs for the double-float kernels
};

static bool is_sliced(int p) { return p == FEM_SLICED_F32 || p == FEM_SLICED_F64 || p == FEM_SLICED_DF48 || p == FEM_SYM_DF48; }
static bool is_df(int p) { return p == FEM_DF48 || p == FEM_SLICED_DF48 || p == FEM_SYM_DF48 || p == FEM_SSYM_DF48; }
// FP32 vectors for FP32 matrices, FP64 vectors otherwise
static bool vec_f32(int p) { return p == FEM_F32 || p == FEM_SLICED_F32; }

// internal status: the FP32 iteration paused for an FP64 residual replacement
constexpr int SOLVE_UPDATE = 10;

enum { FIN_NONE = 0, FIN_PCG_INIT, FIN_PCG_ALPHA, FIN_PCG_UPDATE, FIN_BICG_INIT, FIN_BICG_ALPHA, FIN_BICG_S,
       FIN_BICG_OMEGA, FIN_BICG_UPDATE, FIN_DOT, FIN_REF_BB, FIN_REF_TRUE, FIN_PCGR_START, FIN_PCGR_UPDATE };

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
    case FIN_REF_BB:  // d0 = b.b (FP64): true-residual target and the FP32 pause threshold
      C->bb = d[0];
      C->thresh2 = fmax(C->thresh2 * d[0], C->d1);
      C->check2 = 0.25 * C->thresh2;
      break;
    case FIN_REF_TRUE:  // d0 = ||b - A x||^2 in FP64
      C->rr_true = d[0];
      break;
    case FIN_PCGR_START: {  // d = (r.z, r.r) after a residual replacement
      if (!finite(d[0]) || !finite(d[1])) { C->status = FEM_SOLVE_NAN; C->done = 1; break; }
      C->beta = (C->iter > 0 && C->rho != 0.0) ? d[0] / C->rho : 0.0;
      C->rho = d[0];
      C->rr = d[1];
      C->rmax2 = d[1];
      C->done = 0;
      C->status = FEM_SOLVE_CONVERGED;
      break;
    }
    case FIN_PCGR_UPDATE: {  // d = (r.z, r.r) of the FP32 recursive residual
      C->iter += 1;
      C->rr = d[1];
      if (!finite(d[0]) || !finite(d[1])) { C->status = FEM_SOLVE_NAN; C->done = 1; break; }
      // pause for an FP64 residual replacement: fallen by delta, below the target, or grown 1e4x
      // (a recursive residual that far above its start is no longer trustworthy)
      if (d[1] <= C->check2 || d[1] <= C->delta2 * C->rmax2 || d[1] > 1e8 * C->rmax2) {
        C->status = SOLVE_UPDATE; C->done = 1; break;
      }
      if (C->iter >= C->maxiter) { C->status = FEM_SOLVE_MAXITER; C->done = 1; break; }
      C->beta = d[0] / C->rho;
      C->rho = d[0];
      break;
    }
    default:
      break;
  }
  // split once here: every thread of the double-float kernels would otherwise convert from FP64,
  // and a warp-wide FP64 instruction takes tens of cycles of GB300's FP64 pipe
  C->alpha_h = __double2float_rn(C->alpha);
  C->alpha_l = __double2float_rn(C->alpha - (double)C->alpha_h);
  C->beta_h = __double2float_rn(C->beta);
  C->beta_l = __double2float_rn(C->beta - (double)C->beta_h);
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

// ---- SpMV -------------------------------------------------------------------------
// Eight lanes per node row (vec scalar rows), four node rows per warp: lane `sub` takes
// block columns k = sub, sub+8, ..., loads the block column index and the vec x-entries
// once per block and all vec*vec values of the block, and the eight partial sums of each
// scalar row meet in three xor-shuffle steps.  Value formats:
//   FMT_F32   float values, float x, float y
//   FMT_F64   double values, double x, double y
//   FMT_DF    "double-float" values: float hi plus an int16 correction q scaled to
//             the ulp of hi (a = hi + q * ulp(hi) / 2^16, a 40-bit mantissa in 6 bytes),
//             x given as a (hi, lo) float pair, arithmetic in error-free FP32
//             transformations (two-product / two-sum), y written in FP64.  This keeps
//             the FP64-level accuracy of the operator while using only FP32 pipes.
enum { FMT_F32 = 0, FMT_F64 = 1, FMT_DF = 2 };
constexpr int SPMV_G = 8;

// Component stride of the FP64 transposed-part vector qT of the symmetric SpMVs (component c of
// node i at c * qt_stride + i): the node count rounded up to 32, so that each component of a
// 32-node tile is one 256-byte run (a bulk copy needs 16-byte aligned runs).
__host__ __device__ __forceinline__ int64_t qt_stride(int64_t n_nodes) { return (n_nodes + 31) & ~int64_t(31); }
// Double-float form of reduce_and_finalize for the double-float kernels: per-thread pairs are
// summed in double-float on the FP32 pipes (shuffles within a warp, then one warp over the warps'
// sums), each CTA stores its pairs as floats in its partials slot, and the last CTA sums the slots
// in block order, again in double-float; one thread converts the totals to FP64 for finalize.
// GB300's FP64 pipe takes tens of cycles per warp-wide instruction, so an FP64 epilogue run by
// every warp of an SM at once costs microseconds per launch.
__device__ __forceinline__ df2 df_shfl_down(df2 v, int off) {
  return df2{__shfl_down_sync(0xffffffffu, v.h, off), __shfl_down_sync(0xffffffffu, v.l, off)};
}
template <int ND>
__device__ __forceinline__ void block_sum_df(df2 (&v)[ND], df2* sh) {  // total in thread 0
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int nw = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int k = 0; k < ND; ++k)
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v[k] = df_add(v[k], df_shfl_down(v[k], off));
  if (lane == 0) {
#pragma unroll
    for (int k = 0; k < ND; ++k) sh[k * 32 + wid] = v[k];
  }
  __syncthreads();
  if (wid == 0) {
#pragma unroll
    for (int k = 0; k < ND; ++k) {
      df2 t = lane < nw ? sh[k * 32 + lane] : df2{0.f, 0.f};
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) t = df_add(t, df_shfl_down(t, off));
      v[k] = t;
    }
  }
  __syncthreads();
}
template <int ND>
__device__ __forceinline__ void reduce_and_finalize_df(df2 (&v)[ND], KCtl* C, int op, double* partials,
                                                       unsigned* ticket, double* dot_out) {
  __shared__ df2 sh[3 * 32];
  block_sum_df<ND>(v, sh);
  float* pf = reinterpret_cast<float*>(partials);   // a block's 3 double slots hold 3 float pairs
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < ND; ++k) {
      pf[(size_t)blockIdx.x * 6 + 2 * k] = v[k].h;
      pf[(size_t)blockIdx.x * 6 + 2 * k + 1] = v[k].l;
    }
  }
  if (last_block_ticket(ticket)) {
    df2 acc[ND];
#pragma unroll
    for (int k = 0; k < ND; ++k) acc[k] = df2{0.f, 0.f};
    for (unsigned b = threadIdx.x; b < gridDim.x; b += blockDim.x) {
      const volatile float* p = pf + (size_t)b * 6;
#pragma unroll
      for (int k = 0; k < ND; ++k) acc[k] = df_add(acc[k], df2{p[2 * k], p[2 * k + 1]});
    }
    block_sum_df<ND>(acc, sh);
    if (threadIdx.x == 0) {
      double tot[3] = {0, 0, 0};
#pragma unroll
      for (int k = 0; k < ND; ++k) tot[k] = (double)acc[k].h + (double)acc[k].l;
      finalize(C, op, tot, dot_out);
    }
  }
}

template <int FMT>
struct SpmvTypes;
template <> struct SpmvTypes<FMT_F32> { using V = float; using X = float; using Y = float; };
template <> struct SpmvTypes<FMT_F64> { using V = double; using X = double; using Y = double; };
template <> struct SpmvTypes<FMT_DF> { using V = float; using X = float; using Y = double; };

template <int VEC, int FMT, int ND>
__global__ void __launch_bounds__(SPMV_THREADS)
spmv_kernel(int64_t n_nodes, const int64_t* __restrict__ bp, const int32_t* __restrict__ bcols,
            const typename SpmvTypes<FMT>::V* __restrict__ vals, const int16_t* __restrict__ vlo,
            const typename SpmvTypes<FMT>::X* __restrict__ x, const float* __restrict__ xlo,
            typename SpmvTypes<FMT>::Y* __restrict__ y, const typename SpmvTypes<FMT>::Y* __restrict__ a, KCtl* C,
            int op, double* partials, int ticket_id) {
  using V = typename SpmvTypes<FMT>::V;
  using X = typename SpmvTypes<FMT>::X;
  if (C && C->done) return;
  const int lane = threadIdx.x & 31;
  const int sub = lane & (SPMV_G - 1);
  // groups of SPMV_G lanes own one node row (VEC scalar rows); lane `sub` takes the
  // block columns k = sub, sub + G, ... and all VEC x VEC values of each block
  const int64_t groups = ((int64_t)gridDim.x * blockDim.x) / SPMV_G;
  const int64_t first = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / SPMV_G;
  const int64_t warp_first = first - (lane / SPMV_G);
  double dv[3] = {0.0, 0.0, 0.0};
  for (int64_t base = warp_first; base < n_nodes; base += groups) {
    const int64_t i = base + lane / SPMV_G;
    const bool valid = i < n_nodes;
    const int64_t b0 = valid ? bp[i] : 0;
    const int nb = valid ? (int)(bp[i + 1] - b0) : 0;
    const int64_t rs0 = (int64_t)VEC * VEC * b0;     // first value of scalar row 0
    const int rstride = VEC * nb;                     // values per scalar row
    if constexpr (FMT == FMT_DF) {
      float sh[VEC], sl[VEC];
#pragma unroll
      for (int r = 0; r < VEC; ++r) { sh[r] = 0.0f; sl[r] = 0.0f; }
      for (int k = sub; k < nb; k += SPMV_G) {
        const int64_t col = (int64_t)VEC * __ldg(bcols + b0 + k);
        float xh[VEC], xl[VEC];
#pragma unroll
        for (int d = 0; d < VEC; ++d) { xh[d] = __ldg(x + col + d); xl[d] = __ldg(xlo + col + d); }
#pragma unroll
        for (int r = 0; r < VEC; ++r) {
          const int64_t o = rs0 + (int64_t)r * rstride + VEC * k;
#pragma unroll
          for (int d = 0; d < VEC; ++d) {
            const float ah = __ldcs(vals + o + d);
            // ulp(ah) / 2^16 from the exponent bits; q = 0 wherever this would not be a normal float
            const float sc = __int_as_float((__float_as_int(ah) & 0x7f800000) - (39 << 23));
            const float al = (float)__ldcs(vlo + o + d) * sc;
            const float p = ah * xh[d];
            float err = fmaf(ah, xh[d], -p);
            err = fmaf(ah, xl[d], err);
            err = fmaf(al, xh[d], err);
            float t, te;
            two_sum(sh[r], p, t, te);
            sl[r] += te + err;
            sh[r] = t;
          }
        }
      }
#pragma unroll
      for (int r = 0; r < VEC; ++r) {
#pragma unroll
        for (int o = SPMV_G / 2; o > 0; o >>= 1) {
          const float oh = __shfl_xor_sync(0xffffffffu, sh[r], o);
          const float ol = __shfl_xor_sync(0xffffffffu, sl[r], o);
          float t, te;
          two_sum(sh[r], oh, t, te);
          sl[r] += ol + te;
          sh[r] = t;
        }
      }
      if (valid && sub < VEC) {
        float h = sh[0], l = sl[0];
#pragma unroll
        for (int r = 1; r < VEC; ++r)
          if (sub == r) { h = sh[r]; l = sl[r]; }
        const double out = (double)h + (double)l;
        const int64_t row = (int64_t)VEC * i + sub;
        y[row] = out;
        if constexpr (ND >= 1) dv[0] += a[row] * out;
        if constexpr (ND >= 2) dv[1] += out * out;
      }
    } else {
      V acc[VEC];
#pragma unroll
      for (int r = 0; r < VEC; ++r) acc[r] = V(0);
      for (int k = sub; k < nb; k += SPMV_G) {
        const int64_t col = (int64_t)VEC * __ldg(bcols + b0 + k);
        X xv[VEC];
#pragma unroll
        for (int d = 0; d < VEC; ++d) xv[d] = __ldg(x + col + d);
#pragma unroll
        for (int r = 0; r < VEC; ++r) {
          const int64_t o = rs0 + (int64_t)r * rstride + VEC * k;
#pragma unroll
          for (int d = 0; d < VEC; ++d) acc[r] += __ldcs(vals + o + d) * xv[d];
        }
      }
#pragma unroll
      for (int r = 0; r < VEC; ++r) {
#pragma unroll
        for (int o = SPMV_G / 2; o > 0; o >>= 1) acc[r] += __shfl_xor_sync(0xffffffffu, acc[r], o);
      }
      if (valid && sub < VEC) {
        V out = acc[0];
#pragma unroll
        for (int r = 1; r < VEC; ++r)
          if (sub == r) out = acc[r];
        const int64_t row = (int64_t)VEC * i + sub;
        y[row] = out;
        if constexpr (ND >= 1) dv[0] += double(a[row]) * double(out);
        if constexpr (ND >= 2) dv[1] += double(out) * double(out);
      }
    }
  }
  if constexpr (ND > 0) reduce_and_finalize<ND>(dv, C, op, partials, C->ticket + ticket_id, nullptr);
}

// Sliced SpMV: one warp per 32-node slice, one lane per node row, all vec*vec values of a
// block slot per lane; every column-index and value load is one coalesced line.
template <int VEC, int FMT, int ND>
__global__ void __launch_bounds__(SPMV_THREADS)
spmv_sliced_kernel(int64_t n_nodes, int64_t n_slices, const int64_t* __restrict__ sp,
                   const int32_t* __restrict__ scols, const typename SpmvTypes<FMT>::V* __restrict__ vals,
                   const int16_t* __restrict__ vlo, const typename SpmvTypes<FMT>::X* __restrict__ x,
                   const float* __restrict__ xlo, typename SpmvTypes<FMT>::Y* __restrict__ y,
                   const typename SpmvTypes<FMT>::Y* __restrict__ a, KCtl* C, int op, double* partials,
                   int ticket_id) {
  using V = typename SpmvTypes<FMT>::V;
  using X = typename SpmvTypes<FMT>::X;
  using Y = typename SpmvTypes<FMT>::Y;
  constexpr int VV = VEC * VEC;
  if (C && C->done) return;
  const int lane = threadIdx.x & 31;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  double dv[3] = {0.0, 0.0, 0.0};
  for (int64_t s = warp; s < n_slices; s += nwarps) {
    const int64_t i = s * 32 + lane;
    const int64_t k0 = sp[s], k1 = sp[s + 1];
    Y out[VEC];
    if constexpr (FMT == FMT_DF) {
      float sh[VEC], sl[VEC];
#pragma unroll
      for (int r = 0; r < VEC; ++r) { sh[r] = 0.0f; sl[r] = 0.0f; }
#pragma unroll 2
      for (int64_t k = k0; k < k1; ++k) {
        const int64_t col = (int64_t)VEC * __ldg(scols + k * 32 + lane);
        float xh[VEC], xl[VEC];
#pragma unroll
        for (int d = 0; d < VEC; ++d) { xh[d] = __ldg(x + col + d); xl[d] = __ldg(xlo + col + d); }
        const int64_t vb = k * VV * 32 + lane;
#pragma unroll
        for (int v = 0; v < VV; ++v) {
          const int r = v / VEC, d = v % VEC;
          const float ah = __ldcs(vals + vb + v * 32);
          const float sc = __int_as_float((__float_as_int(ah) & 0x7f800000) - (39 << 23));
          const float al = (float)__ldcs(vlo + vb + v * 32) * sc;
          const float p = ah * xh[d];
          float err = fmaf(ah, xh[d], -p);
          err = fmaf(ah, xl[d], err);
          err = fmaf(al, xh[d], err);
          float t, te;
          two_sum(sh[r], p, t, te);
          sl[r] += te + err;
          sh[r] = t;
        }
      }
#pragma unroll
      for (int r = 0; r < VEC; ++r) out[r] = (double)sh[r] + (double)sl[r];
    } else {
      V acc[VEC];
#pragma unroll
      for (int r = 0; r < VEC; ++r) acc[r] = V(0);
#pragma unroll 2
      for (int64_t k = k0; k < k1; ++k) {
        const int64_t col = (int64_t)VEC * __ldg(scols + k * 32 + lane);
        X xv[VEC];
#pragma unroll
        for (int d = 0; d < VEC; ++d) xv[d] = __ldg(x + col + d);
        const int64_t vb = k * VV * 32 + lane;
#pragma unroll
        for (int v = 0; v < VV; ++v) acc[v / VEC] += __ldcs(vals + vb + v * 32) * xv[v % VEC];
      }
#pragma unroll
      for (int r = 0; r < VEC; ++r) out[r] = acc[r];
    }
    if (i < n_nodes) {
#pragma unroll
      for (int r = 0; r < VEC; ++r) {
        const int64_t row = (int64_t)VEC * i + r;
        y[row] = out[r];
        if constexpr (ND >= 1) dv[0] += double(a[row]) * double(out[r]);
        if constexpr (ND >= 2) dv[1] += double(out[r]) * double(out[r]);
      }
    }
  }
  if constexpr (ND > 0) reduce_and_finalize<ND>(dv, C, op, partials, C->ticket + ticket_id, nullptr);
}

// Node-interleaved double-float vector: node i's component c is (hi, lo) at xp[i * DF_PAD + c];
// for VEC = 3 a node occupies 32 bytes (one sector, two float4 loads per gathered column).
template <int VEC>
struct DfNode {
  static constexpr int PAD = VEC == 3 ? 4 : VEC;
};

template <int VEC>
__device__ __forceinline__ void df_gather(const float2* __restrict__ xp, int64_t node, float* h, float* l) {
  if constexpr (VEC == 3) {
    const float4* p4 = reinterpret_cast<const float4*>(xp) + 2 * node;
    const float4 u0 = __ldg(p4), u1 = __ldg(p4 + 1);
    h[0] = u0.x; l[0] = u0.y; h[1] = u0.z; l[1] = u0.w; h[2] = u1.x; l[2] = u1.y;
  } else {
#pragma unroll
    for (int d = 0; d < VEC; ++d) {
      const float2 u = __ldg(xp + node * VEC + d);
      h[d] = u.x; l[d] = u.y;
    }
  }
}

// Sliced DF48 SpMV with a node-interleaved double-float input xp, double-float output (yh, yl)
// and the fused dot d0 = x.y accumulated in double-float per thread (the mixed CG's p.Ap).
template <int VEC>
__global__ void __launch_bounds__(SPMV_THREADS)
spmv_sliced_dfdf_kernel(int64_t n_nodes, int64_t n_slices, const int64_t* __restrict__ sp,
                        const int32_t* __restrict__ scols, const float* __restrict__ vals,
                        const int16_t* __restrict__ vlo, const float2* __restrict__ xp,
                        float* __restrict__ yh, float* __restrict__ yl, KCtl* C, int op, double* partials) {
  constexpr int PAD = DfNode<VEC>::PAD;
  constexpr int VV = VEC * VEC;
  if (C->done) return;
  const int lane = threadIdx.x & 31;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  float ds = 0.f, de = 0.f;
  for (int64_t s = warp; s < n_slices; s += nwarps) {
    const int64_t i = s * 32 + lane;
    const int64_t k0 = sp[s], k1 = sp[s + 1];
    float sh[VEC], sl[VEC];
#pragma unroll
    for (int r = 0; r < VEC; ++r) { sh[r] = 0.0f; sl[r] = 0.0f; }
#pragma unroll 2
    for (int64_t k = k0; k < k1; ++k) {
      float xvh[VEC], xvl[VEC];
      df_gather<VEC>(xp, __ldg(scols + k * 32 + lane), xvh, xvl);
      const int64_t vb = k * VV * 32 + lane;
#pragma unroll
      for (int v = 0; v < VV; ++v) {
        const int r = v / VEC, d = v % VEC;
        const float ah = __ldcs(vals + vb + v * 32);
        const float al = df48_lo(ah, __ldcs(vlo + vb + v * 32));
        df_acc(sh[r], sl[r], df2{ah, al}, df2{xvh[d], xvl[d]});
      }
    }
    if (i < n_nodes) {
#pragma unroll
      for (int r = 0; r < VEC; ++r) {
        const int64_t row = (int64_t)VEC * i + r;
        const df2 yv = df_fast(sh[r], sl[r]);
        yh[row] = yv.h;
        yl[row] = yv.l;
        const float2 xo = xp[i * PAD + r];
        df_acc(ds, de, df2{xo.x, xo.y}, yv);
      }
    }
  }
  df2 dv[1] = {df2{ds, de}};
  reduce_and_finalize_df<1>(dv, C, op, partials, C->ticket, &C->d0);
}

// ---- bulk-copy (TMA engine) staging for the sliced DF48 SpMV -------------------------
// A slice's values, corrections and block columns are contiguous runs in HBM (slot-major), so
// each warp streams its slices through a ring of shared-memory stages with 1-D
// cp.async.bulk copies completing on one mbarrier per stage.  Lane 0 issues; every lane waits
// on the stage's phase.  The HBM stream no longer depends on the per-thread load queue, so a
// warp keeps BULK_STAGES - 1 chunks in flight while it computes on the third.
// Ring geometry (measured best on GB300 at 1M HEX8 cells; overridable for tuning sweeps)
#ifndef FEM_BULK_WARPS
#define FEM_BULK_WARPS 4
#endif
#ifndef FEM_BULK_STAGES
#define FEM_BULK_STAGES 3
#endif
#ifndef FEM_BULK_SLOTS
#define FEM_BULK_SLOTS 2
#endif
constexpr int BULK_WARPS = FEM_BULK_WARPS;     // warps per CTA
constexpr int BULK_STAGES = FEM_BULK_STAGES;   // ring depth per warp
constexpr int BULK_SLOTS = FEM_BULK_SLOTS;     // block-column slots per stage
constexpr long long BULK_WAIT_CYCLES = 4000000000LL;  // ~2 s at 2 GHz: a wait past this is a fault

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_init_fence() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void async_proxy_fence() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
               ::"r"(smem_addr(dst)), "l"(src), "r"(bytes), "r"(smem_addr(bar))
               : "memory");
}
// The same copy with an L2 eviction-priority hint (a policy from createpolicy): the SpMV streams the
// matrix evict-first, so the CG vectors it gathers and writes, and that the next kernels read, keep
// their L2 lines (the plain-load SpMVs use __ldcs for the same effect).
__device__ __forceinline__ uint64_t l2_evict_first_policy() {
  uint64_t pol;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
  return pol;
}
__device__ __forceinline__ void bulk_load_hint(void* dst, const void* src, uint32_t bytes, uint64_t* bar,
                                               uint64_t pol) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], %4;"
      ::"r"(smem_addr(dst)), "l"(src), "r"(bytes), "r"(smem_addr(bar)), "l"(pol)
      : "memory");
}
__device__ __forceinline__ bool mbar_test(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// bounded wait for a phase; false when the limit ran out
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  const long long t0 = clock64();
  for (int it = 0; it < (1 << 26); ++it) {
    if (mbar_test(bar, parity)) return true;
    if (clock64() - t0 > BULK_WAIT_CYCLES) break;
  }
  return false;
}

// Failure-detection self-test of the bounded wait above: one warp waits on a phase that can never
// complete (an mbarrier expecting two arrivals receives one; no copy, no transaction bytes), gives
// up after the same limit as the bulk-copy kernels and reports the way they do, through the
// control block's fault and done words.
__global__ void bounded_wait_selftest_kernel(KCtl* C) {
  __shared__ __align__(8) uint64_t bar;
  const int lane = threadIdx.x & 31;
  if (lane == 0) {
    mbar_init(&bar, 2);
    mbar_init_fence();
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(&bar)) : "memory");
  }
  __syncwarp();
  const bool ok = mbar_wait(&bar, 0);
  if (!__all_sync(0xffffffffu, ok) && lane == 0) {
    atomicExch(&C->fault, 1);
    atomicExch(&C->done, 1);
  }
}

template <int VEC>
struct BulkGeom {
  static constexpr uint32_t VB = VEC * VEC * 32 * 4;  // value bytes per slot
  static constexpr uint32_t LB = VEC * VEC * 32 * 2;  // correction bytes per slot
  static constexpr uint32_t CB = 32 * 4;              // block-column bytes per slot
  static constexpr uint32_t STAGE = BULK_SLOTS * (VB + LB + CB);
  static constexpr uint32_t BAR_BYTES = (BULK_WARPS * BULK_STAGES * 8 + 127) / 128 * 128;   // barriers, padded
  static constexpr uint32_t SMEM = BAR_BYTES + BULK_WARPS * BULK_STAGES * STAGE;
};

// Sliced DF48 SpMV, bulk-copy staged: same arithmetic and outputs as spmv_sliced_dfdf_kernel.
// Requires 16-byte aligned vals, vlo and slice_cols (checked by the host launcher).
// SYM: the matrix holds the upper node blocks only (FEM_SYM_DF48, diagonal block first in each
// row); row i accumulates A_ij x_j in double-float as before and, for j != i, adds A_ij^T x_i to
// row j through FP64 atomics into qT (zeroed by the caller, combined by the consumer).  The
// fused dot is x.(A x) = sum_i 2 x_i.(sum_j A_ij x_j) - x_i.A_ii x_i.
// GRID: the grid layout of fem_pattern_slices_grid (node grid gnx x gny x gnz) -- slot k of every
// slice couples node n with node n + stencil_offset(k) (clamped to the node range; the slots
// outside the grid hold zero blocks), so no block columns are streamed.  Lane k < 27 holds offset
// k; a slot reads it by one warp shuffle.
template <int VEC, bool SYM = false, bool GRID = false>
__global__ void __launch_bounds__(BULK_WARPS * 32)
spmv_sliced_dfdf_bulk_kernel(int64_t n_nodes, int64_t n_slices, const int64_t* __restrict__ sp,
                             const int32_t* __restrict__ scols, const float* __restrict__ vals,
                             const int16_t* __restrict__ vlo, const float2* __restrict__ xp,
                             float* __restrict__ yh, float* __restrict__ yl, KCtl* C, int op, double* partials,
                             double* __restrict__ qT = nullptr, int64_t gny = 0, int64_t gnz = 0) {
  static_assert(!(GRID && SYM), "the grid layout holds whole rows");
  using G = BulkGeom<VEC>;
  constexpr int VV = VEC * VEC;
  constexpr int PAD = DfNode<VEC>::PAD;
  extern __shared__ __align__(128) unsigned char smem[];
  if (C->done) return;
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem) + wib * BULK_STAGES;
  unsigned char* ring = smem + G::BAR_BYTES + (size_t)wib * BULK_STAGES * G::STAGE;
  const int64_t warp = (int64_t)blockIdx.x * BULK_WARPS + wib;
  const int64_t nwarps = (int64_t)gridDim.x * BULK_WARPS;
  const int32_t lane_off = GRID && lane < 27 ? (int32_t)stencil_offset(lane, gny, gnz) : 0;
  if (lane == 0) {
#pragma unroll
    for (int j = 0; j < BULK_STAGES; ++j) mbar_init(bars + j, 1);
    mbar_init_fence();
  }
  __syncwarp();

  // producer cursor: next chunk to copy (all lanes track it; lane 0 issues)
  int64_t ps = warp, pk = 0, pe = 0;
  if (ps < n_slices) { pk = sp[ps]; pe = sp[ps + 1]; }
  auto produce = [&](int stage) -> bool {
    while (ps < n_slices && pk == pe) {
      ps += nwarps;
      if (ps < n_slices) { pk = sp[ps]; pe = sp[ps + 1]; }
    }
    if (ps >= n_slices) return false;
    const int64_t cnt = pe - pk < BULK_SLOTS ? pe - pk : BULK_SLOTS;
    if (lane == 0) {
      unsigned char* st = ring + (size_t)stage * G::STAGE;
      const uint32_t nb = (uint32_t)cnt;
      async_proxy_fence();
      mbar_expect_tx(bars + stage, nb * (G::VB + G::LB + (GRID ? 0u : G::CB)));
      const uint64_t pol = l2_evict_first_policy();
      bulk_load_hint(st, vals + pk * VV * 32, nb * G::VB, bars + stage, pol);
      bulk_load_hint(st + BULK_SLOTS * G::VB, vlo + pk * VV * 32, nb * G::LB, bars + stage, pol);
      if (!GRID) bulk_load_hint(st + BULK_SLOTS * (G::VB + G::LB), scols + pk * 32, nb * G::CB, bars + stage, pol);
    }
    pk += cnt;
    return true;
  };

  uint32_t parity = 0;  // bit j: phase parity to wait for on stage j
  int inflight = 0;
  for (int j = 0; j < BULK_STAGES; ++j) inflight += produce(j) ? 1 : 0;

  bool fault = false;
  float ds = 0.f, de = 0.f;
  float dd_h = 0.f, dd_l = 0.f;   // SYM: sum of x_i.A_ii x_i
  int stage = 0;
  int64_t cs = warp, ck = 0, ce = 0, cb = 0;   // cb: the slice's first slot (GRID)
  if (cs < n_slices) { ck = cb = sp[cs]; ce = sp[cs + 1]; }
  float sh[VEC], sl[VEC];
#pragma unroll
  for (int r = 0; r < VEC; ++r) { sh[r] = 0.f; sl[r] = 0.f; }
  // The plain (non-SYM) vec-3 kernel accumulates a stage's two slots in two banks at once on the
  // paired FP32 instructions (df_acc2), folded into sh / sl when the slice ends.
  constexpr bool PAIR = !SYM && VEC == 3 && BULK_SLOTS == 2;
  float2 ph[VEC], pl[VEC];
#pragma unroll
  for (int r = 0; r < VEC; ++r) ph[r] = pl[r] = make_float2(0.f, 0.f);
  float xih[VEC], xil[VEC];       // SYM: the row's own x
  bool first = true;              // SYM: next slot is the diagonal block
  auto load_own = [&]() {
    if constexpr (SYM) {
      const int64_t i = cs * 32 + lane;
      if (cs < n_slices && i < n_nodes) {
        df_gather<VEC>(xp, i, xih, xil);
      } else {
#pragma unroll
        for (int r = 0; r < VEC; ++r) { xih[r] = 0.f; xil[r] = 0.f; }
      }
      first = true;
    }
  };
  load_own();
  while (cs < n_slices) {
    if (ck < ce) {
      const bool ok = mbar_wait(bars + stage, (parity >> stage) & 1u);
      if (!__all_sync(0xffffffffu, ok)) { fault = true; break; }
      parity ^= 1u << stage;
      --inflight;
      const unsigned char* st = ring + (size_t)stage * G::STAGE;
      const float* sv = reinterpret_cast<const float*>(st);
      const int16_t* sq = reinterpret_cast<const int16_t*>(st + BULK_SLOTS * G::VB);
      const int32_t* sc = reinterpret_cast<const int32_t*>(st + BULK_SLOTS * (G::VB + G::LB));
      const int cnt = ce - ck < BULK_SLOTS ? (int)(ce - ck) : BULK_SLOTS;
      float xvh[BULK_SLOTS][VEC], xvl[BULK_SLOTS][VEC];
#pragma unroll
      for (int t = 0; t < BULK_SLOTS; ++t) {
        if (t < cnt) {
          int64_t col;
          if constexpr (GRID) {
            col = cs * 32 + lane + __shfl_sync(0xffffffffu, lane_off, (int)(ck - cb) + t);
            col = col < 0 ? 0 : col >= n_nodes ? n_nodes - 1 : col;
          } else {
            col = sc[t * 32 + lane];
          }
          df_gather<VEC>(xp, col, xvh[t], xvl[t]);
        }
      }
      if constexpr (PAIR) {
        // the stage's two slots as the two components of paired FP32 operations; a stage with one
        // slot (a slice's odd last one) pairs it with zeros -- a warp-uniform branch, so the full
        // stages carry no per-value selects
        auto pair_stage = [&](auto two_c) {
          constexpr bool TWO = decltype(two_c)::value;
          float2 xh2[VEC], nxh2[VEC], xl2[VEC];
#pragma unroll
          for (int d = 0; d < VEC; ++d) {
            const float h1 = TWO ? xvh[1][d] : 0.f, l1 = TWO ? xvl[1][d] : 0.f;
            xh2[d] = make_float2(xvh[0][d], h1);
            nxh2[d] = make_float2(-xvh[0][d], -h1);
            xl2[d] = make_float2(xvl[0][d], l1);
          }
#pragma unroll
          for (int v = 0; v < VV; ++v) {
            const int r = v / VEC, d = v % VEC;
            const float h0 = sv[v * 32 + lane];
            const float l0 = df48_lo(h0, sq[v * 32 + lane]);
            const float h1 = TWO ? sv[(VV + v) * 32 + lane] : 0.f;
            const float l1 = TWO ? df48_lo(h1, sq[(VV + v) * 32 + lane]) : 0.f;
            df_acc2(ph[r], pl[r], make_float2(h0, h1), make_float2(l0, l1), xh2[d], nxh2[d], xl2[d]);
          }
        };
        if (cnt > 1) pair_stage(std::true_type{});
        else pair_stage(std::false_type{});
      }
#pragma unroll
      for (int t = 0; t < BULK_SLOTS; ++t) {
        if (!PAIR && t < cnt) {
          if constexpr (SYM) {
            float ah[VV], al[VV];
#pragma unroll
            for (int v = 0; v < VV; ++v) {
              ah[v] = sv[(t * VV + v) * 32 + lane];
              al[v] = df48_lo(ah[v], sq[(t * VV + v) * 32 + lane]);
            }
            if (first) {  // diagonal block: A_ii x_i starts the row and its x.A x term
#pragma unroll
              for (int v = 0; v < VV; ++v) {
                const int r = v / VEC, d = v % VEC;
                df_acc(sh[r], sl[r], df2{ah[v], al[v]}, df2{xvh[t][d], xvl[t][d]});
              }
#pragma unroll
              for (int r = 0; r < VEC; ++r) df_acc(dd_h, dd_l, df2{xih[r], xil[r]}, df_fast(sh[r], sl[r]));
              first = false;
            } else {
#pragma unroll
              for (int v = 0; v < VV; ++v) {
                const int r = v / VEC, d = v % VEC;
                df_acc(sh[r], sl[r], df2{ah[v], al[v]}, df2{xvh[t][d], xvl[t][d]});
              }
              const int j = sc[t * 32 + lane];
              const int64_t i = cs * 32 + lane;
              if (i < n_nodes && j != (int)i) {
#pragma unroll
                for (int d = 0; d < VEC; ++d) {
                  float th = 0.f, tl = 0.f;
#pragma unroll
                  for (int r = 0; r < VEC; ++r)
                    df_acc(th, tl, df2{ah[r * VEC + d], al[r * VEC + d]}, df2{xih[r], xil[r]});
                  atomicAdd(qT + (int64_t)d * qt_stride(n_nodes) + j, (double)th + (double)tl);   // component-major
                }
              }
            }
          } else {
#pragma unroll
            for (int v = 0; v < VV; ++v) {
              const int r = v / VEC, d = v % VEC;
              const float ah = sv[(t * VV + v) * 32 + lane];
              const float al = df48_lo(ah, sq[(t * VV + v) * 32 + lane]);
              df_acc(sh[r], sl[r], df2{ah, al}, df2{xvh[t][d], xvl[t][d]});
            }
          }
        }
      }
      __syncwarp();
      inflight += produce(stage) ? 1 : 0;
      stage = stage + 1 == BULK_STAGES ? 0 : stage + 1;
      ck += cnt;
    }
    if (ck == ce) {  // slice finished: write its rows and the dot contribution
      const int64_t i = cs * 32 + lane;
      if constexpr (PAIR) {   // fold the two banks into the row sums
#pragma unroll
        for (int r = 0; r < VEC; ++r) {
          const df2 f = df_add(df_fast(ph[r].x, pl[r].x), df_fast(ph[r].y, pl[r].y));
          sh[r] = f.h;
          sl[r] = f.l;
          ph[r] = pl[r] = make_float2(0.f, 0.f);
        }
      }
      if (i < n_nodes) {
#pragma unroll
        for (int r = 0; r < VEC; ++r) {
          const int64_t row = (int64_t)VEC * i + r;
          const df2 yv = df_fast(sh[r], sl[r]);
          yh[row] = yv.h;
          yl[row] = yv.l;
          const float2 xo = xp[i * PAD + r];
          df_acc(ds, de, df2{xo.x, xo.y}, yv);
        }
      }
#pragma unroll
      for (int r = 0; r < VEC; ++r) { sh[r] = 0.f; sl[r] = 0.f; }
      cs += nwarps;
      if (cs < n_slices) { ck = cb = sp[cs]; ce = sp[cs + 1]; }
      load_own();
    }
  }
  if (fault) {
    // let the copies already issued land (bounded) before the CTA's shared memory is released
    for (int j = 0; j < inflight; ++j) {
      (void)mbar_wait(bars + stage, (parity >> stage) & 1u);
      parity ^= 1u << stage;
      stage = stage + 1 == BULK_STAGES ? 0 : stage + 1;
    }
    if (lane == 0) {
      atomicExch(&C->fault, 1);
      atomicExch(&C->done, 1);
    }
  }
  df2 dv[1] = {df2{ds, de}};
  if constexpr (SYM) dv[0] = df_add(df2{2.f * ds, 2.f * de}, df2{-dd_h, -dd_l});
  reduce_and_finalize_df<1>(dv, C, op, partials, C->ticket, &C->d0);
}

// y (df) += qT (FP64, component-major: component c of node i at c * qt_stride + i), qT = 0: the
// FEM_SYM_DF48 SpMV's transposed part folded into its result (vec 3)
__global__ void sym_combine_kernel(int64_t n_nodes, float* __restrict__ yh, float* __restrict__ yl,
                                   double* __restrict__ qT) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < 3 * n_nodes;
       k += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = k / 3;
    const int64_t t = (k - 3 * i) * qt_stride(n_nodes) + i;
    const df2 y = df_add(df2{yh[k], yl[k]}, df_from_bits(qT[t]));
    yh[k] = y.h;
    yl[k] = y.l;
    qT[t] = 0.0;
  }
}

}  // namespace fem
#include "fem_ssym.cuh"
namespace fem {

// FP64 CSR values -> sliced layout (FP64, FP32 or DF48 hi/lo), thread per (slice, lane).  Slot k
// of a row holds its k-th block, or with the grid layout (gnx > 0, fem_pattern_slices_grid) the
// block of stencil neighbour k, found by a merge walk over the row's sorted block columns.
template <int VEC, int OUT>
__global__ void to_sliced_kernel(int64_t n_nodes, int64_t n_slices, const int64_t* bp, const int64_t* sp,
                                 const double* v64, void* out, int16_t* lo, const int32_t* bcols, int64_t gnx,
                                 int64_t gny, int64_t gnz) {
  constexpr int VV = VEC * VEC;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n_slices * 32; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t s = t >> 5;
    const int l = (int)(t & 31);
    const int64_t i = s * 32 + l;
    const int64_t b0 = i < n_nodes ? bp[i] : 0;
    const int nb = i < n_nodes ? (int)(bp[i + 1] - b0) : 0;
    const int64_t w = sp[s + 1] - sp[s];
    int p = 0;   // grid layout: merge cursor into the row's block columns
    for (int64_t k = 0; k < w; ++k) {
      int blk = k < nb ? (int)k : -1;
      if (gnx > 0) {
        blk = -1;
        const int64_t j = i < n_nodes ? stencil_neighbour(i, (int)k, gnx, gny, gnz) : -1;
        if (j >= 0) {
          while (p < nb && bcols[b0 + p] < j) ++p;
          if (p < nb && bcols[b0 + p] == j) blk = p;
        }
      }
      for (int v = 0; v < VV; ++v) {
        const int r = v / VEC, d = v % VEC;
        const double a = blk >= 0 ? v64[(int64_t)VV * b0 + (int64_t)r * VEC * nb + VEC * blk + d] : 0.0;
        const int64_t o = ((sp[s] + k) * VV + v) * 32 + l;
        if (OUT == FEM_SLICED_F64) {
          static_cast<double*>(out)[o] = a;
        } else if (OUT == FEM_SLICED_F32) {
          static_cast<float*>(out)[o] = (float)a;
        } else {
          const float h = __double2float_rn(a);
          const int e = (__float_as_int(h) >> 23) & 0xFF;
          int q = 0;
          if (e > 39 && e < 255) {
            double tq = rint(scalbn(a - (double)h, 166 - e));
            tq = fmin(fmax(tq, -32767.0), 32767.0);
            q = (int)tq;
          }
          static_cast<float*>(out)[o] = h;
          lo[o] = (int16_t)q;
        }
      }
    }
  }
}

// FP64 CSR values -> FEM_SYM_DF48 (the upper node blocks of each row), thread per (slice, lane).
template <int VEC>
__global__ void to_sliced_upper_kernel(int64_t n_nodes, int64_t n_slices, const int64_t* bp, const int32_t* bcols,
                                       const int64_t* sp, const double* v64, float* hi, int16_t* lo) {
  constexpr int VV = VEC * VEC;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n_slices * 32; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t s = t >> 5;
    const int l = (int)(t & 31);
    const int64_t i = s * 32 + l;
    const int64_t b0 = i < n_nodes ? bp[i] : 0;
    const int nb = i < n_nodes ? (int)(bp[i + 1] - b0) : 0;
    int u0 = 0;
    while (u0 < nb && bcols[b0 + u0] < i) ++u0;
    const int64_t w = sp[s + 1] - sp[s];
    for (int64_t k = 0; k < w; ++k) {
      for (int v = 0; v < VV; ++v) {
        const int r = v / VEC, d = v % VEC;
        const double a = u0 + k < nb ? v64[(int64_t)VV * b0 + (int64_t)r * VEC * nb + VEC * (u0 + k) + d] : 0.0;
        const int64_t o = ((sp[s] + k) * VV + v) * 32 + l;
        const float h = __double2float_rn(a);
        const int e = (__float_as_int(h) >> 23) & 0xFF;
        int q = 0;
        if (e > 39 && e < 255) {
          double tq = rint(scalbn(a - (double)h, 166 - e));
          tq = fmin(fmax(tq, -32767.0), 32767.0);
          q = (int)tq;
        }
        hi[o] = h;
        lo[o] = (int16_t)q;
      }
    }
  }
}

// DF48 split of an FP64 matrix: hi = fl32(a), q = round((a - hi) * 2^16 / ulp(hi)).
__global__ void split_df_kernel(const double* __restrict__ v, int64_t n, float* __restrict__ hi,
                                int16_t* __restrict__ lo) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    const double a = v[k];
    const float h = __double2float_rn(a);
    const int e = (__float_as_int(h) >> 23) & 0xFF;
    int q = 0;
    if (e > 39 && e < 255) {
      const double rem = a - (double)h;
      double t = rint(scalbn(rem, 166 - e));
      t = fmin(fmax(t, -32767.0), 32767.0);
      q = (int)t;
    }
    hi[k] = h;
    lo[k] = (int16_t)q;
  }
}

// (hi, lo) float split of an FP64 vector, the SpMV input of the DF format
__global__ void split_vec_kernel(const double* __restrict__ v, int64_t n, float* __restrict__ hi,
                                 float* __restrict__ lo) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    const double a = v[k];
    const float h = __double2float_rn(a);
    hi[k] = h;
    lo[k] = __double2float_rn(a - (double)h);
  }
}

// ---- vector kernels (thread per node) ----------------------------------------
// Preconditioner entries per node: the diagonal (FEM_PC_JACOBI), the full VEC x VEC block-Jacobi
// inverse (FEM_PC_BJACOBI) or, in the double-float CG, its upper triangle m00 m01 m02 m11 m12 m22
// (PC_BSYM, vec 3: the inverse of a symmetric block is symmetric, so 6 of 9 floats carry it).
constexpr int PC_BSYM = 3;   // internal template tag next to FEM_PC_NONE / _JACOBI / _BJACOBI
__host__ __device__ constexpr int pc_width(int pc) {
  return pc == FEM_PC_BJACOBI ? 9 : pc == PC_BSYM ? 6 : pc == FEM_PC_JACOBI ? 3 : 0;
}

template <int VEC, typename T, int PC>
__device__ __forceinline__ void precond(const T* pc, int64_t i, const T (&r)[VEC], T (&z)[VEC]) {
  if constexpr (PC == FEM_PC_NONE) {
#pragma unroll
    for (int c = 0; c < VEC; ++c) z[c] = r[c];
  } else if constexpr (PC == FEM_PC_JACOBI) {
#pragma unroll
    for (int c = 0; c < VEC; ++c) z[c] = pc[VEC * i + c] * r[c];
  } else if constexpr (PC == PC_BSYM) {
    static_assert(VEC == 3, "PC_BSYM is the vec-3 block form");
    const T* B = pc + 6 * i;
    z[0] = B[0] * r[0] + B[1] * r[1] + B[2] * r[2];
    z[1] = B[1] * r[0] + B[3] * r[1] + B[4] * r[2];
    z[2] = B[2] * r[0] + B[4] * r[1] + B[5] * r[2];
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
                                  double* partials, int op) {
  if (C->done) return;
  const T alpha = T(C->alpha);
  double dv[3] = {0, 0, 0};
  GRID_STRIDE_NODES(i, n_nodes) {
    T rv[VEC], zv[VEC];
#pragma unroll
    for (int c = 0; c < VEC; ++c) {
      const int64_t k = VEC * i + c;
      // plain loads: each thread walks its node's VEC entries in separate instructions, so a
      // streaming (evict-first) load would drop lines the neighbouring lanes read next (measured:
      // 65 -> 77 us per launch at 3.1M dofs)
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
  reduce_and_finalize<2>(dv, C, op, partials, C->ticket + 1, nullptr);
}

// Reliable-update PCG: FP64 true residual r64 = b - A x (A x in ax; Dirichlet rows b - x),
// its FP32 copy r32, and ||r64||^2.
__global__ void refine_residual_kernel(int64_t n, const double* b, const double* x, const double* ax,
                                       const uint8_t* bc, float* r32, KCtl* C, double* partials, double scale) {
  double dv[3] = {0, 0, 0};
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    const double r = (bc && bc[k]) ? (b[k] - x[k]) : (b[k] - ax[k]);
    r32[k] = (float)(r * scale);   // scale: a power of two keeping the FP32 iteration near unit size
    dv[0] += r * r;
  }
  reduce_and_finalize<1>(dv, C, FIN_REF_TRUE, partials, C->ticket + 1, nullptr);
}

// After a residual replacement: z = M r, dots (r.z, r.r); x32 := 0; p := z on the first start.
template <int VEC, int PC>
__global__ void pcgr_start_kernel(int64_t n_nodes, const float* r, float* z, float* p, float* x32, const float* pc,
                                  int first, KCtl* C, double* partials) {
  double dv[3] = {0, 0, 0};
  GRID_STRIDE_NODES(i, n_nodes) {
    float rv[VEC], zv[VEC];
#pragma unroll
    for (int c = 0; c < VEC; ++c) rv[c] = r[VEC * i + c];
    precond<VEC, float, PC>(pc, i, rv, zv);
#pragma unroll
    for (int c = 0; c < VEC; ++c) {
      const int64_t k = VEC * i + c;
      z[k] = zv[c];
      x32[k] = 0.0f;
      if (first) p[k] = zv[c];
      dv[0] += double(rv[c]) * double(zv[c]);
      dv[1] += double(rv[c]) * double(rv[c]);
    }
  }
  reduce_and_finalize<2>(dv, C, FIN_PCGR_START, partials, C->ticket + 1, nullptr);
}

__global__ void accumulate_kernel(double* x64, const float* x32, int64_t n, double inv_scale) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
    x64[k] += (double)x32[k] * inv_scale;
}

// ---- double-float (DF48) PCG: FP64 vectors, DF48 SpMV, FP32 preconditioner --------
template <int VEC, int PC>
__device__ __forceinline__ void precond32(const float* pc, int64_t i, const double (&r)[VEC], double (&z)[VEC]) {
  float rf[VEC], zf[VEC];
#pragma unroll
  for (int c = 0; c < VEC; ++c) rf[c] = (float)r[c];
  precond<VEC, float, PC>(pc, i, rf, zf);
#pragma unroll
  for (int c = 0; c < VEC; ++c) z[c] = (double)zf[c];
}

__device__ __forceinline__ void split_store(double v, float* hi, float* lo, int64_t k) {
  const float h = __double2float_rn(v);
  hi[k] = h;
  lo[k] = __double2float_rn(v - (double)h);
}

// z = M r; on the first start p = z (and its (hi, lo) split); dots (r.z, r.r)
template <int VEC, int PC>
__global__ void pcgd_start_kernel(int64_t n_nodes, const double* r, double* z, double* p, float* phi, float* plo,
                                  const float* pc, int first, KCtl* C, double* partials) {
  double dv[3] = {0, 0, 0};
  GRID_STRIDE_NODES(i, n_nodes) {
    double rv[VEC], zv[VEC];
#pragma unroll
    for (int c = 0; c < VEC; ++c) rv[c] = r[VEC * i + c];
    precond32<VEC, PC>(pc, i, rv, zv);
#pragma unroll
    for (int c = 0; c < VEC; ++c) {
      const int64_t k = VEC * i + c;
      z[k] = zv[c];
      if (first) { p[k] = zv[c]; split_store(zv[c], phi, plo, k); }
      dv[0] += rv[c] * zv[c];
      dv[1] += rv[c] * rv[c];
    }
  }
  reduce_and_finalize<2>(dv, C, FIN_PCGR_START, partials, C->ticket + 1, nullptr);
}

// x += alpha p ; r -= alpha q ; z = M r ; dots (r.z, r.r)
template <int VEC, int PC>
__global__ void pcgd_update_kernel(int64_t n_nodes, double* x, double* r, double* z, const double* p, const double* q,
                                   const float* pc, KCtl* C, double* partials, int op) {
  if (C->done) return;
  const double alpha = C->alpha;
  double dv[3] = {0, 0, 0};
  GRID_STRIDE_NODES(i, n_nodes) {
    double rv[VEC], zv[VEC];
#pragma unroll
    for (int c = 0; c < VEC; ++c) {
      const int64_t k = VEC * i + c;
      x[k] += alpha * p[k];
      rv[c] = r[k] - alpha * q[k];
      r[k] = rv[c];
    }
    precond32<VEC, PC>(pc, i, rv, zv);
#pragma unroll
    for (int c = 0; c < VEC; ++c) {
      z[VEC * i + c] = zv[c];
      dv[0] += rv[c] * zv[c];
      dv[1] += rv[c] * rv[c];
    }
  }
  reduce_and_finalize<2>(dv, C, op, partials, C->ticket + 1, nullptr);
}

// p = z + beta p and its (hi, lo) split for the DF48 SpMV
__global__ void pcgd_direction_kernel(int64_t n, double* p, const double* z, float* phi, float* plo, const KCtl* C) {
  if (C->done) return;
  const double beta = C->beta;
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    const double v = z[k] + beta * p[k];
    p[k] = v;
    split_store(v, phi, plo, k);
  }
}

// first start / restart after a residual replacement: z = M r.h ; (first) p = z ; dots (r.z, r.r)
template <int VEC, int PC>
__global__ void pcgx_start_kernel(int64_t n_nodes, const float* rh, const float* rl, float* z, float2* pp,
                                  const float* pc, int first, KCtl* C, double* partials) {
  constexpr int PAD = DfNode<VEC>::PAD;
  float s0 = 0.f, e0 = 0.f, s1 = 0.f, e1 = 0.f;
  GRID_STRIDE_NODES(i, n_nodes) {
    float rv[VEC], zv[VEC];
#pragma unroll
    for (int c = 0; c < VEC; ++c) rv[c] = rh[VEC * i + c];
    precond<VEC, float, PC>(pc, i, rv, zv);
#pragma unroll
    for (int c = 0; c < VEC; ++c) {
      const int64_t k = VEC * i + c;
      z[k] = zv[c];
      if (first) pp[i * PAD + c] = make_float2(zv[c], 0.f);
      const df2 r{rv[c], rl[k]};
      df_acc(s0, e0, r, df2{zv[c], 0.f});
      df_acc(s1, e1, r, r);
    }
  }
  df2 dv[2] = {df2{s0, e0}, df2{s1, e1}};
  reduce_and_finalize_df<2>(dv, C, FIN_PCGR_START, partials, C->ticket + 1, nullptr);
}

// x += alpha p ; r -= alpha q ; z = M r.h ; dots (r.z, r.r)
template <int VEC, int PC>
__global__ void pcgx_update_kernel(int64_t n_nodes, float* xh, float* xl, float* rh, float* rl, float* z,
                                   const float2* pp, const float* qh, const float* ql, const float* pc,
                                   KCtl* C, double* partials, int op) {
  constexpr int PAD = DfNode<VEC>::PAD;
  if (C->done) return;
  const df2 a{C->alpha_h, C->alpha_l};
  const df2 na{-a.h, -a.l};
  float s0 = 0.f, e0 = 0.f, s1 = 0.f, e1 = 0.f;
  GRID_STRIDE_NODES(i, n_nodes) {
    float rv[VEC], zv[VEC];
    df2 rr[VEC];
#pragma unroll
    for (int c = 0; c < VEC; ++c) {
      const int64_t k = VEC * i + c;
      const float2 pv = pp[i * PAD + c];
      const df2 p{pv.x, pv.y}, q{qh[k], ql[k]};
      const df2 x = df_add(df2{xh[k], xl[k]}, df_mul(a, p));
      xh[k] = x.h; xl[k] = x.l;
      const df2 r = df_add(df2{rh[k], rl[k]}, df_mul(na, q));
      rh[k] = r.h; rl[k] = r.l;
      rr[c] = r;
      rv[c] = r.h;
    }
    precond<VEC, float, PC>(pc, i, rv, zv);
#pragma unroll
    for (int c = 0; c < VEC; ++c) {
      z[VEC * i + c] = zv[c];
      df_acc(s0, e0, rr[c], df2{zv[c], 0.f});
      df_acc(s1, e1, rr[c], rr[c]);
    }
  }
  df2 dv[2] = {df2{s0, e0}, df2{s1, e1}};
  reduce_and_finalize_df<2>(dv, C, op, partials, C->ticket + 1, nullptr);
}

// vec-3 form of pcgx_update_kernel with every global access coalesced: a warp takes a tile of
// 32 nodes (96 dofs); the dof-ordered arrays (x, r, q, z) move in three full lines per array,
// the preconditioner blocks in nine, and the node-wise z = M r.h regroups through shared memory
// (strides 3 and 9 are bank-conflict free).
constexpr int VTILE_WARPS = VTHREADS / 32;
#ifndef FEM_TILE_MIN_BLOCKS
#define FEM_TILE_MIN_BLOCKS 6   // 40 registers, 48 resident warps per SM: more loads in flight
#endif
// z = M r for one node from its entries e (pc_width(PC) floats)
template <int PC>
__device__ __forceinline__ void pc3_apply(const float* e, const float (&rv)[3], float (&zv)[3]) {
  if constexpr (PC == FEM_PC_BJACOBI) {
#pragma unroll
    for (int c = 0; c < 3; ++c) zv[c] = e[3 * c] * rv[0] + e[3 * c + 1] * rv[1] + e[3 * c + 2] * rv[2];
  } else if constexpr (PC == PC_BSYM) {
    zv[0] = e[0] * rv[0] + e[1] * rv[1] + e[2] * rv[2];
    zv[1] = e[1] * rv[0] + e[3] * rv[1] + e[4] * rv[2];
    zv[2] = e[2] * rv[0] + e[4] * rv[1] + e[5] * rv[2];
  } else if constexpr (PC == FEM_PC_JACOBI) {
#pragma unroll
    for (int c = 0; c < 3; ++c) zv[c] = e[c] * rv[c];
  } else {
#pragma unroll
    for (int c = 0; c < 3; ++c) zv[c] = rv[c];
  }
}

// Upper triangles of the (symmetric) 3x3 block-Jacobi inverses: 9 floats per node -> 6.
__global__ void bsym_compact_kernel(int64_t n_nodes, const float* __restrict__ pc9, float* __restrict__ pc6) {
  GRID_STRIDE_NODES(i, n_nodes) {
    const float* b = pc9 + 9 * i;
    float* o = pc6 + 6 * i;
    o[0] = b[0]; o[1] = b[1]; o[2] = b[2]; o[3] = b[4]; o[4] = b[5]; o[5] = b[8];
  }
}

template <int PC, bool SYM = false>
__global__ void __launch_bounds__(VTHREADS, FEM_TILE_MIN_BLOCKS)
pcgx_update_tile_kernel(int64_t n_nodes, float* __restrict__ xh, float* __restrict__ xl, float* __restrict__ rh,
                        float* __restrict__ rl, float* __restrict__ z, const float2* __restrict__ pp,
                        const float* __restrict__ qh, const float* __restrict__ ql, const float* __restrict__ pc,
                        KCtl* C, double* partials, int op, double* __restrict__ qT) {
  constexpr int PCW = pc_width(PC);
  __shared__ float s_r[VTILE_WARPS][96], s_rl[VTILE_WARPS][96], s_z[VTILE_WARPS][96];
  __shared__ float s_pc[VTILE_WARPS][PCW > 0 ? 32 * PCW : 1];
  if (C->done) return;
  const df2 a{C->alpha_h, C->alpha_l};
  const df2 na{-a.h, -a.l};
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  float* sr = s_r[w];
  float* srl = s_rl[w];
  float* sz = s_z[w];
  float* spc = s_pc[w];
  float s0 = 0.f, e0 = 0.f, s1 = 0.f, e1 = 0.f;
  const int64_t ntiles = (n_nodes + 31) / 32;
  const int64_t nw = (int64_t)gridDim.x * VTILE_WARPS;
  for (int64_t t = (int64_t)blockIdx.x * VTILE_WARPS + w; t < ntiles; t += nw) {
    const int64_t node0 = t * 32;
    const int nn = n_nodes - node0 < 32 ? (int)(n_nodes - node0) : 32;
    const int nd = 3 * nn;
    const int64_t d0 = 3 * node0;
#pragma unroll
    for (int j = 0; j < PCW; ++j) {
      const int o = 32 * j + lane;
      if (o < PCW * nn) spc[o] = pc[PCW * node0 + o];
    }
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const int o = 32 * j + lane;
      if (o < nd) {
        const int64_t k = d0 + o;
        const int nl = o / 3, c = o - 3 * nl;
        const float2 pv = pp[(node0 + nl) * 4 + c];
        const df2 x = df_add(df2{xh[k], xl[k]}, df_mul(a, df2{pv.x, pv.y}));
        xh[k] = x.h;
        xl[k] = x.l;
        df2 qv{qh[k], ql[k]};
        if constexpr (SYM) {   // q = direct part (df) + transposed part (FP64, component-major), consumed here
          const int64_t t = (int64_t)c * qt_stride(n_nodes) + node0 + nl;
          qv = df_add(qv, df_from_bits(qT[t]));
          qT[t] = 0.0;
        }
        const df2 r = df_add(df2{rh[k], rl[k]}, df_mul(na, qv));
        rh[k] = r.h;
        rl[k] = r.l;
        sr[o] = r.h;
        srl[o] = r.l;
      }
    }
    __syncwarp();
    if (lane < nn) {
      float rv[3] = {sr[3 * lane], sr[3 * lane + 1], sr[3 * lane + 2]};
      float zv[3];
      pc3_apply<PC>(spc + PCW * lane, rv, zv);
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        sz[3 * lane + c] = zv[c];
        const df2 r{rv[c], srl[3 * lane + c]};
        df_acc(s0, e0, r, df2{zv[c], 0.f});
        df_acc(s1, e1, r, r);
      }
    }
    __syncwarp();
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const int o = 32 * j + lane;
      if (o < nd) z[d0 + o] = sz[o];
    }
    __syncwarp();
  }
  df2 dv[2] = {df2{s0, e0}, df2{s1, e1}};
  reduce_and_finalize_df<2>(dv, C, op, partials, C->ticket + 1, nullptr);
}

// ---- bulk-copy staged form of pcgx_update_tile_kernel (vec 3, general storage) --------
// A tile's x, r, q (hi and lo), p and preconditioner blocks are eight contiguous runs, so each
// warp streams whole 32-node tiles through a ring of UPD_STAGES shared-memory stages with 1-D
// cp.async.bulk copies (lane 0 issues, one mbarrier per stage) and computes on one tile while the
// next ones are in flight; the plain-load kernel above had only the current tile's loads in
// flight per warp.  Same arithmetic per dof; x, r and z are stored straight from registers.  The
// partial last tile (n_nodes % 32 nodes) is filled with plain loads into a drained stage.
constexpr int UPD_WARPS = 4;
constexpr int UPD_STAGES = 3;

template <int PC, bool SYM = false>
struct UpdGeom {
  static constexpr int PCW = pc_width(PC);
  static constexpr uint32_t VB = 96 * 4;        // one dof-ordered float array of a tile
  static constexpr uint32_t PB = 32 * 4 * 8;    // p: 32 nodes x 4 (hi, lo) pairs
  static constexpr uint32_t CB = 32 * PCW * 4;  // preconditioner blocks
  static constexpr uint32_t QB = SYM ? 3 * 32 * 8 : 0;   // SYM: the tile's qT, three component runs
  static constexpr uint32_t STAGE = 6 * VB + PB + CB + QB;
  static constexpr uint32_t BAR_BYTES = 128;    // UPD_WARPS * UPD_STAGES barriers, padded
  static constexpr uint32_t SMEM = BAR_BYTES + UPD_WARPS * UPD_STAGES * STAGE;
};

// SYM: q is the double-float part of A p plus the FP64 transposed part qT of a symmetric SpMV
// (component c of node i at c * qt_stride + i), streamed with the tile and zeroed once consumed.
template <int PC, bool SYM = false>
__global__ void __launch_bounds__(UPD_WARPS * 32)
pcgx_update_bulk_kernel(int64_t n_nodes, float* __restrict__ xh, float* __restrict__ xl, float* __restrict__ rh,
                        float* __restrict__ rl, float* __restrict__ z, const float2* __restrict__ pp,
                        const float* __restrict__ qh, const float* __restrict__ ql, const float* __restrict__ pc,
                        KCtl* C, double* partials, int op, double* __restrict__ qT = nullptr) {
  using G = UpdGeom<PC, SYM>;
  const int64_t qs = qt_stride(n_nodes);
  constexpr int PCW = G::PCW;
  extern __shared__ __align__(128) unsigned char smem[];
  if (C->done) return;
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem) + wib * UPD_STAGES;
  unsigned char* ring = smem + G::BAR_BYTES + (size_t)wib * UPD_STAGES * G::STAGE;
  const int64_t nfull = n_nodes / 32;   // whole tiles, streamed by bulk copies
  const int64_t nw = (int64_t)gridDim.x * UPD_WARPS;
  const int64_t warp = (int64_t)blockIdx.x * UPD_WARPS + wib;
  if (lane == 0) {
#pragma unroll
    for (int j = 0; j < UPD_STAGES; ++j) mbar_init(bars + j, 1);
    mbar_init_fence();
  }
  __syncwarp();
  const df2 a{C->alpha_h, C->alpha_l};
  const df2 na{-a.h, -a.l};
  float s0 = 0.f, e0 = 0.f, s1 = 0.f, e1 = 0.f;

  int64_t pt = warp;  // producer cursor: next whole tile to copy
  auto produce = [&](int stage) -> bool {
    if (pt >= nfull) return false;
    if (lane == 0) {
      unsigned char* st = ring + (size_t)stage * G::STAGE;
      uint64_t* bar = bars + stage;
      const int64_t d0 = pt * 96;
      async_proxy_fence();
      mbar_expect_tx(bar, G::STAGE);
      // L2 priorities by reuse distance: x, r and the preconditioner come back only in the next
      // iteration's update (after a full matrix stream), so they go evict-first; q (written by the
      // SpMV just before), p and the z written here are read again within this iteration.
      const uint64_t pol = l2_evict_first_policy();
      bulk_load_hint(st, xh + d0, G::VB, bar, pol);
      bulk_load_hint(st + G::VB, xl + d0, G::VB, bar, pol);
      bulk_load_hint(st + 2 * G::VB, rh + d0, G::VB, bar, pol);
      bulk_load_hint(st + 3 * G::VB, rl + d0, G::VB, bar, pol);
      bulk_load(st + 4 * G::VB, qh + d0, G::VB, bar);
      bulk_load(st + 5 * G::VB, ql + d0, G::VB, bar);
      bulk_load(st + 6 * G::VB, pp + pt * 128, G::PB, bar);
      if constexpr (PCW > 0) bulk_load_hint(st + 6 * G::VB + G::PB, pc + pt * 32 * PCW, G::CB, bar, pol);
      if constexpr (SYM) {
#pragma unroll
        for (int c = 0; c < 3; ++c) bulk_load(st + 6 * G::VB + G::PB + G::CB + c * 256, qT + c * qs + pt * 32, 256, bar);
      }
    }
    pt += nw;
    return true;
  };

  // one tile of nn nodes staged at st: x += a p, r -= a q (df), z = M r.h (FP32), dots r.z, r.r
  auto compute = [&](unsigned char* st, int64_t t, int nn) {
    float* sxh = reinterpret_cast<float*>(st);
    float* sxl = sxh + 96;
    float* srh = sxh + 192;
    float* srl = sxh + 288;
    float* sqh = sxh + 384;   // q.h, then z
    const float* sql = sxh + 480;
    const float2* spp = reinterpret_cast<const float2*>(st + 6 * G::VB);
    const float* spc = reinterpret_cast<const float*>(st + 6 * G::VB + G::PB);
    const double* sqt = reinterpret_cast<const double*>(st + 6 * G::VB + G::PB + G::CB);
    const int nd = 3 * nn;
    const int64_t d0 = t * 96;
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const int o = 32 * j + lane;
      if (o < nd) {
        const int nl = o / 3, c = o - 3 * nl;
        const float2 pv = spp[nl * 4 + c];
        const df2 x = df_add(df2{sxh[o], sxl[o]}, df_mul(a, df2{pv.x, pv.y}));
        __stcs(xh + d0 + o, x.h);   // streaming stores: next read one iteration later
        __stcs(xl + d0 + o, x.l);
        df2 qv{sqh[o], sql[o]};
        if constexpr (SYM) qv = df_add(qv, df_from_bits(sqt[c * 32 + nl]));
        const df2 r = df_add(df2{srh[o], srl[o]}, df_mul(na, qv));
        __stcs(rh + d0 + o, r.h);
        __stcs(rl + d0 + o, r.l);
        srh[o] = r.h;
        srl[o] = r.l;
      }
    }
    __syncwarp();
    if (lane < nn) {
      const float rv[3] = {srh[3 * lane], srh[3 * lane + 1], srh[3 * lane + 2]};
      float zv[3];
      pc3_apply<PC>(spc + PCW * lane, rv, zv);
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        sqh[3 * lane + c] = zv[c];
        const df2 r{rv[c], srl[3 * lane + c]};
        df_acc(s0, e0, r, df2{zv[c], 0.f});
        df_acc(s1, e1, r, r);
      }
    }
    __syncwarp();
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const int o = 32 * j + lane;
      if (o < nd) z[d0 + o] = sqh[o];
    }
    if constexpr (SYM) {   // the transposed part is consumed: zero it for the next SpMV
#pragma unroll
      for (int c = 0; c < 3; ++c)
        if (lane < nn) qT[c * qs + t * 32 + lane] = 0.0;
    }
    async_proxy_fence();   // this lane's shared-memory writes before the stage's next bulk copy
    __syncwarp();
  };

  uint32_t parity = 0;  // bit j: phase parity to wait for on stage j
  int inflight = 0;
  for (int j = 0; j < UPD_STAGES; ++j) inflight += produce(j) ? 1 : 0;
  int stage = 0;
  bool fault = false;
  for (int64_t t = warp; t < nfull; t += nw) {
    const bool ok = mbar_wait(bars + stage, (parity >> stage) & 1u);
    if (!__all_sync(0xffffffffu, ok)) { fault = true; break; }
    parity ^= 1u << stage;
    --inflight;
    compute(ring + (size_t)stage * G::STAGE, t, 32);
    inflight += produce(stage) ? 1 : 0;
    stage = stage + 1 == UPD_STAGES ? 0 : stage + 1;
  }
  if (fault) {
    // let the copies already issued land (bounded) before the CTA's shared memory is released
    for (int j = 0; j < inflight; ++j) {
      (void)mbar_wait(bars + stage, (parity >> stage) & 1u);
      parity ^= 1u << stage;
      stage = stage + 1 == UPD_STAGES ? 0 : stage + 1;
    }
    if (lane == 0) {
      atomicExch(&C->fault, 1);
      atomicExch(&C->done, 1);
    }
  } else if (n_nodes % 32 != 0 && warp == nfull % nw) {
    // partial last tile: plain loads into stage 0 (every copy of this warp has landed)
    const int nn = (int)(n_nodes - nfull * 32);
    const int64_t d0 = nfull * 96;
    float* s = reinterpret_cast<float*>(ring);
    for (int o = lane; o < 96; o += 32) {
      const bool in = o < 3 * nn;
      s[o] = in ? xh[d0 + o] : 0.f;
      s[96 + o] = in ? xl[d0 + o] : 0.f;
      s[192 + o] = in ? rh[d0 + o] : 0.f;
      s[288 + o] = in ? rl[d0 + o] : 0.f;
      s[384 + o] = in ? qh[d0 + o] : 0.f;
      s[480 + o] = in ? ql[d0 + o] : 0.f;
    }
    float2* spp = reinterpret_cast<float2*>(ring + 6 * G::VB);
    for (int o = lane; o < 128; o += 32) spp[o] = o < 4 * nn ? pp[nfull * 128 + o] : make_float2(0.f, 0.f);
    if constexpr (PCW > 0) {
      float* spc = reinterpret_cast<float*>(ring + 6 * G::VB + G::PB);
      for (int o = lane; o < 32 * PCW; o += 32) spc[o] = o < PCW * nn ? pc[nfull * 32 * PCW + o] : 0.f;
    }
    if constexpr (SYM) {
      double* sqt = reinterpret_cast<double*>(ring + 6 * G::VB + G::PB + G::CB);
      for (int c = 0; c < 3; ++c) sqt[c * 32 + lane] = lane < nn ? qT[c * qs + nfull * 32 + lane] : 0.0;
    }
    __syncwarp();
    compute(ring, nfull, nn);
  }
  df2 dv[2] = {df2{s0, e0}, df2{s1, e1}};
  reduce_and_finalize_df<2>(dv, C, op, partials, C->ticket + 1, nullptr);
}

// vec-3 form of pcgx_direction_kernel, thread per dof: z coalesced, p gathered within the tile.
__global__ void pcgx_direction3_kernel(int64_t n, const float* __restrict__ z, float2* __restrict__ pp,
                                       const KCtl* C) {
  if (C->done) return;
  const df2 b{C->beta_h, C->beta_l};
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = k / 3;
    const int64_t o = i * 4 + (k - 3 * i);
    const float2 pv = pp[o];
    const df2 p = df_add(df2{__ldcs(z + k), 0.f}, df_mul(b, df2{pv.x, pv.y}));   // z: last use
    pp[o] = make_float2(p.h, p.l);
  }
}

// p = z + beta p (df), the SpMV input of the next iteration
template <int VEC>
__global__ void pcgx_direction_kernel(int64_t n_nodes, const float* z, float2* pp, const KCtl* C) {
  constexpr int PAD = DfNode<VEC>::PAD;
  if (C->done) return;
  const df2 b{C->beta_h, C->beta_l};
  GRID_STRIDE_NODES(i, n_nodes) {
#pragma unroll
    for (int c = 0; c < VEC; ++c) {
      const float2 pv = pp[i * PAD + c];
      const df2 p = df_add(df2{z[VEC * i + c], 0.f}, df_mul(b, df2{pv.x, pv.y}));
      pp[i * PAD + c] = make_float2(p.h, p.l);
    }
  }
}

// df <-> FP64 for the reliable updates: (r.h, r.l) = split(r64 * scale), and the accumulation below.
// scale is a power of two (exact both ways): it keeps the double-float vectors of a solve near
// unit size, away from the ends of FP32's exponent range.
// x64 += x (df) / scale ; x (df) := 0: a reliable update moves the correction that the double-float
// iteration accumulated since the last update into the FP64 iterate, so the iterate itself keeps
// FP64 precision (a 48-bit double-float iterate would floor the true residual near kappa * 2^-48)
__global__ void df_accumulate_kernel(int64_t n, float* h, float* l, double* x64, double inv_scale) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    x64[k] += ((double)h[k] + (double)l[k]) * inv_scale;
    h[k] = 0.f;
    l[k] = 0.f;
  }
}
__global__ void f64_to_df_kernel(int64_t n, const double* v, float* h, float* l, double scale) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    const df2 d = df_of(v[k] * scale);
    h[k] = d.h;
    l[k] = d.l;
  }
}

// FP64 true residual r = b - A x (Dirichlet rows: b - x) and ||r||^2
__global__ void refine_residual64_kernel(int64_t n, const double* b, const double* x, const double* ax,
                                         const uint8_t* bc, double* r, KCtl* C, double* partials) {
  double dv[3] = {0, 0, 0};
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    const double v = (bc && bc[k]) ? (b[k] - x[k]) : (b[k] - ax[k]);
    r[k] = v;
    dv[0] += v * v;
  }
  reduce_and_finalize<1>(dv, C, FIN_REF_TRUE, partials, C->ticket + 1, nullptr);
}

template <typename T>
__global__ void pcg_direction_kernel(int64_t n, T* p, const T* z, const KCtl* C) {
  if (C->done) return;
  const T beta = T(C->beta);
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
    p[k] = __ldcs(z + k) + beta * p[k];   // z: last use
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
__global__ void dot_kernel(int64_t n, const T* x, const T* y, KCtl* C, double* partials, double* out,
                           int op = FIN_DOT) {
  double dv[3] = {0, 0, 0};
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
    dv[0] += double(x[k]) * double(y[k]);
  reduce_and_finalize<1>(dv, C, op, partials, C->ticket + 2, out);
}

__global__ void init_ctl_kernel(KCtl* C, double thresh2_rel, double atol2, long long maxiter) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    C->done = 0; C->status = 0; C->exit_early = 0; C->fault = 0;
    C->thresh2 = thresh2_rel; C->d1 = atol2; C->maxiter = maxiter; C->iter = 0;
    C->ticket[0] = C->ticket[1] = C->ticket[2] = C->ticket[3] = 0;
    C->alpha_h = C->alpha_l = C->beta_h = C->beta_l = 0.f;
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

// A^T in the same node-block CSR pattern (the pattern is structurally symmetric: the union of
// every cell's dof pairs).  Thread per node row I: for each block (I, J) it finds block (J, I) in
// row J by binary search and writes the transposed block, value (r, d) of (I, J) := value (d, r)
// of (J, I).  Rows are independent, so the output needs no atomics.
template <typename T>
__global__ void transpose_kernel(int vec, int64_t n_nodes, const int64_t* __restrict__ bp,
                                 const int32_t* __restrict__ bcols, const T* __restrict__ v, T* __restrict__ vt,
                                 int* __restrict__ err) {
  GRID_STRIDE_NODES(I, n_nodes) {
    const int64_t bI = bp[I];
    const int nI = (int)(bp[I + 1] - bI);
    for (int k = 0; k < nI; ++k) {
      const int64_t J = bcols[bI + k];
      const int64_t bJ = bp[J];
      const int nJ = (int)(bp[J + 1] - bJ);
      int lo = 0, hi = nJ - 1, kt = -1;
      while (lo <= hi) {
        const int mid = (lo + hi) >> 1;
        const int64_t c = bcols[bJ + mid];
        if (c == I) { kt = mid; break; }
        if (c < I) lo = mid + 1; else hi = mid - 1;
      }
      if (kt < 0) { atomicExch(err, 1); continue; }   // pattern not structurally symmetric
      for (int r = 0; r < vec; ++r)
        for (int d = 0; d < vec; ++d)
          vt[(int64_t)vec * vec * bI + (int64_t)r * vec * nI + vec * k + d] =
              v[(int64_t)vec * vec * bJ + (int64_t)d * vec * nJ + vec * kt + r];
    }
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

// 8 vectors of n_dofs elements plus 4 KB of alignment slack: the double-float CG carves 7 float
// vectors, a node-interleaved direction (<= 11 bytes per dof) and 3 double vectors from the
// FP64 size, i.e. <= 63 n bytes plus 256-byte rounding of each of its 11 arrays.
static size_t krylov_ws_bytes(int64_t n_dofs, int precision) {
  const size_t es = precision == FEM_F32 ? 4 : 8;
  return al(sizeof(KCtl)) + al(sizeof(double) * 3 * MAX_PARTIAL_BLOCKS) + 8 * al(es * (size_t)n_dofs) + 4096;
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
  int g = grid_for(n, VTHREADS, 8);
  return g > MAX_PARTIAL_BLOCKS ? MAX_PARTIAL_BLOCKS : g;
}


template <typename K>
static int spmv_blocks_per_sm(K kern) {
  int b = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, kern, SPMV_THREADS, 0) != cudaSuccess || b < 1) b = 4;
  return b;
}

// Grid = resident CTAs (no partial waves), capped by the rows to process.
template <int VEC, int FMT, int ND>
static void launch_spmv_fmt(const fem_pattern_t* pat, int64_t n_nodes, const void* vals, const int16_t* vlo,
                            const void* x, const float* xlo, void* y, const void* a, KCtl* C, int op,
                            double* partials, cudaStream_t s) {
  using Tp = SpmvTypes<FMT>;
  auto kern = spmv_kernel<VEC, FMT, ND>;
  static int per_sm = 0;
  if (per_sm == 0) per_sm = spmv_blocks_per_sm(kern);
  const int64_t need = (n_nodes * SPMV_G + SPMV_THREADS - 1) / SPMV_THREADS;
  int64_t g = (int64_t)sm_count() * per_sm;
  if (g > need) g = need;
  if (g > MAX_PARTIAL_BLOCKS) g = MAX_PARTIAL_BLOCKS;
  if (g < 1) g = 1;
  kern<<<(unsigned)g, SPMV_THREADS, 0, s>>>(n_nodes, pat->block_ptr, pat->block_cols,
                                             (const typename Tp::V*)vals, vlo, (const typename Tp::X*)x, xlo,
                                             (typename Tp::Y*)y, (const typename Tp::Y*)a, C, op, partials, 0);
  note_launches(1);
}

template <int VEC, int FMT>
static void launch_spmv_nd(const fem_pattern_t* pat, int64_t n_nodes, const void* vals, const int16_t* vlo,
                           const void* x, const float* xlo, void* y, const void* a, KCtl* C, int op,
                           double* partials, int nd, cudaStream_t s) {
  if (nd == 0) launch_spmv_fmt<VEC, FMT, 0>(pat, n_nodes, vals, vlo, x, xlo, y, a, C, op, partials, s);
  else if (nd == 1) launch_spmv_fmt<VEC, FMT, 1>(pat, n_nodes, vals, vlo, x, xlo, y, a, C, op, partials, s);
  else launch_spmv_fmt<VEC, FMT, 2>(pat, n_nodes, vals, vlo, x, xlo, y, a, C, op, partials, s);
}

template <int VEC, int FMT, int ND>
static void launch_spmv_sliced(const fem_pattern_t* pat, int64_t n_nodes, const void* vals, const int16_t* vlo,
                               const void* x, const float* xlo, void* y, const void* a, KCtl* C, int op,
                               double* partials, cudaStream_t s) {
  using Tp = SpmvTypes<FMT>;
  auto kern = spmv_sliced_kernel<VEC, FMT, ND>;
  static int per_sm = 0;
  if (per_sm == 0) per_sm = spmv_blocks_per_sm(kern);
  const int64_t need = (pat->n_slices * 32 + SPMV_THREADS - 1) / SPMV_THREADS;
  int64_t g = (int64_t)sm_count() * per_sm;
  if (g > need) g = need;
  if (g > MAX_PARTIAL_BLOCKS) g = MAX_PARTIAL_BLOCKS;
  if (g < 1) g = 1;
  kern<<<(unsigned)g, SPMV_THREADS, 0, s>>>(n_nodes, pat->n_slices, pat->slice_ptr, pat->slice_cols,
                                             (const typename Tp::V*)vals, vlo, (const typename Tp::X*)x, xlo,
                                             (typename Tp::Y*)y, (const typename Tp::Y*)a, C, op, partials, 0);
  note_launches(1);
}

// One entry for every value format: mfmt is the FEM_* precision of `vals`.
template <int VEC, int FMT>
static void launch_spmv_any(const fem_pattern_t* pat, int64_t n_nodes, int mfmt, const void* vals, const int16_t* vlo,
                            const void* x, const float* xlo, void* y, const void* a, KCtl* C, int op,
                            double* partials, int nd, cudaStream_t s) {
  if (mfmt >= FEM_SLICED_F32) {
    if (nd == 0) launch_spmv_sliced<VEC, FMT, 0>(pat, n_nodes, vals, vlo, x, xlo, y, a, C, op, partials, s);
    else if (nd == 1) launch_spmv_sliced<VEC, FMT, 1>(pat, n_nodes, vals, vlo, x, xlo, y, a, C, op, partials, s);
    else launch_spmv_sliced<VEC, FMT, 2>(pat, n_nodes, vals, vlo, x, xlo, y, a, C, op, partials, s);
  } else {
    launch_spmv_nd<VEC, FMT>(pat, n_nodes, vals, vlo, x, xlo, y, a, C, op, partials, nd, s);
  }
}

template <int VEC, typename T>
static void launch_spmv(const fem_pattern_t* pat, int64_t n_nodes, const T* vals, const T* x, T* y, const T* a,
                        KCtl* C, int op, double* partials, int nd, cudaStream_t s, int mfmt = -1) {
  constexpr int FMT = sizeof(T) == 4 ? FMT_F32 : FMT_F64;
  if (mfmt < 0) mfmt = sizeof(T) == 4 ? FEM_F32 : FEM_F64;
  launch_spmv_any<VEC, FMT>(pat, n_nodes, mfmt, vals, nullptr, x, nullptr, y, a, C, op, partials, nd, s);
}

// Optional in-solve timing of the mixed CG's SpMV (fem_spmv_timing_start / _stop): a CUDA event
// pair around the second SpMV of every CHUNK-iteration chunk, on the solver's stream, read back
// at the next poll (which has synchronised the stream).  Process-wide; not for concurrent solves.
struct SpmvTimer {
  bool on = false;
  cudaEvent_t ev[2 * 64] = {};
  int used = 0;          // pairs recorded since the last read-back
  double seconds = 0.0;  // summed durations
  int64_t samples = 0;
  cudaEvent_t gev[2] = {};   // the pair recorded by a captured chunk (ChunkGraph), once per replay
  bool graph_pending = false;
};
static SpmvTimer g_spmv_timer;

// Record one of the captured chunk's pair while a ChunkGraph is being captured on st.
static void spmv_timer_mark_graph(int end, cudaStream_t st) {
  SpmvTimer& T = g_spmv_timer;
  if (!T.on) return;
  cudaEvent_t& e = T.gev[end];
  if (!e) return;   // created before the capture (ChunkGraph::build)
  // an external record node: a plain record inside a capture only orders the captured work
  cudaEventRecordWithFlags(e, st, cudaEventRecordExternal);
}

static void spmv_timer_mark(int end, cudaStream_t s) {
  SpmvTimer& T = g_spmv_timer;
  if (!T.on || T.used >= 64) return;
  cudaEvent_t& e = T.ev[2 * T.used + end];
  if (!e && cudaEventCreate(&e) != cudaSuccess) { e = nullptr; T.on = false; return; }
  cudaEventRecord(e, s);
  if (end) ++T.used;
}

static void spmv_timer_collect() {
  SpmvTimer& T = g_spmv_timer;
  if (T.graph_pending && T.gev[0] && T.gev[1]) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, T.gev[0], T.gev[1]) == cudaSuccess) {
      T.seconds += 1e-3 * ms;
      ++T.samples;
    } else {
      cudaGetLastError();   // a measurement miss must not surface as a later launch error
    }
  }
  T.graph_pending = false;
  for (int k = 0; k < T.used; ++k) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, T.ev[2 * k], T.ev[2 * k + 1]) == cudaSuccess) {
      T.seconds += 1e-3 * ms;
      ++T.samples;
    } else {
      cudaGetLastError();
    }
  }
  T.used = 0;
}

static int poll(KCtl* C, cudaStream_t s, KCtl* host) {
  FEM_CUDA(cudaMemcpyAsync(host, C, sizeof(KCtl), cudaMemcpyDeviceToHost, s));
  FEM_CUDA(cudaStreamSynchronize(s));
  if (g_spmv_timer.used || g_spmv_timer.graph_pending) spmv_timer_collect();
  if (host->fault) return fail(FEM_ERR_DEVICE, "a bounded device wait (bulk-copy barrier) ran out");
  return FEM_OK;
}

// One chunk of a Krylov loop captured as a CUDA graph and replayed.  The chunk's kernels are the
// same launch after launch (fixed pointers; the scalars live in the control block), so one capture
// per solve replaces 3 x CHUNK stream launches by one graph launch.  The capture runs on a private
// non-blocking stream (the caller's stream may be the legacy default stream, which cannot be
// captured); the replays go to the caller's stream.  Launch counts: the kernels recorded during
// the capture did not run, so they are taken back and credited at every replay.
struct ChunkGraph {
  cudaGraphExec_t exec = nullptr;
  uint64_t launches = 0;     // kernels per replay
  bool timed = false;        // the capture recorded the SpMV timing pair
  ChunkGraph() = default;
  ChunkGraph(const ChunkGraph&) = delete;
  ChunkGraph& operator=(const ChunkGraph&) = delete;
  ~ChunkGraph() {
    if (exec) cudaGraphExecDestroy(exec);
  }
  // launch_chunk(stream) launches one chunk and returns FEM_OK; false: no graph (plain launches)
  template <class F>
  bool build(F&& launch_chunk) {
    // an error left by the launches queued just before stays for the caller's check_launch
    if (cudaPeekAtLastError() != cudaSuccess) return false;
    cudaStream_t cs = nullptr;
    if (cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking) != cudaSuccess) { cudaGetLastError(); return false; }
    const uint64_t l0 = fem_kernel_launches();
    timed = g_spmv_timer.on;
    for (int k = 0; k < 2 && timed; ++k)   // the timing pair exists before the capture records it
      if (!g_spmv_timer.gev[k] && cudaEventCreate(&g_spmv_timer.gev[k]) != cudaSuccess) {
        g_spmv_timer.gev[k] = nullptr;
        timed = false;
        cudaGetLastError();
      }
    bool ok = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
    int rc = FEM_OK;
    if (ok) rc = launch_chunk(cs);
    cudaGraph_t g = nullptr;
    if (ok) ok = cudaStreamEndCapture(cs, &g) == cudaSuccess && g != nullptr && rc == FEM_OK;
    if (ok) ok = cudaGraphInstantiate(&exec, g, 0) == cudaSuccess;
    if (g) cudaGraphDestroy(g);
    cudaStreamDestroy(cs);
    const uint64_t captured = fem_kernel_launches() - l0;
    note_launches(-(int)captured);
    launches = captured;
    if (!ok) {
      if (exec) cudaGraphExecDestroy(exec);
      exec = nullptr;
    }
    cudaGetLastError();   // a failed capture leaves its error behind
    return ok;
  }
  int launch(cudaStream_t s) {
    FEM_CUDA(cudaGraphLaunch(exec, s));
    note_launches((int)launches);
    if (timed && g_spmv_timer.on) g_spmv_timer.graph_pending = true;
    return FEM_OK;
  }
  // The next chunk of a loop: a replay of the captured chunk while a full chunk remains, plain
  // launches otherwise.  The capture follows the first plain chunk (whose launches set up the
  // launchers' occupancy state) as soon as it is queued, so the host captures and instantiates
  // while the GPU runs that chunk.  run_iters(stream, k, captured) launches k iterations.
  template <class F>
  int step(cudaStream_t s, int64_t& launched, int64_t maxiter, F&& run_iters) {
    if (exec && maxiter - launched >= CHUNK) {
      const int rc = launch(s);
      if (rc) return rc;
      launched += CHUNK;
      return FEM_OK;
    }
    const int k = (int)std::min<int64_t>(CHUNK, maxiter - launched);
    const int rc = run_iters(s, k, false);
    if (rc) return rc;
    launched += k;
    if (!tried && maxiter - launched >= CHUNK) {
      tried = true;
      build([&](cudaStream_t cs) { return run_iters(cs, CHUNK, true); });
    }
    return FEM_OK;
  }
  bool tried = false;   // set to skip graphs (the allocation-free entry point)
};

static bool aligned16(const void* p) { return ((uintptr_t)p & 15u) == 0; }

// The mixed CG's update (vec 3, general storage) by the bulk-copy staged kernel; false when an
// array is not 16-byte aligned (the caller then launches pcgx_update_tile_kernel).  Grid:
// resident CTAs, capped by the tiles.
template <int PC, bool SYM = false>
static bool launch_update_bulk(int64_t n_nodes, float* xh, float* xl, float* rh, float* rl, float* z,
                               const float2* pp, const float* qh, const float* ql, const float* pc, KCtl* C,
                               double* partials, int op, cudaStream_t s, double* qT = nullptr) {
  using G = UpdGeom<PC, SYM>;
  if (!(aligned16(xh) && aligned16(xl) && aligned16(rh) && aligned16(rl) && aligned16(pp) && aligned16(qh) &&
        aligned16(ql) && (G::PCW == 0 || aligned16(pc)) && (!SYM || aligned16(qT))))
    return false;
  auto kern = pcgx_update_bulk_kernel<PC, SYM>;
  constexpr int smem = (int)G::SMEM;
  static int per_sm = 0;
  if (per_sm == 0) {
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, UPD_WARPS * 32, smem) != cudaSuccess ||
        per_sm < 1)
      per_sm = 1;
  }
  int64_t g = (int64_t)sm_count() * per_sm;
  const int64_t need = ((n_nodes + 31) / 32 + UPD_WARPS - 1) / UPD_WARPS;
  if (g > need) g = need;
  if (g > MAX_PARTIAL_BLOCKS) g = MAX_PARTIAL_BLOCKS;
  if (g < 1) g = 1;
  kern<<<(unsigned)g, UPD_WARPS * 32, smem, s>>>(n_nodes, xh, xl, rh, rl, z, pp, qh, ql, pc, C, partials, op, qT);
  return true;
}

// The mixed CG's SpMV: bulk-copy staged kernel for vec 3 when the streamed arrays are 16-byte
// aligned, the register-streaming kernel otherwise.  Grid: resident CTAs, capped by the slices.
// SYM (FEM_SYM_DF48, vec 3 only): the upper-block layout, transposed part into qT.
template <int VEC, bool SYM = false>
static int launch_dfdf(const fem_pattern_t* pat, int64_t n_nodes, const float* vhi, const int16_t* vlo,
                       const float2* xp, float* yh, float* yl, KCtl* C, int op, double* partials, cudaStream_t s,
                       double* qT = nullptr) {
  const int64_t ns = pat->n_slices;
  const int64_t* sp = SYM ? pat->slice_ptr_u : pat->slice_ptr;
  const int32_t* sc = SYM ? pat->slice_cols_u : pat->slice_cols;
  const bool bulk = VEC == 3 && aligned16(vhi) && aligned16(vlo) && aligned16(sc);
  if (SYM && !(bulk && qT)) return fail(FEM_ERR_ARG, "FEM_SYM_DF48 needs vec 3 and 16-byte aligned arrays");
  if (bulk) {
    constexpr int smem = (int)BulkGeom<VEC>::SMEM;
    auto prepare = [&](auto kern, int& per_sm) -> unsigned {
      if (per_sm == 0) {
        cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
        if (smem > 48 * 1024) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, BULK_WARPS * 32, smem) != cudaSuccess ||
            per_sm < 1)
          per_sm = 1;
      }
      int64_t g = (int64_t)sm_count() * per_sm;
      const int64_t need = (ns + BULK_WARPS - 1) / BULK_WARPS;
      if (g > need) g = need;
      if (g > MAX_PARTIAL_BLOCKS) g = MAX_PARTIAL_BLOCKS;
      return (unsigned)(g < 1 ? 1 : g);
    };
    if constexpr (!SYM && VEC == 3) {
      if (pat->slices_grid) {   // grid layout: columns from the stencil, none streamed
        auto kern = spmv_sliced_dfdf_bulk_kernel<VEC, false, true>;
        static int per_sm_grid = 0;
        const unsigned g = prepare(kern, per_sm_grid);
        kern<<<g, BULK_WARPS * 32, smem, s>>>(n_nodes, ns, sp, sc, vhi, vlo, xp, yh, yl, C, op, partials, qT,
                                              pat->grid_ny, pat->grid_nz);
        note_launches(1);
        return FEM_OK;
      }
    }
    auto kern = spmv_sliced_dfdf_bulk_kernel<VEC, SYM>;
    static int per_sm = 0;
    const unsigned g = prepare(kern, per_sm);
    kern<<<g, BULK_WARPS * 32, smem, s>>>(n_nodes, ns, sp, sc, vhi, vlo, xp, yh, yl, C, op, partials, qT, 0, 0);
  } else {
    auto kern = spmv_sliced_dfdf_kernel<VEC>;
    static int per_sm = 0;
    if (per_sm == 0) per_sm = spmv_blocks_per_sm(kern);
    int64_t g = (int64_t)sm_count() * per_sm;
    const int64_t need = (ns * 32 + SPMV_THREADS - 1) / SPMV_THREADS;
    if (g > need) g = need;
    if (g > MAX_PARTIAL_BLOCKS) g = MAX_PARTIAL_BLOCKS;
    if (g < 1) g = 1;
    kern<<<(unsigned)g, SPMV_THREADS, 0, s>>>(n_nodes, ns, sp, sc, vhi, vlo, xp, yh, yl, C, op, partials);
  }
  note_launches(1);
  return FEM_OK;
}

// The structured symmetric SpMV (FEM_SSYM_DF48).  Work items are (group of 32 lines, k range);
// the groups are cut into as few k ranges as fill the resident warps in one round (every cut adds
// boundary rows whose transposed parts go through atomics).  Grid: min(items, resident warps)
// warps.  Needs 16-byte aligned values and corrections.
static int launch_ssym(const fem_pattern_t* pat, const float* vhi, const int16_t* vlo, const float2* xp, float* yh,
                       float* yl, double* qT, KCtl* C, int op, double* partials, cudaStream_t s) {
  if (!(aligned16(vhi) && aligned16(vlo) && qT))
    return fail(FEM_ERR_ARG, "FEM_SSYM_DF48 needs 16-byte aligned values and a transposed-part vector");
  auto kern = spmv_ssym_bulk_kernel;
  constexpr int smem = (int)SsGeom::SMEM;
  static int per_sm = 0;
  if (per_sm == 0) {
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, SS_WARPS * 32, smem) != cudaSuccess ||
        per_sm < 1)
      per_sm = 1;
  }
  const int64_t resident = (int64_t)sm_count() * per_sm * SS_WARPS;
  const SsGrid G0 = ss_grid(pat, 1);
  const int chunks = (int)std::max<int64_t>(1, std::min<int64_t>(G0.nz, resident / std::max<int64_t>(G0.groups, 1)));
  const SsGrid G = ss_grid(pat, chunks);
  int64_t warps = std::min<int64_t>(G.groups * G.chunks, resident);
  int64_t g = (warps + SS_WARPS - 1) / SS_WARPS;
  if (g > MAX_PARTIAL_BLOCKS) g = MAX_PARTIAL_BLOCKS;
  if (g < 1) g = 1;
  kern<<<(unsigned)g, SS_WARPS * 32, smem, s>>>(G, vhi, vlo, xp, yh, yl, qT, C, op, partials);
  note_launches(1);
  return FEM_OK;
}

template <int VEC, typename T, int PC>
static int pcg_impl(const fem_pattern_t* pat, int64_t n_nodes, const T* vals, const T* pc, const T* b, T* x,
                    double rtol, double atol, int64_t maxiter, void* ws, int64_t* iters, double* rnorm,
                    int32_t* status, cudaStream_t s, int mfmt, bool graphs = true) {
  const int64_t n = n_nodes * VEC;
  KWs w = carve(ws, n, sizeof(T) == 4 ? FEM_F32 : FEM_F64);
  T* r = reinterpret_cast<T*>(w.vecs);
  T* z = reinterpret_cast<T*>(w.vecs + w.vec_bytes);
  T* p = reinterpret_cast<T*>(w.vecs + 2 * w.vec_bytes);
  T* q = reinterpret_cast<T*>(w.vecs + 3 * w.vec_bytes);
  KCtl* C = w.ctl;
  init_ctl_kernel<<<1, 32, 0, s>>>(C, rtol * rtol, atol * atol, (long long)maxiter);
  note_launches(1);
  launch_spmv<VEC, T>(pat, n_nodes, vals, x, q, nullptr, nullptr, FIN_NONE, nullptr, 0, s, mfmt);
  pcg_init_kernel<VEC, T, PC><<<vec_grid(n_nodes), VTHREADS, 0, s>>>(n_nodes, b, q, r, z, p, pc, C, w.partials);
  note_launches(1);
  int rc = check_launch("pcg init");
  if (rc) return rc;
  KCtl h;
  int64_t launched = 0;
  auto run_iters = [&](cudaStream_t st, int k_count, bool) -> int {
    for (int k = 0; k < k_count; ++k) {
      launch_spmv<VEC, T>(pat, n_nodes, vals, p, q, p, C, FIN_PCG_ALPHA, w.partials, 1, st, mfmt);
      pcg_update_kernel<VEC, T, PC><<<vec_grid(n_nodes), VTHREADS, 0, st>>>(n_nodes, x, r, z, p, q, pc, C,
                                                                             w.partials, FIN_PCG_UPDATE);
      note_launches(1);
      pcg_direction_kernel<T><<<vec_grid(n), VTHREADS, 0, st>>>(n, p, z, C);
      note_launches(1);
    }
    return FEM_OK;
  };
  // full chunks after the first replay one captured chunk (ChunkGraph); the allocation-free entry
  // point keeps plain launches (instantiating a graph allocates)
  ChunkGraph graph;
  graph.tried = !graphs;
  while (true) {
    rc = poll(C, s, &h);
    if (rc) return rc;
    if (h.done || launched >= maxiter) break;
    rc = graph.step(s, launched, maxiter, run_iters);
    if (rc) return rc;
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
                     int32_t* status, cudaStream_t s, int mfmt) {
  const int64_t n = n_nodes * VEC;
  KWs w = carve(ws, n, sizeof(T) == 4 ? FEM_F32 : FEM_F64);
  T* v[8];
  for (int k = 0; k < 8; ++k) v[k] = reinterpret_cast<T*>(w.vecs + k * w.vec_bytes);
  T *r = v[0], *rhat = v[1], *p = v[2], *phat = v[3], *q = v[4], *sv = v[5], *shat = v[6], *t = v[7];
  KCtl* C = w.ctl;
  init_ctl_kernel<<<1, 32, 0, s>>>(C, tol * tol, atol * atol, (long long)maxiter);
  note_launches(1);
  launch_spmv<VEC, T>(pat, n_nodes, vals, x, q, nullptr, nullptr, FIN_NONE, nullptr, 0, s, mfmt);
  bicg_init_kernel<T><<<vec_grid(n), VTHREADS, 0, s>>>(n, b, q, r, rhat, p, C, w.partials);
  note_launches(1);
  int rc = check_launch("bicgstab init");
  if (rc) return rc;
  KCtl h;
  int64_t launched = 0;
  auto run_iters = [&](cudaStream_t st, int k_count, bool) -> int {
    for (int k = 0; k < k_count; ++k) {
      bicg_p_kernel<VEC, T, PC><<<vec_grid(n_nodes), VTHREADS, 0, st>>>(n_nodes, r, p, q, phat, pc, C);
      note_launches(1);
      launch_spmv<VEC, T>(pat, n_nodes, vals, phat, q, rhat, C, FIN_BICG_ALPHA, w.partials, 1, st, mfmt);
      bicg_s_kernel<VEC, T, PC><<<vec_grid(n_nodes), VTHREADS, 0, st>>>(n_nodes, r, q, sv, shat, pc, C, w.partials);
      note_launches(1);
      launch_spmv<VEC, T>(pat, n_nodes, vals, shat, t, sv, C, FIN_BICG_OMEGA, w.partials, 2, st, mfmt);
      bicg_update_kernel<T><<<vec_grid(n), VTHREADS, 0, st>>>(n, x, r, rhat, phat, sv, shat, t, C, w.partials);
      note_launches(1);
    }
    return FEM_OK;
  };
  ChunkGraph graph;
  while (true) {
    rc = poll(C, s, &h);
    if (rc) return rc;
    if (h.done || launched >= maxiter) break;
    rc = graph.step(s, launched, maxiter, run_iters);
    if (rc) return rc;
    rc = check_launch("bicgstab iteration");
    if (rc) return rc;
  }
  if (iters) *iters = h.iter;
  if (rnorm) *rnorm = std::sqrt(h.rr);
  if (status) *status = h.done ? h.status : FEM_SOLVE_MAXITER;
  return FEM_OK;
}

// FP64 operator of the reliable updates: an FP64 matrix (CSR or sliced) when given, else
// the matrix-free tangent action of `mat` at u_lin.  ax := K x (Dirichlet-eliminated).
struct RefOp {
  const fem_mesh_t* mesh;
  const fem_material_t* mat;
  const double* u_lin;
  const void* vals;
  int prec;
  const uint8_t* bc;
};

template <int VEC>
static int ref_apply(const fem_pattern_t* pat, int64_t n_nodes, const RefOp& op, const double* x, double* ax,
                     cudaStream_t s) {
  if (op.vals) {
    launch_spmv<VEC, double>(pat, n_nodes, (const double*)op.vals, x, ax, nullptr, nullptr, FIN_NONE, nullptr, 0, s,
                             op.prec);
    return check_launch("reliable-update SpMV");
  }
  FEM_CUDA(cudaMemsetAsync(ax, 0, sizeof(double) * (size_t)(n_nodes * VEC), s));
  return fem_assemble(op.mesh, op.mat, pat, FEM_OUT_APPLY, FEM_F64, op.u_lin, x, op.bc, FEM_BC_SYMMETRIC, nullptr,
                      nullptr, ax, s);
}

// FP32 PCG with FP64 reliable updates (residual replacement).  The iteration runs on
// the FP32 matrix; whenever the FP32 recursive residual has fallen by `delta` since the
// last replacement (or below a quarter of the target), the device pauses, the host adds
// the FP32 increment into the FP64 solution and recomputes the true residual b - A x in
// FP64 (with the FP64 CSR tangent when given, else the matrix-free tangent action,
// fem_assemble FEM_OUT_APPLY), which replaces the FP32 residual.  The search direction is
// kept, so the Krylov recurrence continues instead of restarting.  Convergence is declared
// only on the FP64 true residual; three replacements in a row that do not cut it by
// stall_factor(delta) end the solve as stagnated.  r and the increment carry a power-of-two scale (see below).
// Progress an FP64 residual replacement must show to reset the stagnation count: the squared
// true residual below this fraction of the best so far.  A healthy replacement follows a pause
// of the recursive residual at delta^2 of its start, so it cuts the squared true residual by
// about delta^2; the fraction max(1/4, delta) sits above that for every delta in (0, 1) and is
// the plain "halve the norm" rule for delta <= 1/4.
static inline double stall_factor(double delta) { return std::max(0.25, delta); }

template <int VEC, int PC>
static int pcg_refined_impl(const fem_pattern_t* pat, int64_t n_nodes, const float* vals, const float* pc,
                            const RefOp& op, const double* b, double* x, double rtol, double atol, double delta,
                            int64_t maxiter, void* ws, int64_t* iters, int64_t* updates, double* rnorm,
                            int32_t* status, cudaStream_t s, int mfmt) {
  const uint8_t* bc = op.bc;
  const int64_t n = n_nodes * VEC;
  KWs w = carve(ws, n, FEM_F64);
  const size_t f4 = al(sizeof(float) * (size_t)n);
  float* r = reinterpret_cast<float*>(w.vecs);
  float* z = reinterpret_cast<float*>(w.vecs + f4);
  float* p = reinterpret_cast<float*>(w.vecs + 2 * f4);
  float* q = reinterpret_cast<float*>(w.vecs + 3 * f4);
  float* x32 = reinterpret_cast<float*>(w.vecs + 4 * f4);
  double* ax = reinterpret_cast<double*>(w.vecs + 5 * f4);
  KCtl* C = w.ctl;
  init_ctl_kernel<<<1, 32, 0, s>>>(C, rtol * rtol, atol * atol, (long long)maxiter);
  dot_kernel<double><<<vec_grid(n), VTHREADS, 0, s>>>(n, b, b, C, w.partials, nullptr, FIN_REF_BB);
  note_launches(2);
  int rc = check_launch("pcg_refined init");
  if (rc) return rc;
  KCtl h;
  rc = poll(C, s, &h);
  if (rc) return rc;
  // r and the correction x32 are carried times a power of two that brings b's RMS near 1 (fixed
  // for the solve), so that the FP32 iteration stays inside FP32's exponent range however the
  // problem is scaled; the pause threshold on the recursive residual is rescaled to match.
  double scale = 1.0;
  if (h.bb > 0.0 && std::isfinite(h.bb)) {
    const int e = std::ilogb(std::sqrt(h.bb / (double)n));
    scale = std::ldexp(1.0, -std::max(-900, std::min(900, e)));
  }
  const double inv_scale = 1.0 / scale;
  const double check2 = h.check2 * scale * scale;
  auto true_residual = [&]() -> int {
    const int r2 = ref_apply<VEC>(pat, n_nodes, op, x, ax, s);
    if (r2) return r2;
    refine_residual_kernel<<<vec_grid(n), VTHREADS, 0, s>>>(n, b, x, ax, bc, r, C, w.partials, scale);
    note_launches(1);
    return check_launch("refine_residual");
  };
  rc = true_residual();
  if (rc) return rc;
  rc = poll(C, s, &h);
  if (rc) return rc;
  int64_t n_updates = 0;
  int final_status = FEM_SOLVE_CONVERGED;
  double best_rr = h.rr_true;   // stagnation: three updates in a row without progress (stall_factor)
  int stalls = 0;
  const double delta2 = delta * delta;
  if (!(h.rr_true <= h.thresh2)) {
    // first start: z = M r, p = z
    FEM_CUDA(cudaMemcpyAsync(&C->delta2, &delta2, sizeof(double), cudaMemcpyHostToDevice, s));
    FEM_CUDA(cudaMemcpyAsync(&C->check2, &check2, sizeof(double), cudaMemcpyHostToDevice, s));
    pcgr_start_kernel<VEC, PC><<<vec_grid(n_nodes), VTHREADS, 0, s>>>(n_nodes, r, z, p, x32, pc, 1, C, w.partials);
    note_launches(1);
    int64_t launched = 0;
    while (true) {
      rc = poll(C, s, &h);
      if (rc) return rc;
      if (h.done) {
        if (h.status == SOLVE_UPDATE) {
          // residual replacement: x += x32 in FP64, r = b - A x in FP64
          accumulate_kernel<<<vec_grid(n), VTHREADS, 0, s>>>(x, x32, n, inv_scale);
          note_launches(1);
          rc = true_residual();
          if (rc) return rc;
          rc = poll(C, s, &h);
          if (rc) return rc;
          ++n_updates;
          if (h.rr_true <= h.thresh2) { final_status = FEM_SOLVE_CONVERGED; break; }
          if (!std::isfinite(h.rr_true)) { final_status = FEM_SOLVE_NAN; break; }
          if (h.iter >= maxiter) { final_status = FEM_SOLVE_MAXITER; break; }
          if (h.rr_true < stall_factor(delta) * best_rr) { best_rr = h.rr_true; stalls = 0; }
          else if (++stalls >= 3) { final_status = FEM_SOLVE_STAGNATED; break; }
          pcgr_start_kernel<VEC, PC><<<vec_grid(n_nodes), VTHREADS, 0, s>>>(n_nodes, r, z, p, x32, pc, 0, C,
                                                                           w.partials);
          pcg_direction_kernel<float><<<vec_grid(n), VTHREADS, 0, s>>>(n, p, z, C);
          note_launches(2);
          continue;
        }
        if (h.status == FEM_SOLVE_MAXITER) {
          accumulate_kernel<<<vec_grid(n), VTHREADS, 0, s>>>(x, x32, n, inv_scale);
          note_launches(1);
          rc = true_residual();
          if (rc) return rc;
          rc = poll(C, s, &h);
          if (rc) return rc;
          final_status = h.rr_true <= h.thresh2 ? FEM_SOLVE_CONVERGED : FEM_SOLVE_MAXITER;
          break;
        }
        final_status = h.status;  // NaN or breakdown
        break;
      }
      if (launched >= maxiter) { final_status = FEM_SOLVE_MAXITER; break; }
      for (int k = 0; k < CHUNK && launched < maxiter; ++k, ++launched) {
        launch_spmv<VEC, float>(pat, n_nodes, vals, p, q, p, C, FIN_PCG_ALPHA, w.partials, 1, s, mfmt);
        pcg_update_kernel<VEC, float, PC><<<vec_grid(n_nodes), VTHREADS, 0, s>>>(n_nodes, x32, r, z, p, q, pc, C,
                                                                                w.partials, FIN_PCGR_UPDATE);
        pcg_direction_kernel<float><<<vec_grid(n), VTHREADS, 0, s>>>(n, p, z, C);
        note_launches(2);
      }
      rc = check_launch("pcg_refined iteration");
      if (rc) return rc;
    }
  }
  if (iters) *iters = h.iter;
  if (updates) *updates = n_updates;
  if (rnorm) *rnorm = std::sqrt(h.rr_true);
  if (status) *status = final_status;
  return FEM_OK;
}

// Byte offset of the int16 corrections inside a DF48 value buffer.
static inline size_t df_lo_offset(int64_t nnz) { return al(sizeof(float) * (size_t)nnz); }

// Number of stored values of a matrix in `mfmt` (sliced layouts include their padding).
static inline int64_t n_values(const fem_pattern_t* pat, int vec, int mfmt) {
  if (mfmt == FEM_SYM_DF48) return pat->n_slots_u * vec * vec * 32;
  if (mfmt == FEM_SSYM_DF48) return ((pat->grid_nx * pat->grid_ny + 31) / 32) * pat->grid_nz * SS_SLOTS * 9 * 32;
  if (mfmt >= FEM_SLICED_F32) return pat->n_slots * vec * vec * 32;
  return pat->nnzb * vec * vec;
}

// DF48 PCG with FP64 reliable updates: FP64 CG vectors and dots, the matrix stream in the
// 6-byte double-float format (SpMV on FP32 pipes, FP64-level accuracy), FP32 block-Jacobi.
// The FP64 true residual (matrix-free tangent action) replaces the recursive residual
// whenever it has fallen by `delta`, and is the only convergence test.
// Double-float CG on the sliced DF48 matrix with FP64 reliable updates.  x, r, p, q live
// as float pairs (FP32 pipes only); the FP64 true residual b - K x (matrix-free tangent
// action) replaces r whenever the recursive residual has fallen by `delta`, and is the
// only convergence test.  x (FP64, caller's buffer) is read at start and written back.
// MODE: DFX_SLICED (FEM_SLICED_DF48), DFX_SYM (FEM_SYM_DF48), DFX_SSYM (FEM_SSYM_DF48).  The two
// symmetric storages leave part of A p in the FP64 vector qT, which the update kernel folds in.
enum { DFX_SLICED = 0, DFX_SYM = 1, DFX_SSYM = 2 };
template <int VEC, int PC, int MODE = DFX_SLICED>
static int pcg_dfx_impl(const fem_pattern_t* pat, int64_t n_nodes, const void* vals, const float* pc, const RefOp& op,
                        const double* b, double* x, double rtol, double atol, double delta, int64_t maxiter,
                        void* ws, int64_t* iters, int64_t* updates, double* rnorm, int32_t* status, cudaStream_t s) {
  constexpr bool SYM = MODE != DFX_SLICED;
  const uint8_t* bc = op.bc;
  const int64_t n = n_nodes * VEC;
  const int64_t m = n_values(pat, VEC, MODE == DFX_SSYM ? FEM_SSYM_DF48 : MODE == DFX_SYM ? FEM_SYM_DF48
                                                                                          : FEM_SLICED_DF48);
  const float* vhi = static_cast<const float*>(vals);
  const int16_t* vlo = reinterpret_cast<const int16_t*>(static_cast<const char*>(vals) + df_lo_offset(m));
  KWs w = carve(ws, n, FEM_F64);
  const size_t f4 = al(sizeof(float) * (size_t)n), d8 = al(sizeof(double) * (size_t)n);
  char* v = w.vecs;
  float* xh = reinterpret_cast<float*>(v); v += f4;
  float* xl = reinterpret_cast<float*>(v); v += f4;
  float* rh = reinterpret_cast<float*>(v); v += f4;
  float* rl = reinterpret_cast<float*>(v); v += f4;
  float* z = reinterpret_cast<float*>(v); v += f4;
  float2* pp = reinterpret_cast<float2*>(v); v += al(sizeof(float2) * DfNode<VEC>::PAD * (size_t)n_nodes);
  float* qh = reinterpret_cast<float*>(v); v += f4;
  float* ql = reinterpret_cast<float*>(v); v += f4;
  double* ax = reinterpret_cast<double*>(v); v += d8;
  double* r64 = reinterpret_cast<double*>(v); v += d8;
  double* qT = SYM ? reinterpret_cast<double*>(v) : nullptr;   // transposed part of the SYM SpMV
  if (SYM) FEM_CUDA(cudaMemsetAsync(qT, 0, sizeof(double) * (size_t)(VEC * qt_stride(n_nodes)), s));
  KCtl* C = w.ctl;
  const int gv = vec_grid(n), gn = vec_grid(n_nodes);
  // Block-Jacobi in the sliced mode: the kernels stream the upper triangles of the symmetric
  // inverse blocks (6 of 9 floats per node, 12 B per node less per iteration), copied once here
  // into the workspace the sliced mode leaves free; the symmetric modes keep the full blocks.
  constexpr int PCK = (PC == FEM_PC_BJACOBI && VEC == 3 && !SYM) ? PC_BSYM : PC;
  const float* pck = pc;
  if constexpr (PCK == PC_BSYM) {
    float* p6 = reinterpret_cast<float*>(v);
    v += al(sizeof(float) * 6 * (size_t)n_nodes);
    bsym_compact_kernel<<<gn, VTHREADS, 0, s>>>(n_nodes, pc, p6);
    note_launches(1);
    pck = p6;
  }
  // tile kernel: one warp per 32-node tile, grid = resident CTAs (no partial second wave)
  static int tile_per_sm = 0;
  if (tile_per_sm == 0 &&
      (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&tile_per_sm, pcgx_update_tile_kernel<PCK, SYM>, VTHREADS, 0) !=
           cudaSuccess ||
       tile_per_sm < 1))
    tile_per_sm = 1;
  int gt = (int)std::min<int64_t>((int64_t)sm_count() * tile_per_sm, ((n_nodes + 31) / 32 + VTILE_WARPS - 1) / VTILE_WARPS);
  if (gt > MAX_PARTIAL_BLOCKS) gt = MAX_PARTIAL_BLOCKS;
  if (gt < 1) gt = 1;
  init_ctl_kernel<<<1, 32, 0, s>>>(C, rtol * rtol, atol * atol, (long long)maxiter);
  dot_kernel<double><<<gv, VTHREADS, 0, s>>>(n, b, b, C, w.partials, nullptr, FIN_REF_BB);
  note_launches(2);
  int rc = check_launch("pcg_dfx init");
  if (rc) return rc;
  // FP64 true residual at the FP64 iterate held in x, and ||r||^2
  auto true_residual = [&]() -> int {
    const int r2 = ref_apply<VEC>(pat, n_nodes, op, x, ax, s);
    if (r2) return r2;
    refine_residual64_kernel<<<gv, VTHREADS, 0, s>>>(n, b, x, ax, bc, r64, C, w.partials);
    note_launches(1);
    return check_launch("refine_residual (df)");
  };
  rc = true_residual();
  if (rc) return rc;
  KCtl h;
  rc = poll(C, s, &h);
  if (rc) return rc;
  // The double-float vectors carry x and r times a power of two that brings the initial residual's
  // RMS near 1, so that r, z, p, q and their dot products stay inside FP32's range (products near
  // 1e-38 would lose precision in subnormals, above 3e38 overflow) however the problem is scaled.
  // Every step of the iteration commutes exactly with a power-of-two scale.
  double scale = 1.0;
  if (h.rr_true > 0.0 && std::isfinite(h.rr_true)) {
    const int e = std::ilogb(std::sqrt(h.rr_true / (double)n));
    scale = std::ldexp(1.0, -std::max(-900, std::min(900, e)));
  }
  const double inv_scale = 1.0 / scale;
  FEM_CUDA(cudaMemsetAsync(xh, 0, sizeof(float) * (size_t)n, s));   // the correction since the last update
  FEM_CUDA(cudaMemsetAsync(xl, 0, sizeof(float) * (size_t)n, s));
  f64_to_df_kernel<<<gv, VTHREADS, 0, s>>>(n, r64, rh, rl, scale);
  note_launches(1);
  int64_t n_updates = 0;
  int final_status = FEM_SOLVE_CONVERGED;
  double best_rr = h.rr_true;   // stagnation: three updates in a row without progress (stall_factor)
  int stalls = 0;
  const double delta2 = delta * delta;
  const double check2 = h.check2 * scale * scale;   // the pause test runs on the scaled recursive residual
  if (!(h.rr_true <= h.thresh2)) {
    FEM_CUDA(cudaMemcpyAsync(&C->delta2, &delta2, sizeof(double), cudaMemcpyHostToDevice, s));
    FEM_CUDA(cudaMemcpyAsync(&C->check2, &check2, sizeof(double), cudaMemcpyHostToDevice, s));
    pcgx_start_kernel<VEC, PCK><<<gn, VTHREADS, 0, s>>>(n_nodes, rh, rl, z, pp, pck, 1, C, w.partials);
    note_launches(1);
    int64_t launched = 0;
    // k_count iterations (SpMV, update, direction) on stream st; the timed pair brackets the second
    // SpMV (the first follows the host poll on an idle GPU, so its bracket would hold the launch
    // latency too)
    auto run_iters = [&](cudaStream_t st, int k_count, bool captured) -> int {
      for (int k = 0; k < k_count; ++k) {
        if (k == 1) { if (captured) spmv_timer_mark_graph(0, st); else spmv_timer_mark(0, st); }
        int r2;
        if constexpr (MODE == DFX_SSYM)
          r2 = launch_ssym(pat, vhi, vlo, pp, qh, ql, qT, C, FIN_PCG_ALPHA, w.partials, st);
        else
          r2 = launch_dfdf<VEC, SYM>(pat, n_nodes, vhi, vlo, pp, qh, ql, C, FIN_PCG_ALPHA, w.partials, st, qT);
        if (r2) return r2;
        if (k == 1) { if (captured) spmv_timer_mark_graph(1, st); else spmv_timer_mark(1, st); }
        if constexpr (VEC == 3) {
          if (!launch_update_bulk<PCK, SYM>(n_nodes, xh, xl, rh, rl, z, pp, qh, ql, pck, C, w.partials,
                                            FIN_PCGR_UPDATE, st, qT))
            pcgx_update_tile_kernel<PCK, SYM><<<gt, VTHREADS, 0, st>>>(n_nodes, xh, xl, rh, rl, z, pp, qh, ql, pck,
                                                                       C, w.partials, FIN_PCGR_UPDATE, qT);
          pcgx_direction3_kernel<<<gv, VTHREADS, 0, st>>>(n, z, pp, C);
        } else {
          pcgx_update_kernel<VEC, PC><<<gn, VTHREADS, 0, st>>>(n_nodes, xh, xl, rh, rl, z, pp, qh, ql, pc, C,
                                                              w.partials, FIN_PCGR_UPDATE);
          pcgx_direction_kernel<VEC><<<gn, VTHREADS, 0, st>>>(n_nodes, z, pp, C);
        }
        note_launches(2);
      }
      return FEM_OK;
    };
    ChunkGraph graph;
    while (true) {
      rc = poll(C, s, &h);
      if (rc) return rc;
      if (h.done) {
        if (h.status == SOLVE_UPDATE || h.status == FEM_SOLVE_MAXITER) {
          const bool at_max = h.status == FEM_SOLVE_MAXITER;
          df_accumulate_kernel<<<gv, VTHREADS, 0, s>>>(n, xh, xl, x, inv_scale);
          note_launches(1);
          rc = true_residual();
          if (rc) return rc;
          f64_to_df_kernel<<<gv, VTHREADS, 0, s>>>(n, r64, rh, rl, scale);
          note_launches(1);
          rc = poll(C, s, &h);
          if (rc) return rc;
          ++n_updates;
          if (h.rr_true <= h.thresh2) { final_status = FEM_SOLVE_CONVERGED; break; }
          if (!std::isfinite(h.rr_true)) { final_status = FEM_SOLVE_NAN; break; }
          if (at_max || h.iter >= maxiter) { final_status = FEM_SOLVE_MAXITER; break; }
          if (h.rr_true < stall_factor(delta) * best_rr) { best_rr = h.rr_true; stalls = 0; }
          else if (++stalls >= 3) { final_status = FEM_SOLVE_STAGNATED; break; }
          pcgx_start_kernel<VEC, PCK><<<gn, VTHREADS, 0, s>>>(n_nodes, rh, rl, z, pp, pck, 0, C, w.partials);
          pcgx_direction_kernel<VEC><<<gn, VTHREADS, 0, s>>>(n_nodes, z, pp, C);
          note_launches(2);
          continue;
        }
        final_status = h.status;  // NaN or breakdown
        df_accumulate_kernel<<<gv, VTHREADS, 0, s>>>(n, xh, xl, x, inv_scale);
        note_launches(1);
        break;
      }
      if (launched >= maxiter) {
        final_status = FEM_SOLVE_MAXITER;
        df_accumulate_kernel<<<gv, VTHREADS, 0, s>>>(n, xh, xl, x, inv_scale);
        note_launches(1);
        break;
      }
      rc = graph.step(s, launched, maxiter, run_iters);
      if (rc) return rc;
      rc = check_launch("pcg_dfx iteration");
      if (rc) return rc;
    }
  }
  if (iters) *iters = h.iter;
  if (updates) *updates = n_updates;
  if (rnorm) *rnorm = std::sqrt(h.rr_true);
  if (status) *status = final_status;
  return FEM_OK;
}

template <int VEC, int PC>
static int pcg_df_impl(const fem_pattern_t* pat, int64_t n_nodes, const void* vals, const float* pc, const RefOp& op,
                       const double* b, double* x, double rtol, double atol, double delta, int64_t maxiter, void* ws,
                       int64_t* iters, int64_t* updates, double* rnorm, int32_t* status, cudaStream_t s, int mfmt) {
  const uint8_t* bc = op.bc;
  const int64_t n = n_nodes * VEC;
  const int64_t nnz = pat->nnzb * VEC * VEC;
  const float* vhi = static_cast<const float*>(vals);
  const int64_t m = mfmt == FEM_SLICED_DF48 ? n_values(pat, VEC, mfmt) : nnz;
  const int16_t* vlo = reinterpret_cast<const int16_t*>(static_cast<const char*>(vals) + df_lo_offset(m));
  KWs w = carve(ws, n, FEM_F64);
  const size_t d8 = al(sizeof(double) * (size_t)n), f4 = al(sizeof(float) * (size_t)n);
  double* r = reinterpret_cast<double*>(w.vecs);
  double* z = reinterpret_cast<double*>(w.vecs + d8);
  double* p = reinterpret_cast<double*>(w.vecs + 2 * d8);
  double* q = reinterpret_cast<double*>(w.vecs + 3 * d8);
  double* ax = reinterpret_cast<double*>(w.vecs + 4 * d8);
  float* phi = reinterpret_cast<float*>(w.vecs + 5 * d8);
  float* plo = reinterpret_cast<float*>(w.vecs + 5 * d8 + f4);
  KCtl* C = w.ctl;
  init_ctl_kernel<<<1, 32, 0, s>>>(C, rtol * rtol, atol * atol, (long long)maxiter);
  dot_kernel<double><<<vec_grid(n), VTHREADS, 0, s>>>(n, b, b, C, w.partials, nullptr, FIN_REF_BB);
  note_launches(2);
  int rc = check_launch("pcg_df init");
  if (rc) return rc;
  auto true_residual = [&]() -> int {
    const int r2 = ref_apply<VEC>(pat, n_nodes, op, x, ax, s);
    if (r2) return r2;
    refine_residual64_kernel<<<vec_grid(n), VTHREADS, 0, s>>>(n, b, x, ax, bc, r, C, w.partials);
    note_launches(1);
    return check_launch("refine_residual64");
  };
  rc = true_residual();
  if (rc) return rc;
  KCtl h;
  rc = poll(C, s, &h);
  if (rc) return rc;
  int64_t n_updates = 0;
  int final_status = FEM_SOLVE_CONVERGED;
  double best_rr = h.rr_true;   // stagnation: three updates in a row without progress (stall_factor)
  int stalls = 0;
  const double delta2 = delta * delta;
  if (!(h.rr_true <= h.thresh2)) {
    FEM_CUDA(cudaMemcpyAsync(&C->delta2, &delta2, sizeof(double), cudaMemcpyHostToDevice, s));
    pcgd_start_kernel<VEC, PC><<<vec_grid(n_nodes), VTHREADS, 0, s>>>(n_nodes, r, z, p, phi, plo, pc, 1, C,
                                                                     w.partials);
    note_launches(1);
    int64_t launched = 0;
    while (true) {
      rc = poll(C, s, &h);
      if (rc) return rc;
      if (h.done) {
        if (h.status == SOLVE_UPDATE || h.status == FEM_SOLVE_MAXITER) {
          const bool at_max = h.status == FEM_SOLVE_MAXITER;
          rc = true_residual();
          if (rc) return rc;
          rc = poll(C, s, &h);
          if (rc) return rc;
          ++n_updates;
          if (h.rr_true <= h.thresh2) { final_status = FEM_SOLVE_CONVERGED; break; }
          if (!std::isfinite(h.rr_true)) { final_status = FEM_SOLVE_NAN; break; }
          if (at_max || h.iter >= maxiter) { final_status = FEM_SOLVE_MAXITER; break; }
          if (h.rr_true < stall_factor(delta) * best_rr) { best_rr = h.rr_true; stalls = 0; }
          else if (++stalls >= 3) { final_status = FEM_SOLVE_STAGNATED; break; }
          pcgd_start_kernel<VEC, PC><<<vec_grid(n_nodes), VTHREADS, 0, s>>>(n_nodes, r, z, p, phi, plo, pc, 0, C,
                                                                           w.partials);
          pcgd_direction_kernel<<<vec_grid(n), VTHREADS, 0, s>>>(n, p, z, phi, plo, C);
          note_launches(2);
          continue;
        }
        final_status = h.status;  // NaN or breakdown
        break;
      }
      if (launched >= maxiter) { final_status = FEM_SOLVE_MAXITER; break; }
      for (int k = 0; k < CHUNK && launched < maxiter; ++k, ++launched) {
        launch_spmv_any<VEC, FMT_DF>(pat, n_nodes, mfmt, vhi, vlo, phi, plo, q, p, C, FIN_PCG_ALPHA, w.partials, 1,
                                     s);
        pcgd_update_kernel<VEC, PC><<<vec_grid(n_nodes), VTHREADS, 0, s>>>(n_nodes, x, r, z, p, q, pc, C, w.partials,
                                                                          FIN_PCGR_UPDATE);
        pcgd_direction_kernel<<<vec_grid(n), VTHREADS, 0, s>>>(n, p, z, phi, plo, C);
        note_launches(2);
      }
      rc = check_launch("pcg_df iteration");
      if (rc) return rc;
    }
  }
  if (iters) *iters = h.iter;
  if (updates) *updates = n_updates;
  if (rnorm) *rnorm = std::sqrt(h.rr_true);
  if (status) *status = final_status;
  return FEM_OK;
}

}  // namespace fem

using namespace fem;


static int check_pat(const fem_pattern_t* pat, int64_t n_nodes, int32_t vec, int32_t precision) {
  FEM_REQUIRE(pat && pat->block_ptr && pat->block_cols, "pattern NULL");
  FEM_REQUIRE(n_nodes > 0, "n_nodes must be positive");
  FEM_REQUIRE(vec == 1 || vec == 3, "vec must be 1 or 3");
  FEM_REQUIRE(precision >= FEM_F32 && precision <= FEM_SSYM_DF48, "bad precision");
  FEM_REQUIRE(precision != FEM_SSYM_DF48 ||
                  (vec == 3 && pat->grid_nx > 0 && pat->grid_ny > 0 && pat->grid_nz > 0 &&
                   pat->grid_nx * pat->grid_ny * pat->grid_nz == n_nodes),
              "FEM_SSYM_DF48 needs vec 3 and the pattern's node grid (grid_nx*grid_ny*grid_nz == n_nodes)");
  FEM_REQUIRE(!is_sliced(precision) || (pat->n_slices == (n_nodes + 31) / 32 && pat->slice_ptr && pat->slice_cols),
              "sliced format needs the pattern's slice arrays (fem_pattern_slices)");
  FEM_REQUIRE(!pat->slices_grid || (pat->grid_nx > 0 && pat->grid_ny > 0 && pat->grid_nz > 0 &&
                                    pat->grid_nx * pat->grid_ny * pat->grid_nz == n_nodes &&
                                    pat->n_slots == 27 * pat->n_slices),
              "slices_grid needs the node grid and the 27-slot layout of fem_pattern_slices_grid");
  FEM_REQUIRE(precision != FEM_SYM_DF48 || (pat->slice_ptr_u && pat->slice_cols_u && pat->n_slots_u > 0),
              "FEM_SYM_DF48 needs the upper-block slice arrays (fem_pattern_slices_upper)");
  return FEM_OK;
}

extern "C" int fem_spmv(const fem_pattern_t* pat, int64_t n_nodes, int32_t vec, int32_t precision, const void* vals,
                        const void* x, void* y, void* stream) {
  int rc = check_pat(pat, n_nodes, vec, precision);
  if (rc) return rc;
  FEM_REQUIRE(precision != FEM_SYM_DF48 && precision != FEM_SSYM_DF48,
              "FEM_SYM_DF48 / FEM_SSYM_DF48 matrices are applied by fem_spmv_dfx");
  FEM_REQUIRE(vals && x && y, "NULL vector");
  cudaStream_t s = as_stream(stream);
  if (is_df(precision)) {
    const int64_t n = n_nodes * vec;
    const float* hi = (const float*)vals;
    const int16_t* lo =
        reinterpret_cast<const int16_t*>((const char*)vals + df_lo_offset(n_values(pat, vec, precision)));
    const float* xh = (const float*)x;
    const float* xl = xh + n;
    if (vec == 3) launch_spmv_any<3, FMT_DF>(pat, n_nodes, precision, hi, lo, xh, xl, y, nullptr, nullptr, 0, nullptr, 0, s);
    else launch_spmv_any<1, FMT_DF>(pat, n_nodes, precision, hi, lo, xh, xl, y, nullptr, nullptr, 0, nullptr, 0, s);
    return check_launch("spmv_df");
  }
  if (vec_f32(precision)) {
    if (vec == 3) launch_spmv<3, float>(pat, n_nodes, (const float*)vals, (const float*)x, (float*)y, nullptr, nullptr, 0, nullptr, 0, s, precision);
    else launch_spmv<1, float>(pat, n_nodes, (const float*)vals, (const float*)x, (float*)y, nullptr, nullptr, 0, nullptr, 0, s, precision);
  } else {
    if (vec == 3) launch_spmv<3, double>(pat, n_nodes, (const double*)vals, (const double*)x, (double*)y, nullptr, nullptr, 0, nullptr, 0, s, precision);
    else launch_spmv<1, double>(pat, n_nodes, (const double*)vals, (const double*)x, (double*)y, nullptr, nullptr, 0, nullptr, 0, s, precision);
  }
  return check_launch("spmv");
}

extern "C" int fem_zero_rows(const fem_pattern_t* pat, int32_t vec, int32_t precision, void* vals, const int32_t* rows,
                             int64_t n_rows, double diag_value, void* stream) {
  FEM_REQUIRE(pat && pat->block_ptr && pat->indptr && pat->diag && vals, "pattern/vals NULL");
  FEM_REQUIRE(precision == FEM_F32 || precision == FEM_F64, "fem_zero_rows works on CSR-order FP32/FP64 values");
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

extern "C" int fem_matrix_transpose(const fem_pattern_t* pat, int64_t n_nodes, int32_t vec, int32_t precision,
                                    const void* vals, void* vals_t, void* ws, size_t ws_bytes, void* stream) {
  FEM_REQUIRE(pat && pat->block_ptr && pat->block_cols && vals && vals_t, "pattern/vals NULL");
  FEM_REQUIRE(vals != vals_t, "fem_matrix_transpose works out of place");
  FEM_REQUIRE(precision == FEM_F32 || precision == FEM_F64, "fem_matrix_transpose works on CSR-order FP32/FP64 values");
  FEM_REQUIRE(vec == 1 || vec == 3, "vec must be 1 or 3");
  FEM_REQUIRE(n_nodes >= 0, "n_nodes < 0");
  FEM_REQUIRE(ws && ws_bytes >= sizeof(int), "workspace of at least 4 bytes required (error flag)");
  if (n_nodes == 0) return FEM_OK;
  cudaStream_t s = as_stream(stream);
  int* err = static_cast<int*>(ws);
  FEM_CUDA(cudaMemsetAsync(err, 0, sizeof(int), s));
  if (precision == FEM_F32)
    transpose_kernel<float><<<grid_for(n_nodes, 128), 128, 0, s>>>(vec, n_nodes, pat->block_ptr, pat->block_cols,
                                                                   (const float*)vals, (float*)vals_t, err);
  else
    transpose_kernel<double><<<grid_for(n_nodes, 128), 128, 0, s>>>(vec, n_nodes, pat->block_ptr, pat->block_cols,
                                                                    (const double*)vals, (double*)vals_t, err);
  note_launches(1);
  int rc = check_launch("matrix_transpose");
  if (rc) return rc;
  int h = 0;
  FEM_CUDA(cudaMemcpyAsync(&h, err, sizeof(int), cudaMemcpyDeviceToHost, s));
  FEM_CUDA(cudaStreamSynchronize(s));
  if (h) return fail(FEM_ERR_ARG, "fem_matrix_transpose: the block pattern is not structurally symmetric");
  return FEM_OK;
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
  FEM_REQUIRE(precision == FEM_F32 || precision == FEM_F64, "preconditioners are set up from CSR FP32/FP64 values");
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
  FEM_REQUIRE(precision >= FEM_F32 && precision <= FEM_SSYM_DF48, "bad precision");
  *bytes = krylov_ws_bytes(n_dofs, vec_f32(precision) ? FEM_F32 : FEM_F64);
  return FEM_OK;
}

template <typename T>
static int solve_dispatch(bool bicg, const fem_pattern_t* pat, int64_t n_nodes, int vec, const void* vals, int pc_kind,
                          const void* pc, const void* b, void* x, double rtol, double atol, int64_t maxiter, void* ws,
                          int64_t* it, double* rn, int32_t* st, cudaStream_t s, int mfmt, bool graphs = true) {
  const T* V = (const T*)vals;
  const T* P = (const T*)pc;
  const T* B = (const T*)b;
  T* X = (T*)x;
#define FEM_SOLVE_CASE(VEC, PC)                                                                          \
  if (vec == VEC && pc_kind == PC)                                                                       \
    return bicg ? bicg_impl<VEC, T, PC>(pat, n_nodes, V, P, B, X, rtol, atol, maxiter, ws, it, rn, st, s, mfmt) \
                : pcg_impl<VEC, T, PC>(pat, n_nodes, V, P, B, X, rtol, atol, maxiter, ws, it, rn, st, s, mfmt, graphs);
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
  FEM_REQUIRE(!is_df(precision), "use fem_pcg_refined for DF48 matrices");
  FEM_REQUIRE(ws_bytes >= krylov_ws_bytes(n_nodes * vec, vec_f32(precision) ? FEM_F32 : FEM_F64),
              "krylov workspace too small");
  cudaStream_t s = as_stream(stream);
  if (vec_f32(precision))
    return solve_dispatch<float>(bicg, pat, n_nodes, vec, vals, pc_kind, pc, b, x, rtol, atol, maxiter, ws, iterations,
                                 res_norm, status, s, precision);
  return solve_dispatch<double>(bicg, pat, n_nodes, vec, vals, pc_kind, pc, b, x, rtol, atol, maxiter, ws, iterations,
                                res_norm, status, s, precision);
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

extern "C" int fem_spmv_timing_start(void) {
  g_spmv_timer.on = true;
  g_spmv_timer.used = 0;
  g_spmv_timer.seconds = 0.0;
  g_spmv_timer.samples = 0;
  return FEM_OK;
}

extern "C" int fem_spmv_timing_stop(double* seconds, int64_t* samples) {
  FEM_REQUIRE(seconds && samples, "NULL argument");
  if (g_spmv_timer.used) {
    FEM_CUDA(cudaDeviceSynchronize());
    spmv_timer_collect();
  }
  g_spmv_timer.on = false;
  *seconds = g_spmv_timer.seconds;
  *samples = g_spmv_timer.samples;
  return FEM_OK;
}

extern "C" int fem_selftest_bounded_wait(void* ws, size_t ws_bytes, void* stream) {
  FEM_REQUIRE(ws, "NULL argument");
  FEM_REQUIRE(ws_bytes >= al(sizeof(KCtl)) + al(sizeof(double) * 3 * MAX_PARTIAL_BLOCKS), "workspace too small");
  cudaStream_t s = as_stream(stream);
  KWs w = carve(ws, 0, FEM_F64);
  init_ctl_kernel<<<1, 32, 0, s>>>(w.ctl, 0.0, 0.0, 0);
  bounded_wait_selftest_kernel<<<1, 32, 0, s>>>(w.ctl);
  note_launches(2);
  const int rc = check_launch("bounded-wait self-test");
  if (rc) return rc;
  KCtl h;
  return poll(w.ctl, s, &h);   // FEM_ERR_DEVICE when the wait ran out, as designed
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

extern "C" int fem_pcg_refined(const fem_pattern_t* pat, int64_t n_nodes, int32_t vec, int32_t precision,
                               const void* vals32, int32_t pc_kind, const void* pc32, const fem_mesh_t* mesh,
                               const fem_material_t* mat, const double* u_lin, const void* vals_ref,
                               int32_t ref_precision, const uint8_t* bc_mask,
                               const double* b, double* x, double rtol, double atol, double delta, int64_t maxiter,
                               void* ws, size_t ws_bytes, int64_t* iterations, int64_t* updates, double* res_norm,
                               int32_t* status, void* stream) {
  FEM_REQUIRE(precision == FEM_F32 || precision == FEM_SLICED_F32 || is_df(precision),
              "precision must be FEM_F32, FEM_DF48 or a sliced variant");
  int rc = check_pat(pat, n_nodes, vec, precision);
  if (rc) return rc;
  FEM_REQUIRE(vals32 && b && x && ws, "NULL argument");
  FEM_REQUIRE(vals_ref || (mesh && mat), "need an FP64 reference matrix or mesh + material");
  FEM_REQUIRE(!vals_ref || ref_precision == FEM_F64 || ref_precision == FEM_SLICED_F64,
              "reference matrix must be FEM_F64 or FEM_SLICED_F64");
  FEM_REQUIRE(vals_ref || (mesh->n_nodes == n_nodes && mesh->vec == vec), "mesh does not match the pattern");
  const RefOp op{mesh, mat, u_lin, vals_ref, ref_precision, bc_mask};
  FEM_REQUIRE(pc_kind == FEM_PC_NONE || pc32, "preconditioner data NULL");
  FEM_REQUIRE(pc_kind >= FEM_PC_NONE && pc_kind <= FEM_PC_BJACOBI, "bad pc_kind");
  FEM_REQUIRE(rtol >= 0 && atol >= 0 && maxiter >= 0 && delta > 0 && delta < 1, "bad tolerances");
  FEM_REQUIRE(ws_bytes >= krylov_ws_bytes(n_nodes * vec, FEM_F64), "workspace too small (fem_krylov_workspace FP64)");
  cudaStream_t s = as_stream(stream);
  const float* V = (const float*)vals32;
  const float* P = (const float*)pc32;
#define FEM_REF_CASE(VEC, PC)                                                                                   \
  if (vec == VEC && pc_kind == PC)                                                                              \
    return precision == FEM_SSYM_DF48                                                                           \
               ? pcg_dfx_impl<VEC, PC, DFX_SSYM>(pat, n_nodes, vals32, P, op, b, x, rtol, atol, delta, maxiter, \
                                                 ws, iterations, updates, res_norm, status, s)                 \
           : precision == FEM_SYM_DF48                                                                          \
               ? pcg_dfx_impl<VEC, PC, DFX_SYM>(pat, n_nodes, vals32, P, op, b, x, rtol, atol, delta, maxiter,  \
                                                ws, iterations, updates, res_norm, status, s)                  \
           : precision == FEM_SLICED_DF48                                                                       \
               ? pcg_dfx_impl<VEC, PC>(pat, n_nodes, vals32, P, op, b, x, rtol, atol, delta, maxiter, ws,       \
                                       iterations, updates, res_norm, status, s)                               \
           : is_df(precision)                                                                                   \
               ? pcg_df_impl<VEC, PC>(pat, n_nodes, vals32, P, op, b, x, rtol, atol, delta, maxiter, ws,        \
                                      iterations, updates, res_norm, status, s, precision)                     \
               : pcg_refined_impl<VEC, PC>(pat, n_nodes, V, P, op, b, x, rtol, atol, delta, maxiter, ws,        \
                                           iterations, updates, res_norm, status, s, precision);
  FEM_REF_CASE(3, FEM_PC_NONE)
  FEM_REF_CASE(3, FEM_PC_JACOBI)
  FEM_REF_CASE(3, FEM_PC_BJACOBI)
  FEM_REF_CASE(1, FEM_PC_NONE)
  FEM_REF_CASE(1, FEM_PC_JACOBI)
  FEM_REF_CASE(1, FEM_PC_BJACOBI)
#undef FEM_REF_CASE
  return fail(FEM_ERR_ARG, "bad vec / preconditioner");
}

extern "C" int fem_matrix_bytes(const fem_pattern_t* pat, int32_t vec, int32_t precision, size_t* bytes) {
  FEM_REQUIRE(pat && bytes && (vec == 1 || vec == 3), "bad arguments");
  FEM_REQUIRE(precision >= FEM_F32 && precision <= FEM_SSYM_DF48, "bad precision");
  FEM_REQUIRE(!is_sliced(precision) || pat->n_slices > 0, "sliced format needs fem_pattern_slices first");
  FEM_REQUIRE(precision != FEM_SYM_DF48 || pat->n_slots_u > 0, "FEM_SYM_DF48 needs fem_pattern_slices_upper first");
  FEM_REQUIRE(precision != FEM_SSYM_DF48 || (vec == 3 && pat->grid_nx > 0 && pat->grid_ny > 0 && pat->grid_nz > 0),
              "FEM_SSYM_DF48 needs vec 3 and the pattern's node grid");
  const int64_t m = n_values(pat, vec, precision);
  if (precision == FEM_SSYM_DF48) *bytes = al(df_lo_offset(m) + sizeof(int16_t) * (size_t)m) + 256;
  else if (is_df(precision)) *bytes = df_lo_offset(m) + sizeof(int16_t) * (size_t)m;
  else if (vec_f32(precision)) *bytes = sizeof(float) * (size_t)m;
  else *bytes = sizeof(double) * (size_t)m;
  return FEM_OK;
}

extern "C" int fem_matrix_convert(const fem_pattern_t* pat, int64_t n_nodes, int32_t vec, const double* vals64,
                                  int32_t precision, void* out, void* stream) {
  int rc = check_pat(pat, n_nodes, vec, precision);
  if (rc) return rc;
  FEM_REQUIRE(vals64 && out, "NULL argument");
  FEM_REQUIRE(precision != FEM_F64, "FP64 CSR values need no conversion");
  cudaStream_t s = as_stream(stream);
  const int64_t nnz = pat->nnzb * vec * vec;
  if (precision == FEM_SSYM_DF48) {
    const int64_t m = n_values(pat, vec, precision);
    int16_t* lo = reinterpret_cast<int16_t*>((char*)out + df_lo_offset(m));
    int* err = reinterpret_cast<int*>((char*)out + al(df_lo_offset(m) + sizeof(int16_t) * (size_t)m));
    FEM_CUDA(cudaMemsetAsync(err, 0, sizeof(int), s));
    const SsGrid G = ss_grid(pat, 1);
    to_ssym_kernel<<<grid_for(G.groups * G.nz * 32, 256), 256, 0, s>>>(G, pat->block_ptr, pat->block_cols, vals64,
                                                                        (float*)out, lo, err);
    note_launches(1);
    int rc2 = check_launch("matrix_convert (ssym)");
    if (rc2) return rc2;
    int h = 0;
    FEM_CUDA(cudaMemcpyAsync(&h, err, sizeof(int), cudaMemcpyDeviceToHost, s));
    FEM_CUDA(cudaStreamSynchronize(s));
    if (h) return fail(FEM_ERR_ARG, "FEM_SSYM_DF48: the node pattern is not the 27-point stencil of the grid");
    return FEM_OK;
  } else if (precision == FEM_SYM_DF48) {
    FEM_REQUIRE(vec == 3, "FEM_SYM_DF48 is built for vec 3");
    const int64_t m = n_values(pat, vec, precision);
    int16_t* lo = reinterpret_cast<int16_t*>((char*)out + df_lo_offset(m));
    to_sliced_upper_kernel<3><<<grid_for(pat->n_slices * 32, 256), 256, 0, s>>>(
        n_nodes, pat->n_slices, pat->block_ptr, pat->block_cols, pat->slice_ptr_u, vals64, (float*)out, lo);
  } else if (precision == FEM_DF48) {
    float* hi = (float*)out;
    int16_t* lo = reinterpret_cast<int16_t*>((char*)out + df_lo_offset(nnz));
    split_df_kernel<<<grid_for(nnz, 256), 256, 0, s>>>(vals64, nnz, hi, lo);
  } else if (precision == FEM_F32) {
    cast_kernel<<<grid_for(nnz, 256), 256, 0, s>>>(vals64, (float*)out, nnz, nullptr);
  } else {
    const int64_t m = n_values(pat, vec, precision);
    int16_t* lo = is_df(precision) ? reinterpret_cast<int16_t*>((char*)out + df_lo_offset(m)) : nullptr;
    const int g = grid_for(pat->n_slices * 32, 256);
    const bool gl = pat->slices_grid != 0;
#define FEM_TO_SLICED(VEC, OUT)                                                                              \
  to_sliced_kernel<VEC, OUT><<<g, 256, 0, s>>>(n_nodes, pat->n_slices, pat->block_ptr, pat->slice_ptr, vals64, \
                                                out, lo, pat->block_cols, gl ? pat->grid_nx : 0, pat->grid_ny, \
                                                pat->grid_nz)
    if (vec == 3) {
      if (precision == FEM_SLICED_F64) FEM_TO_SLICED(3, FEM_SLICED_F64);
      else if (precision == FEM_SLICED_F32) FEM_TO_SLICED(3, FEM_SLICED_F32);
      else FEM_TO_SLICED(3, FEM_SLICED_DF48);
    } else {
      if (precision == FEM_SLICED_F64) FEM_TO_SLICED(1, FEM_SLICED_F64);
      else if (precision == FEM_SLICED_F32) FEM_TO_SLICED(1, FEM_SLICED_F32);
      else FEM_TO_SLICED(1, FEM_SLICED_DF48);
    }
#undef FEM_TO_SLICED
  }
  note_launches(1);
  return check_launch("matrix_convert");
}

extern "C" int fem_vector_split(const double* x, int64_t n, float* x_df, void* stream) {
  FEM_REQUIRE(n >= 0 && (n == 0 || (x && x_df)), "NULL argument");
  if (n == 0) return FEM_OK;
  split_vec_kernel<<<grid_for(n, 256), 256, 0, as_stream(stream)>>>(x, n, x_df, x_df + n);
  note_launches(1);
  return check_launch("split_vec");
}

extern "C" int fem_spmv_dfx(const fem_pattern_t* pat, int64_t n_nodes, int32_t vec, int32_t precision,
                            const void* vals, const void* x_df, float* y_hi, float* y_lo, double* xy_dot, void* ws,
                            size_t ws_bytes, void* stream) {
  FEM_REQUIRE(pat && vals && x_df && y_hi && y_lo && ws, "NULL argument");
  FEM_REQUIRE(precision == FEM_SLICED_DF48 || precision == FEM_SYM_DF48 || precision == FEM_SSYM_DF48,
              "precision must be a sliced or symmetric DF48 type");
  int rc0 = check_pat(pat, n_nodes, vec, precision);
  if (rc0) return rc0;
  FEM_REQUIRE(ws_bytes >= krylov_ws_bytes(n_nodes * vec, FEM_F64), "workspace too small");
  cudaStream_t s = as_stream(stream);
  const int64_t m = n_values(pat, vec, precision);
  const float* vhi = static_cast<const float*>(vals);
  const int16_t* vlo = reinterpret_cast<const int16_t*>(static_cast<const char*>(vals) + df_lo_offset(m));
  KWs w = carve(ws, n_nodes * vec, FEM_F64);
  init_ctl_kernel<<<1, 32, 0, s>>>(w.ctl, 0.0, 0.0, 0);
  note_launches(1);
  const float2* xp = static_cast<const float2*>(x_df);
  int rc;
  if (precision == FEM_SYM_DF48 || precision == FEM_SSYM_DF48) {
    double* qT = reinterpret_cast<double*>(w.vecs);
    FEM_CUDA(cudaMemsetAsync(qT, 0, sizeof(double) * (size_t)(vec * qt_stride(n_nodes)), s));
    if (precision == FEM_SSYM_DF48)
      rc = launch_ssym(pat, vhi, vlo, xp, y_hi, y_lo, qT, w.ctl, FIN_DOT, w.partials, s);
    else
      rc = launch_dfdf<3, true>(pat, n_nodes, vhi, vlo, xp, y_hi, y_lo, w.ctl, FIN_DOT, w.partials, s, qT);
    if (rc) return rc;
    sym_combine_kernel<<<vec_grid(n_nodes * vec), VTHREADS, 0, s>>>(n_nodes, y_hi, y_lo, qT);
    note_launches(1);
  } else if (vec == 3) {
    rc = launch_dfdf<3>(pat, n_nodes, vhi, vlo, xp, y_hi, y_lo, w.ctl, FIN_DOT, w.partials, s);
  } else {
    rc = launch_dfdf<1>(pat, n_nodes, vhi, vlo, xp, y_hi, y_lo, w.ctl, FIN_DOT, w.partials, s);
  }
  if (rc) return rc;
  rc = check_launch("spmv_dfx");
  if (rc) return rc;
  if (xy_dot) FEM_CUDA(cudaMemcpyAsync(xy_dot, &w.ctl->d0, sizeof(double), cudaMemcpyDeviceToDevice, s));
  return FEM_OK;
}

// ---- allocation-free PCG ----------------------------------------------------------
// For callers that cannot allocate device memory themselves -- a host framework whose
// device allocator is closed to plug-ins, or an embedding that reserves device memory up
// front and forbids allocation after start-up -- fem_pcg_static runs the same PCG as
// fem_pcg with its scratch (control block, per-CTA partial sums, four Krylov vectors) in
// this file-scope device array.  Every GPU that loads the library holds the array until
// the process exits; every call shares it, so calls that overlap on the GPU race.  Like
// fem_pcg, it reads the convergence flag back to the host every 16 iterations.
namespace fem {
constexpr int64_t STATIC_PCG_MAX_DOFS = 262144;
constexpr size_t al_c(size_t x) { return (x + 255) & ~size_t(255); }
constexpr size_t STATIC_PCG_BYTES = al_c(sizeof(KCtl)) + al_c(sizeof(double) * 3 * MAX_PARTIAL_BLOCKS) +
                                    4 * al_c(sizeof(double) * STATIC_PCG_MAX_DOFS);
__device__ __align__(256) unsigned char g_static_pcg_scratch[STATIC_PCG_BYTES];

// Device address of the scratch array on the current device, looked up once per device
// (on the first call there).  The host-side
// name g_static_pcg_scratch is only a stand-in for the symbol and is never passed to a
// kernel.  The cached address belongs to the context of that first call; it is not
// looked up again, so it does not survive a cudaDeviceReset of the device.
static int static_pcg_scratch(void** out) {
  static std::mutex mu;
  static void* addr[128] = {};
  int dev = 0;
  FEM_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 128) return fail(FEM_ERR_ARG, "device ordinal out of range");
  std::lock_guard<std::mutex> lk(mu);
  if (addr[dev] == nullptr) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_static_pcg_scratch);
    if (e != cudaSuccess || p == nullptr)
      return fail(FEM_ERR_CUDA, std::string("cudaGetSymbolAddress(g_static_pcg_scratch): ") + cudaGetErrorString(e));
    addr[dev] = p;
  }
  *out = addr[dev];
  return FEM_OK;
}
}  // namespace fem

extern "C" int fem_pcg_static(const fem_pattern_t* pat, int64_t n_nodes, int32_t vec, int32_t precision,
                              const void* vals, int32_t pc_kind, const void* pc, const void* b, void* x,
                              double rtol, double atol, int64_t maxiter, int64_t* iterations, double* res_norm,
                              int32_t* status, void* stream) {
  int rc = check_pat(pat, n_nodes, vec, precision);
  if (rc) return rc;
  if (n_nodes * vec > STATIC_PCG_MAX_DOFS)
    return fail(FEM_ERR_CAPACITY, "fem_pcg_static: " + std::to_string(n_nodes * vec) +
                                      " dofs exceed its fixed scratch limit of " +
                                      std::to_string(STATIC_PCG_MAX_DOFS) +
                                      " dofs; use fem_pcg with a caller workspace");
  FEM_REQUIRE(vals && b && x, "NULL argument");
  FEM_REQUIRE(pc_kind == FEM_PC_NONE || pc, "preconditioner data NULL");
  FEM_REQUIRE(pc_kind >= FEM_PC_NONE && pc_kind <= FEM_PC_BJACOBI, "bad pc_kind");
  FEM_REQUIRE(rtol >= 0 && atol >= 0 && maxiter >= 0, "tolerances / maxiter must be non-negative");
  FEM_REQUIRE(!is_df(precision), "fem_pcg_static takes FP32 / FP64 (CSR or sliced) matrices");
  void* ws = nullptr;
  rc = static_pcg_scratch(&ws);
  if (rc) return rc;
  // the control block (done flag, tickets, scalars) is reset by the solver's first kernel;
  // partial sums and vectors are written before they are read, so nothing else is cleared
  cudaStream_t s = as_stream(stream);
  if (vec_f32(precision))
    return solve_dispatch<float>(false, pat, n_nodes, vec, vals, pc_kind, pc, b, x, rtol, atol, maxiter, ws,
                                 iterations, res_norm, status, s, precision, false);
  return solve_dispatch<double>(false, pat, n_nodes, vec, vals, pc_kind, pc, b, x, rtol, atol, maxiter, ws,
                                iterations, res_norm, status, s, precision, false);
}
