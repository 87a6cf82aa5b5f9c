// Vector kernels of the nonlinear drivers other than Newton: dynamic relaxation
// (jax_fem/solver.py:918-1049, after Luet 2016, ch. 4.3) and the lumped mass of
// assembleCSR's row-eliminated tangent (solver.py:875-888, 959-961).  Every iteration of
// dynamic relaxation is one residual assembly plus three of these fused passes; the
// reductions (max |R|, S0, q'Mq', max eps) go through per-CTA partials reduced in a fixed order.
#include <cmath>

#include "fem_common.cuh"

namespace fem {

constexpr int DR_THREADS = 256;
constexpr int DR_MAX_BLOCKS = 2048;

#define DR_LOOP(i, n) \
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < (n); i += (int64_t)gridDim.x * blockDim.x)

// M_row = h~^2/4 * sum_j |A_row,j| over the scalar CSR row (solver.py:959-961)
__global__ void row_abs_sum_kernel(int64_t n_rows, const int64_t* __restrict__ indptr, const double* __restrict__ vals,
                                   double scale, double* __restrict__ out) {
  DR_LOOP(r, n_rows) {
    double s = 0.0;
    for (int64_t k = indptr[r]; k < indptr[r + 1]; ++k) s += fabs(vals[k]);
    out[r] = scale * s;
  }
}

// q_old = q ; R_old = R ; q += h qdot (solver.py:983-985)
__global__ void dr_march_kernel(int64_t n, double h, double* __restrict__ q, double* __restrict__ q_old,
                                const double* __restrict__ qdot, const double* __restrict__ R,
                                double* __restrict__ R_old) {
  DR_LOOP(i, n) {
    q_old[i] = q[i];
    R_old[i] = R[i];
    q[i] += h * qdot[i];
  }
}

// partials per CTA: [max|R|, S0 = sum (R - R_old)/h qdot, sum qdot M qdot, max eps]
__global__ void __launch_bounds__(DR_THREADS)
dr_measure_kernel(int64_t n, double h, double ht2_4, const double* __restrict__ R, const double* __restrict__ R_old,
                  const double* __restrict__ qdot, const double* __restrict__ M, const double* __restrict__ q,
                  const double* __restrict__ q_old, const double* __restrict__ qdd,
                  const double* __restrict__ qdd_old, double* partials) {
  double rmax = 0.0, s0 = 0.0, den = 0.0, emax = 0.0;
  DR_LOOP(i, n) {
    rmax = fmax(rmax, fabs(R[i]));
    s0 += (R[i] - R_old[i]) / h * qdot[i];
    den += qdot[i] * M[i] * qdot[i];
    const double dq = q[i] - q_old[i];
    if (dq != 0.0) emax = fmax(emax, ht2_4 * fabs((qdd[i] - qdd_old[i]) / dq));
  }
  __shared__ double sh[4][DR_THREADS / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  double v[4] = {rmax, s0, den, emax};
  for (int k = 0; k < 4; ++k) {
    double t = v[k];
    for (int o = 16; o > 0; o >>= 1) {
      const double u = __shfl_xor_sync(0xffffffffu, t, o);
      t = (k == 1 || k == 2) ? t + u : fmax(t, u);
    }
    if (lane == 0) sh[k][w] = t;
  }
  __syncthreads();
  if (threadIdx.x < 4) {
    const int k = threadIdx.x;
    double acc = sh[k][0];
    for (int j = 1; j < DR_THREADS / 32; ++j) acc = (k == 1 || k == 2) ? acc + sh[k][j] : fmax(acc, sh[k][j]);
    partials[blockIdx.x * 4 + k] = acc;
  }
}

__global__ void dr_reduce_kernel(const double* __restrict__ partials, int nb, double* out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double v[4] = {0.0, 0.0, 0.0, 0.0};
  for (int b = 0; b < nb; ++b) {
    v[0] = fmax(v[0], partials[b * 4]);
    v[1] += partials[b * 4 + 1];
    v[2] += partials[b * 4 + 2];
    v[3] = fmax(v[3], partials[b * 4 + 3]);
  }
  for (int k = 0; k < 4; ++k) out[k] = v[k];
}

// qdot_old = qdot ; qdd_old = qdd ; qdot = (2 - c h)/(2 + c h) qdot_old - 2h/(2 + c h) R/M ;
// qdd = (qdot - qdot_old)/h (solver.py:1020-1022)
__global__ void dr_velocity_kernel(int64_t n, double h, double c, const double* __restrict__ R,
                                   const double* __restrict__ M, double* __restrict__ qdot,
                                   double* __restrict__ qdot_old, double* __restrict__ qdd,
                                   double* __restrict__ qdd_old) {
  const double a = (2.0 - c * h) / (2.0 + c * h), b = 2.0 * h / (2.0 + c * h);
  DR_LOOP(i, n) {
    const double vo = qdot[i];
    qdot_old[i] = vo;
    qdd_old[i] = qdd[i];
    const double vn = a * vo - b * R[i] / M[i];
    qdot[i] = vn;
    qdd[i] = (vn - vo) / h;
  }
}

static int dr_grid(int64_t n) {
  int g = grid_for(n, DR_THREADS, 8);
  return g > DR_MAX_BLOCKS ? DR_MAX_BLOCKS : g;
}

}  // namespace fem

using namespace fem;

extern "C" int fem_row_abs_sum(int64_t n_rows, const int64_t* indptr, const double* vals, double scale, double* out,
                               void* stream) {
  FEM_REQUIRE(n_rows >= 0 && (n_rows == 0 || (indptr && vals && out)), "NULL argument");
  if (n_rows == 0) return FEM_OK;
  row_abs_sum_kernel<<<dr_grid(n_rows), DR_THREADS, 0, as_stream(stream)>>>(n_rows, indptr, vals, scale, out);
  note_launches(1);
  return check_launch("row_abs_sum");
}

extern "C" int fem_dr_march(int64_t n, double h, double* q, double* q_old, const double* qdot, const double* R,
                            double* R_old, void* stream) {
  FEM_REQUIRE(n > 0 && q && q_old && qdot && R && R_old, "NULL argument");
  dr_march_kernel<<<dr_grid(n), DR_THREADS, 0, as_stream(stream)>>>(n, h, q, q_old, qdot, R, R_old);
  note_launches(1);
  return check_launch("dr_march");
}

extern "C" int fem_dr_measure(int64_t n, double h, double h_tilde, const double* R, const double* R_old,
                              const double* qdot, const double* M, const double* q, const double* q_old,
                              const double* qdd, const double* qdd_old, double* out4, double* ws, size_t ws_bytes,
                              void* stream) {
  FEM_REQUIRE(n > 0 && R && R_old && qdot && M && q && q_old && qdd && qdd_old && out4 && ws, "NULL argument");
  const int g = dr_grid(n);
  FEM_REQUIRE(ws_bytes >= sizeof(double) * (size_t)(4 * DR_MAX_BLOCKS + 4), "workspace too small");
  cudaStream_t s = as_stream(stream);
  dr_measure_kernel<<<g, DR_THREADS, 0, s>>>(n, h, h_tilde * h_tilde / 4.0, R, R_old, qdot, M, q, q_old, qdd, qdd_old,
                                             ws);
  dr_reduce_kernel<<<1, 32, 0, s>>>(ws, g, ws + 4 * DR_MAX_BLOCKS);
  note_launches(2);
  FEM_CUDA(cudaMemcpyAsync(out4, ws + 4 * DR_MAX_BLOCKS, 4 * sizeof(double), cudaMemcpyDeviceToHost, s));
  FEM_CUDA(cudaStreamSynchronize(s));
  return check_launch("dr_measure");
}

extern "C" int fem_dr_velocity(int64_t n, double h, double c, const double* R, const double* M, double* qdot,
                               double* qdot_old, double* qdd, double* qdd_old, void* stream) {
  FEM_REQUIRE(n > 0 && R && M && qdot && qdot_old && qdd && qdd_old, "NULL argument");
  dr_velocity_kernel<<<dr_grid(n), DR_THREADS, 0, as_stream(stream)>>>(n, h, c, R, M, qdot, qdot_old, qdd, qdd_old);
  note_launches(1);
  return check_launch("dr_velocity");
}
