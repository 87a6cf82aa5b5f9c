// Shared helpers for the jax-fem GB300 kernels: error reporting, launch
// geometry, FP64 block reductions with a deterministic last-block finalize.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <string>

#include "../../include/jaxfem_gb300.h"

namespace fem {

// ---- error reporting (thread-local text behind fem_last_error) ------------
void set_error(const std::string& msg);
int fail(int code, const std::string& msg);
int check_launch(const char* what);
// Count kernel launches (fem_kernel_launches); call next to each <<<...>>>.
void note_launches(int n);

#define FEM_REQUIRE(cond, msg)                                   \
  do {                                                           \
    if (!(cond)) return ::fem::fail(FEM_ERR_ARG, (msg));         \
  } while (0)

#define FEM_CUDA(call)                                                        \
  do {                                                                        \
    cudaError_t e__ = (call);                                                 \
    if (e__ != cudaSuccess)                                                   \
      return ::fem::fail(FEM_ERR_CUDA, std::string(#call ": ") +              \
                                           cudaGetErrorString(e__));          \
  } while (0)

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

// Number of SMs on the current device (cached per process and device).
int sm_count();

// Grid size for a grid-stride kernel: a multiple of the SM count, capped by work.
inline int grid_for(int64_t work_items, int threads, int per_sm = 8) {
  int64_t need = (work_items + threads - 1) / threads;
  int64_t cap = (int64_t)sm_count() * per_sm;
  if (need < 1) need = 1;
  return (int)(need < cap ? need : cap);
}

// ---- reductions ------------------------------------------------------------
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Block-wide sum of NV doubles; result valid in thread 0. `sh` needs
// NV*32 doubles of shared memory. Fixed order => deterministic.
template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV], double* sh) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int nw = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k) v[k] = warp_sum(v[k]);
  if (lane == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) sh[k * 32 + wid] = v[k];
  }
  __syncthreads();
  if (wid == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      double t = lane < nw ? sh[k * 32 + lane] : 0.0;
      v[k] = warp_sum(t);
    }
  }
  __syncthreads();
}

// Last-block-done pattern: every block writes its partials, the block that
// finishes last (atomic ticket) sums all partials in block order and runs
// `finalize`.  No block ever waits on another, so nothing can hang; the
// ticket counter is reset by the last block for the next launch.
// Returns true in (all threads of) the last block.
__device__ __forceinline__ bool last_block_ticket(unsigned int* counter) {
  __shared__ bool is_last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned int t = atomicAdd(counter, 1u);
    is_last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (is_last) {
    __threadfence();
    if (threadIdx.x == 0) *counter = 0u;
  }
  return is_last;
}

// Sum `n` per-block partial vectors (stride NV) in block order; valid in thread 0.
template <int NV>
__device__ __forceinline__ void sum_partials(const double* partials, int n, double (&out)[NV], double* sh) {
#pragma unroll
  for (int k = 0; k < NV; ++k) out[k] = 0.0;
  // each thread sums a strided subset in increasing index order, then a fixed-shape tree
  for (int b = threadIdx.x; b < n; b += blockDim.x) {
    const volatile double* p = partials + (size_t)b * NV;
#pragma unroll
    for (int k = 0; k < NV; ++k) out[k] += p[k];
  }
  block_sum<NV>(out, sh);
}

// Grid stencil: slot k = (di+1)*9 + (dj+1)*3 + (dk+1) of node n = (i*ny + j)*nz + k.  Its column
// offset (the same for every node) and the neighbour's node id, or -1 outside the grid.  Node
// ids grow with (i, j, k) in lexicographic order, so the in-grid slots of a row come in the order
// of its sorted block columns.
__host__ __device__ __forceinline__ int64_t stencil_offset(int k, int64_t ny, int64_t nz) {
  return ((int64_t)(k / 9 - 1) * ny + (k / 3 % 3 - 1)) * nz + (k % 3 - 1);
}
__device__ __forceinline__ int64_t stencil_neighbour(int64_t n, int k, int64_t nx, int64_t ny, int64_t nz) {
  const int64_t i = n / (ny * nz) + k / 9 - 1, j = n / nz % ny + k / 3 % 3 - 1, l = n % nz + k % 3 - 1;
  if (i < 0 || i >= nx || j < 0 || j >= ny || l < 0 || l >= nz) return -1;
  return (i * ny + j) * nz + l;
}

}  // namespace fem
