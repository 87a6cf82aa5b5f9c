// Sparsity pattern of the global matrix, built on the device.
//
// The reference builds COO indices I/J of every cell's (nn*vec)^2 dof pairs
// (jax_fem/problem.py:86-107, plus face blocks that add no new pairs) and lets
// PETSc coalesce them into an AIJ pattern (setPreallocationCOO,
// jax_fem/solver.py:474-478): rows sorted by column, duplicates summed.  That
// pattern is the union of the node pairs that share a cell, each pair a full
// vec x vec block.  Here it is built node-wise without materialising I/J:
//   1. node -> cell incidence (count, scan, fill);
//   2. per node: gather the nodes of its cells, sort + unique -> block row;
//   3. per cell: slot of each (a, b) node pair inside row conn[a];
//   4. the scalar CSR view (indptr, diag offsets, optional indices).
// Every step is wait-free; device-side faults in the input (node ids out of
// range, rows longer than the local buffer) set an error word read by the host.
#include "fem_common.cuh"
#include "fem_elements.cuh"

namespace fem {

constexpr int SCAN_THREADS = 1024;
constexpr int SCAN_ITEMS = 8;

// Single-CTA exclusive scan in place: data[0..n) -> prefix sums, data[n] = total.
// Deterministic and wait-free; used only on node-sized arrays at setup time.
__global__ void scan_single_block(int64_t* data, int64_t n) {
  __shared__ int64_t warp_tot[32];
  __shared__ int64_t carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int64_t base = 0; base < n; base += (int64_t)SCAN_THREADS * SCAN_ITEMS) {
    int64_t v[SCAN_ITEMS];
    int64_t local = 0;
    const int64_t start = base + (int64_t)threadIdx.x * SCAN_ITEMS;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k) {
      const int64_t idx = start + k;
      v[k] = idx < n ? data[idx] : 0;
      local += v[k];
    }
    // inclusive warp scan of per-thread totals
    int64_t incl = local;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int64_t t = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += t;
    }
    if (lane == 31) warp_tot[wid] = incl;
    __syncthreads();
    if (wid == 0) {
      int64_t wt = lane < (SCAN_THREADS / 32) ? warp_tot[lane] : 0;
      int64_t wincl = wt;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int64_t t = __shfl_up_sync(0xffffffffu, wincl, o);
        if (lane >= o) wincl += t;
      }
      if (lane < (SCAN_THREADS / 32)) warp_tot[lane] = wincl - wt;  // exclusive warp offsets
    }
    __syncthreads();
    int64_t run = carry + warp_tot[wid] + (incl - local);
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k) {
      const int64_t idx = start + k;
      if (idx < n) data[idx] = run;
      run += v[k];
    }
    __syncthreads();
    if (threadIdx.x == SCAN_THREADS - 1) carry = run;
    __syncthreads();
  }
  if (threadIdx.x == 0) data[n] = carry;
}

__global__ void count_node_cells(const int32_t* conn, int64_t n_entries, int64_t n_nodes, int64_t* cnt, int* err) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n_entries; k += (int64_t)gridDim.x * blockDim.x) {
    const int node = conn[k];
    if (node < 0 || node >= n_nodes) { atomicExch(err, 1); continue; }
    atomicAdd(reinterpret_cast<unsigned long long*>(cnt + node), 1ull);
  }
}

__global__ void fill_node_cells(const int32_t* conn, int64_t n_entries, int npc, int64_t n_nodes, const int64_t* ptr,
                                int* cursor, int32_t* idx) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n_entries; k += (int64_t)gridDim.x * blockDim.x) {
    const int node = conn[k];
    if (node < 0 || node >= n_nodes) continue;
    const int pos = atomicAdd(cursor + node, 1);
    idx[ptr[node] + pos] = (int32_t)(k / npc);
  }
}

// Sorted-unique insertion into a small local buffer. Returns new size (or -1 on overflow).
template <int MAXB>
__device__ __forceinline__ int insert_unique(int* buf, int size, int v) {
  int lo = 0, hi = size;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (buf[mid] < v) lo = mid + 1; else hi = mid;
  }
  if (lo < size && buf[lo] == v) return size;
  if (size >= MAXB) return -1;
  for (int k = size; k > lo; --k) buf[k] = buf[k - 1];
  buf[lo] = v;
  return size + 1;
}

template <int MAXB, bool FILL>
__global__ void node_rows_kernel(const int32_t* conn, int npc, int64_t n_nodes, const int64_t* nc_ptr,
                                 const int32_t* nc_idx, int64_t* row_len, const int64_t* block_ptr,
                                 int32_t* block_cols, int* err) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n_nodes; i += (int64_t)gridDim.x * blockDim.x) {
    int buf[MAXB];
    int size = 0;
    bool overflow = false;
    for (int64_t p = nc_ptr[i]; p < nc_ptr[i + 1] && !overflow; ++p) {
      const int64_t e = nc_idx[p];
      for (int b = 0; b < npc; ++b) {
        const int s = insert_unique<MAXB>(buf, size, conn[e * npc + b]);
        if (s < 0) { overflow = true; break; }
        size = s;
      }
    }
    if (overflow || size > 255) { atomicExch(err, 2); if (!FILL) row_len[i] = 0; continue; }
    if (!FILL) {
      row_len[i] = size;
    } else {
      const int64_t off = block_ptr[i];
      if (block_ptr[i + 1] - off != size) { atomicExch(err, 3); continue; }
      for (int k = 0; k < size; ++k) block_cols[off + k] = buf[k];
    }
  }
}

__global__ void slots_kernel(const int32_t* conn, int npc, int64_t n_cells, const int64_t* block_ptr,
                             const int32_t* block_cols, uint8_t* slots, int* err) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n_cells * npc; k += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = k / npc;
    const int row = conn[k];
    const int64_t s0 = block_ptr[row], s1 = block_ptr[row + 1];
    for (int b = 0; b < npc; ++b) {
      const int col = conn[e * npc + b];
      int64_t lo = s0, hi = s1;
      while (lo < hi) {
        const int64_t mid = (lo + hi) >> 1;
        if (block_cols[mid] < col) lo = mid + 1; else hi = mid;
      }
      if (lo >= s1 || block_cols[lo] != col) { atomicExch(err, 4); slots[k * npc + b] = 0; continue; }
      slots[k * npc + b] = (uint8_t)(lo - s0);
    }
  }
}

__global__ void scalar_view_kernel(int64_t n_nodes, int vec, const int64_t* bp, const int32_t* bcols, int64_t* indptr,
                                   int64_t* diag, int32_t* indices, int* err) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n_nodes; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b0 = bp[i], nb = bp[i + 1] - b0;
    int64_t kd = -1;
    {
      int64_t lo = b0, hi = b0 + nb;
      while (lo < hi) {
        const int64_t mid = (lo + hi) >> 1;
        if (bcols[mid] < i) lo = mid + 1; else hi = mid;
      }
      if (lo < b0 + nb && bcols[lo] == i) kd = lo - b0;
    }
    if (kd < 0) atomicExch(err, 5);
    for (int c = 0; c < vec; ++c) {
      const int64_t r = (int64_t)vec * i + c;
      const int64_t rs = (int64_t)vec * vec * b0 + (int64_t)c * vec * nb;
      if (indptr) indptr[r] = rs;
      if (diag) diag[r] = kd < 0 ? -1 : rs + vec * kd + c;
      if (indices)
        for (int64_t k = 0; k < nb; ++k)
          for (int d = 0; d < vec; ++d) indices[rs + vec * k + d] = vec * bcols[b0 + k] + d;
    }
    if (i == n_nodes - 1 && indptr) indptr[(int64_t)vec * n_nodes] = (int64_t)vec * vec * bp[n_nodes];
  }
}

// Error words of the two pattern calls that take no workspace (setup-time only;
// calls on different streams must not overlap).
__device__ int g_pattern_err[2];

struct PatternWs {
  int64_t* nc_ptr;   // n_nodes + 1
  int32_t* nc_idx;   // n_cells * npc
  int* cursor;       // n_nodes
  int* err;          // 1
};

static size_t align_up(size_t x) { return (x + 255) & ~size_t(255); }

static size_t pattern_ws_bytes(int64_t n_cells, int npc, int64_t n_nodes) {
  return align_up(sizeof(int64_t) * (n_nodes + 1)) + align_up(sizeof(int32_t) * n_cells * npc) +
         align_up(sizeof(int) * n_nodes) + align_up(sizeof(int) * 4);
}

static PatternWs carve(void* ws, int64_t n_cells, int npc, int64_t n_nodes) {
  char* p = static_cast<char*>(ws);
  PatternWs w;
  w.nc_ptr = reinterpret_cast<int64_t*>(p); p += align_up(sizeof(int64_t) * (n_nodes + 1));
  w.nc_idx = reinterpret_cast<int32_t*>(p); p += align_up(sizeof(int32_t) * n_cells * npc);
  w.cursor = reinterpret_cast<int*>(p); p += align_up(sizeof(int) * n_nodes);
  w.err = reinterpret_cast<int*>(p);
  return w;
}

static int read_err(const int* err_dev, cudaStream_t s, const char* what) {
  int h = 0;
  FEM_CUDA(cudaMemcpyAsync(&h, err_dev, sizeof(int), cudaMemcpyDeviceToHost, s));
  FEM_CUDA(cudaStreamSynchronize(s));
  if (h == 0) return FEM_OK;
  const char* why = h == 1 ? "connectivity holds a node id outside [0, n_nodes)"
                  : h == 2 ? "a node has more than 255 neighbouring nodes (8-bit slots)"
                  : h == 3 ? "block_ptr does not match the counted rows"
                  : h == 4 ? "pattern does not contain a cell's node pair"
                           : "a node row lacks its diagonal block";
  return fail(h == 2 ? FEM_ERR_CAPACITY : FEM_ERR_DEVICE, std::string(what) + ": " + why);
}

template <bool FILL>
static void launch_rows(int elem, const int32_t* conn, int npc, int64_t n_nodes, const PatternWs& w, int64_t* row_len,
                        const int64_t* bp, int32_t* bcols, cudaStream_t s) {
  const int g = grid_for(n_nodes, 128);
  if (elem == FEM_TET10)
    node_rows_kernel<256, FILL><<<g, 128, 0, s>>>(conn, npc, n_nodes, w.nc_ptr, w.nc_idx, row_len, bp, bcols, w.err);
  else
    node_rows_kernel<128, FILL><<<g, 128, 0, s>>>(conn, npc, n_nodes, w.nc_ptr, w.nc_idx, row_len, bp, bcols, w.err);
  note_launches(1);
}

}  // namespace fem

using namespace fem;

extern "C" int fem_pattern_workspace(int64_t n_cells, int32_t nodes_per_cell, int64_t n_nodes, size_t* bytes) {
  FEM_REQUIRE(bytes && n_cells >= 0 && n_nodes >= 0 && nodes_per_cell > 0, "bad arguments");
  *bytes = pattern_ws_bytes(n_cells, nodes_per_cell, n_nodes);
  return FEM_OK;
}

extern "C" int fem_pattern_count(int32_t elem_type, const int32_t* conn, int64_t n_cells, int64_t n_nodes, void* ws,
                                 size_t ws_bytes, int64_t* block_ptr, int64_t* nnzb_out, void* stream) {
  const int npc = elem_nn(elem_type);
  FEM_REQUIRE(npc > 0, "unknown element type");
  FEM_REQUIRE(n_nodes > 0 && n_cells > 0 && conn && block_ptr && nnzb_out && ws, "bad arguments");
  FEM_REQUIRE(ws_bytes >= pattern_ws_bytes(n_cells, npc, n_nodes), "pattern workspace too small");
  cudaStream_t s = as_stream(stream);
  PatternWs w = carve(ws, n_cells, npc, n_nodes);
  FEM_CUDA(cudaMemsetAsync(w.nc_ptr, 0, sizeof(int64_t) * (n_nodes + 1), s));
  FEM_CUDA(cudaMemsetAsync(w.cursor, 0, sizeof(int) * n_nodes, s));
  FEM_CUDA(cudaMemsetAsync(w.err, 0, sizeof(int), s));
  const int64_t ne = n_cells * npc;
  count_node_cells<<<grid_for(ne, 256), 256, 0, s>>>(conn, ne, n_nodes, w.nc_ptr, w.err);
  note_launches(1);
  scan_single_block<<<1, SCAN_THREADS, 0, s>>>(w.nc_ptr, n_nodes);
  note_launches(1);
  fill_node_cells<<<grid_for(ne, 256), 256, 0, s>>>(conn, ne, npc, n_nodes, w.nc_ptr, w.cursor, w.nc_idx);
  note_launches(1);
  launch_rows<false>(elem_type, conn, npc, n_nodes, w, block_ptr, nullptr, nullptr, s);
  scan_single_block<<<1, SCAN_THREADS, 0, s>>>(block_ptr, n_nodes);
  note_launches(1);
  int rc = check_launch("pattern count kernels");
  if (rc) return rc;
  rc = read_err(w.err, s, "fem_pattern_count");
  if (rc) return rc;
  FEM_CUDA(cudaMemcpyAsync(nnzb_out, block_ptr + n_nodes, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  FEM_CUDA(cudaStreamSynchronize(s));
  return FEM_OK;
}

extern "C" int fem_pattern_fill(int32_t elem_type, const int32_t* conn, int64_t n_cells, int64_t n_nodes, void* ws,
                                size_t ws_bytes, const int64_t* block_ptr, int32_t* block_cols, void* stream) {
  const int npc = elem_nn(elem_type);
  FEM_REQUIRE(npc > 0, "unknown element type");
  FEM_REQUIRE(n_nodes > 0 && n_cells > 0 && conn && block_ptr && block_cols && ws, "bad arguments");
  FEM_REQUIRE(ws_bytes >= pattern_ws_bytes(n_cells, npc, n_nodes), "pattern workspace too small");
  cudaStream_t s = as_stream(stream);
  PatternWs w = carve(ws, n_cells, npc, n_nodes);
  FEM_CUDA(cudaMemsetAsync(w.err, 0, sizeof(int), s));
  launch_rows<true>(elem_type, conn, npc, n_nodes, w, nullptr, block_ptr, block_cols, s);
  int rc = check_launch("pattern fill kernel");
  if (rc) return rc;
  return read_err(w.err, s, "fem_pattern_fill");
}

extern "C" int fem_pattern_slots(int32_t elem_type, const int32_t* conn, int64_t n_cells, const int64_t* block_ptr,
                                 const int32_t* block_cols, uint8_t* slots, void* stream) {
  const int npc = elem_nn(elem_type);
  FEM_REQUIRE(npc > 0, "unknown element type");
  FEM_REQUIRE(conn && block_ptr && block_cols && slots && n_cells > 0, "bad arguments");
  cudaStream_t s = as_stream(stream);
  int* err = nullptr;
  FEM_CUDA(cudaGetSymbolAddress(reinterpret_cast<void**>(&err), g_pattern_err));
  FEM_CUDA(cudaMemsetAsync(err, 0, sizeof(int), s));
  slots_kernel<<<grid_for(n_cells * npc, 256), 256, 0, s>>>(conn, npc, n_cells, block_ptr, block_cols, slots, err);
  note_launches(1);
  int rc = check_launch("slots kernel");
  if (rc) return rc;
  return read_err(err, s, "fem_pattern_slots");
}

extern "C" int fem_pattern_scalar(int64_t n_nodes, int32_t vec, const int64_t* block_ptr, const int32_t* block_cols,
                                  int64_t* indptr, int64_t* diag, int32_t* indices, void* stream) {
  FEM_REQUIRE(n_nodes > 0 && (vec == 1 || vec == 3) && block_ptr && block_cols, "bad arguments");
  cudaStream_t s = as_stream(stream);
  int* err = nullptr;
  FEM_CUDA(cudaGetSymbolAddress(reinterpret_cast<void**>(&err), g_pattern_err));
  err += 1;
  FEM_CUDA(cudaMemsetAsync(err, 0, sizeof(int), s));
  scalar_view_kernel<<<grid_for(n_nodes, 256), 256, 0, s>>>(n_nodes, vec, block_ptr, block_cols, indptr, diag, indices,
                                                            err);
  note_launches(1);
  int rc = check_launch("scalar view kernel");
  if (rc) return rc;
  return read_err(err, s, "fem_pattern_scalar");
}

// ---- sliced layout: 32 node rows per slice, width = longest row in the slice --------
namespace fem {
__global__ void slice_width_kernel(int64_t n_nodes, int64_t n_slices, const int64_t* bp, int64_t* widths) {
  for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < n_slices; s += (int64_t)gridDim.x * blockDim.x) {
    int64_t w = 0;
    for (int l = 0; l < 32; ++l) {
      const int64_t i = s * 32 + l;
      if (i < n_nodes) { const int64_t nb = bp[i + 1] - bp[i]; w = nb > w ? nb : w; }
    }
    widths[s] = w;
  }
}

// slice_cols[(slice_ptr[s] + k) * 32 + l] = block column k of node 32 s + l (0 beyond the row)
__global__ void slice_cols_kernel(int64_t n_nodes, int64_t n_slices, const int64_t* bp, const int32_t* bcols,
                                  const int64_t* sp, int32_t* scols) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n_slices * 32; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t s = t >> 5;
    const int l = (int)(t & 31);
    const int64_t i = s * 32 + l;
    const int64_t b0 = i < n_nodes ? bp[i] : 0;
    const int64_t nb = i < n_nodes ? bp[i + 1] - b0 : 0;
    for (int64_t k = 0; k < sp[s + 1] - sp[s]; ++k)
      scols[(sp[s] + k) * 32 + l] = k < nb ? bcols[b0 + k] : 0;
  }
}
// Grid layout: every block of row n must couple a stencil neighbour (|di|, |dj|, |dk| <= 1);
// a row that does not sets *bad (thread per node row).
__global__ void slice_grid_check_kernel(int64_t n_nodes, const int64_t* bp, const int32_t* bcols, int64_t ny,
                                        int64_t nz, unsigned long long* bad) {
  for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < n_nodes; n += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = n / (ny * nz), j = n / nz % ny, k = n % nz;
    bool ok = true;
    for (int64_t b = bp[n]; b < bp[n + 1]; ++b) {
      const int64_t c = bcols[b];
      if (c < 0 || c >= n_nodes) { ok = false; break; }
      const int64_t di = c / (ny * nz) - i, dj = c / nz % ny - j, dk = c % nz - k;
      if (di < -1 || di > 1 || dj < -1 || dj > 1 || dk < -1 || dk > 1) { ok = false; break; }
    }
    if (!ok) atomicOr(bad, 1ull);
  }
}

// Grid layout: slice_ptr[s] = 27 s; slice_cols of slot k, lane l = node + stencil offset k,
// clamped to the node range (thread per (slice, lane)).
__global__ void slice_grid_cols_kernel(int64_t n_nodes, int64_t n_slices, int64_t ny, int64_t nz, int64_t* sp,
                                       int32_t* scols) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n_slices * 32; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t s = t >> 5;
    const int l = (int)(t & 31);
    const int64_t n = s * 32 + l;
    for (int k = 0; k < 27; ++k) {
      int64_t c = n + stencil_offset(k, ny, nz);
      c = c < 0 ? 0 : c >= n_nodes ? n_nodes - 1 : c;
      scols[(s * 27 + k) * 32 + l] = (int32_t)c;
    }
    if (l == 0) sp[s] = s * 27;
    if (t == 0) sp[n_slices] = n_slices * 27;
  }
}

// Upper node blocks of row i: the suffix of its sorted block columns starting at the first
// column >= i (the diagonal).
__device__ __forceinline__ int64_t first_upper(const int32_t* bcols, int64_t b0, int64_t nb, int64_t i) {
  int64_t u = 0;
  while (u < nb && bcols[b0 + u] < i) ++u;
  return u;
}

__global__ void slice_width_upper_kernel(int64_t n_nodes, int64_t n_slices, const int64_t* bp, const int32_t* bcols,
                                         int64_t* widths) {
  for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < n_slices; s += (int64_t)gridDim.x * blockDim.x) {
    int64_t w = 0;
    for (int l = 0; l < 32; ++l) {
      const int64_t i = s * 32 + l;
      if (i < n_nodes) {
        const int64_t nb = bp[i + 1] - bp[i];
        const int64_t nu = nb - first_upper(bcols, bp[i], nb, i);
        w = nu > w ? nu : w;
      }
    }
    widths[s] = w;
  }
}

__global__ void slice_cols_upper_kernel(int64_t n_nodes, int64_t n_slices, const int64_t* bp, const int32_t* bcols,
                                        const int64_t* sp, int32_t* scols) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n_slices * 32; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t s = t >> 5;
    const int l = (int)(t & 31);
    const int64_t i = s * 32 + l;
    const int64_t b0 = i < n_nodes ? bp[i] : 0;
    const int64_t nb = i < n_nodes ? bp[i + 1] - b0 : 0;
    const int64_t u0 = i < n_nodes ? first_upper(bcols, b0, nb, i) : 0;
    const int32_t pad = i < n_nodes ? (int32_t)i : 0;
    for (int64_t k = 0; k < sp[s + 1] - sp[s]; ++k)
      scols[(sp[s] + k) * 32 + l] = u0 + k < nb ? bcols[b0 + u0 + k] : pad;
  }
}
}  // namespace fem

extern "C" int fem_pattern_slices_upper(int64_t n_nodes, const int64_t* block_ptr, const int32_t* block_cols,
                                        int64_t* slice_ptr_u, int32_t* slice_cols_u, int64_t* n_slots_u,
                                        void* stream) {
  FEM_REQUIRE(n_nodes > 0 && block_ptr && block_cols && slice_ptr_u, "bad arguments");
  cudaStream_t s = as_stream(stream);
  const int64_t n_slices = (n_nodes + 31) / 32;
  if (slice_cols_u == nullptr) {
    FEM_REQUIRE(n_slots_u, "n_slots_u NULL");
    slice_width_upper_kernel<<<grid_for(n_slices, 256), 256, 0, s>>>(n_nodes, n_slices, block_ptr, block_cols,
                                                                      slice_ptr_u);
    scan_single_block<<<1, SCAN_THREADS, 0, s>>>(slice_ptr_u, n_slices);
    note_launches(2);
    int rc = check_launch("upper slice widths");
    if (rc) return rc;
    FEM_CUDA(cudaMemcpyAsync(n_slots_u, slice_ptr_u + n_slices, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    FEM_CUDA(cudaStreamSynchronize(s));
    return FEM_OK;
  }
  slice_cols_upper_kernel<<<grid_for(n_slices * 32, 256), 256, 0, s>>>(n_nodes, n_slices, block_ptr, block_cols,
                                                                        slice_ptr_u, slice_cols_u);
  note_launches(1);
  return check_launch("upper slice cols");
}

extern "C" int fem_pattern_slices_grid(int64_t n_nodes, const int64_t* block_ptr, const int32_t* block_cols,
                                       int64_t nx, int64_t ny, int64_t nz, int64_t* slice_ptr, int32_t* slice_cols,
                                       void* stream) {
  FEM_REQUIRE(n_nodes > 0 && block_ptr && block_cols && slice_ptr && slice_cols, "bad arguments");
  FEM_REQUIRE(nx > 0 && ny > 0 && nz > 0 && nx <= n_nodes && ny <= n_nodes && nz <= n_nodes &&
                  nx * ny <= n_nodes && nx * ny * nz == n_nodes,
              "the node grid must hold n_nodes nodes");
  FEM_REQUIRE(n_nodes < (int64_t(1) << 31), "node ids must fit int32");
  cudaStream_t s = as_stream(stream);
  const int64_t n_slices = (n_nodes + 31) / 32;
  unsigned long long* bad = reinterpret_cast<unsigned long long*>(slice_ptr + n_slices);
  FEM_CUDA(cudaMemsetAsync(bad, 0, sizeof(unsigned long long), s));
  slice_grid_check_kernel<<<grid_for(n_nodes, 256), 256, 0, s>>>(n_nodes, block_ptr, block_cols, ny, nz, bad);
  note_launches(1);
  int rc = check_launch("grid slice check");
  if (rc) return rc;
  unsigned long long h = 0;
  FEM_CUDA(cudaMemcpyAsync(&h, bad, sizeof(h), cudaMemcpyDeviceToHost, s));
  FEM_CUDA(cudaStreamSynchronize(s));
  if (h) return fail(FEM_ERR_ARG, "fem_pattern_slices_grid: a node row couples a node outside its 27-point stencil");
  slice_grid_cols_kernel<<<grid_for(n_slices * 32, 256), 256, 0, s>>>(n_nodes, n_slices, ny, nz, slice_ptr,
                                                                       slice_cols);
  note_launches(1);
  return check_launch("grid slice cols");
}

extern "C" int fem_pattern_slices(int64_t n_nodes, const int64_t* block_ptr, const int32_t* block_cols,
                                  int64_t* slice_ptr, int32_t* slice_cols, int64_t* n_slots, void* stream) {
  FEM_REQUIRE(n_nodes > 0 && block_ptr && block_cols && slice_ptr, "bad arguments");
  cudaStream_t s = as_stream(stream);
  const int64_t n_slices = (n_nodes + 31) / 32;
  if (slice_cols == nullptr) {
    FEM_REQUIRE(n_slots, "n_slots NULL");
    slice_width_kernel<<<grid_for(n_slices, 256), 256, 0, s>>>(n_nodes, n_slices, block_ptr, slice_ptr);
    scan_single_block<<<1, SCAN_THREADS, 0, s>>>(slice_ptr, n_slices);
    note_launches(2);
    int rc = check_launch("slice widths");
    if (rc) return rc;
    FEM_CUDA(cudaMemcpyAsync(n_slots, slice_ptr + n_slices, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    FEM_CUDA(cudaStreamSynchronize(s));
    return FEM_OK;
  }
  slice_cols_kernel<<<grid_for(n_slices * 32, 256), 256, 0, s>>>(n_nodes, n_slices, block_ptr, block_cols, slice_ptr,
                                                                  slice_cols);
  note_launches(1);
  return check_launch("slice cols");
}
