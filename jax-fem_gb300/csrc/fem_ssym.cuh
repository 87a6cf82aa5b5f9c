// Structured symmetric DF48 SpMV (FEM_SSYM_DF48), included by fem_krylov.cu.
//
// For a node grid numbered node = (i*ny + j)*nz + k (x slowest, z fastest: the box meshes of
// this path) the node-block pattern is the 27-point stencil and the symmetric tangent is carried
// by 14 blocks per node row: the diagonal and the 13 neighbours with a larger index,
//   slot 0 (0,0,0)   slot 1 (0,0,+1)   slots 2-4 (0,+1,-1..+1)
//   slots 5-7 (+1,-1,-1..+1)   slots 8-10 (+1,0,-1..+1)   slots 11-13 (+1,+1,-1..+1)   (di,dj,dk).
// Block columns are implicit (no index array) and each off-diagonal block serves twice: A_ij x_j
// for row i and A_ij^T x_i for row j, so the SpMV streams 14 of the 27 blocks of each row.
//
// The transposed half is accumulated where it stays cheap.  A "line" is the z-column (i, j, *),
// line index L = i*ny + j.  A warp takes 32 consecutive lines (lane l: line L0 + l) over a range
// of k (a chunk) and steps through k, so for row (L, k):
//   slot 1  -> (L, k+1): the lane's own next row, a register carry;
//   slots 2-4 -> line L+1, rows k-1..k+1: lane l+1's own rows, a warp shuffle;
//   slots 5-13 -> plane i+1, lines L+ny-1..L+ny+1: shuffled across lanes so that lane m holds the
//     sum for line L0+ny+m, summed over three steps for each row, then ONE FP64 atomic per
//     component and row into qT (the only traffic that leaves the warp).
// Contributions that cross a warp's edge (lane 31's next line, the far lines just outside the
// warp's 32, the rows next to a chunk boundary) also go to qT by atomics.  The consumer (the CG
// update kernel) adds qT to the double-float result and zeroes it.  Neighbour x values come from
// a per-warp shared-memory window holding three k positions of the warp's 33 own lines and 34 far
// lines; matrix values stream through the same bulk-copy ring as the sliced DF48 kernel.
namespace fem {

constexpr int SS_SLOTS = 14;
constexpr int SS_WARPS = 4;
constexpr int SS_STAGES = 2;           // ring depth per warp (2 x 3456 B in flight)
constexpr int SS_STAGE_SLOTS = 2;          // 14 slots per row step = 7 stages
constexpr int SS_WIN_LINES = 67;           // 33 own lines (L0 .. L0+32) + 34 far (L0+ny-1 .. L0+ny+32)

__host__ __device__ constexpr int ss_di(int s) { return s < 5 ? 0 : 1; }
__host__ __device__ constexpr int ss_dj(int s) { return s < 2 ? 0 : s < 5 ? 1 : s < 8 ? -1 : s < 11 ? 0 : 1; }
__host__ __device__ constexpr int ss_dk(int s) { return s == 0 ? 0 : s == 1 ? 1 : ((s - 2) % 3) - 1; }

struct SsGrid {
  int64_t nx, ny, nz, nl, groups;   // nl = nx*ny lines, groups = ceil(nl / 32)
  int chunks;                       // k ranges per group (launch choice)
};

__host__ __device__ inline SsGrid ss_grid(const fem_pattern_t* p, int chunks) {
  SsGrid g;
  g.nx = p->grid_nx; g.ny = p->grid_ny; g.nz = p->grid_nz;
  g.nl = g.nx * g.ny;
  g.groups = (g.nl + 31) / 32;
  g.chunks = chunks;
  return g;
}

// value v (r*3+d) of slot s of row step k of group g, lane l
__host__ __device__ inline int64_t ss_index(const SsGrid& G, int64_t g, int64_t k, int s, int v, int l) {
  return (((g * G.nz + k) * SS_SLOTS + s) * 9 + v) * 32 + l;
}

template <typename T>
__device__ __forceinline__ int bsearch_cols(const int32_t* c, int n, T key) {
  int lo = 0, hi = n - 1;
  while (lo <= hi) {
    const int mid = (lo + hi) >> 1;
    const T v = (T)c[mid];
    if (v == key) return mid;
    if (v < key) lo = mid + 1; else hi = mid - 1;
  }
  return -1;
}

__device__ __forceinline__ void df48_encode(double a, float& h, int16_t& q) {
  h = __double2float_rn(a);
  const int e = (__float_as_int(h) >> 23) & 0xFF;
  int qq = 0;
  if (e > 39 && e < 255) {
    double tq = rint(scalbn(a - (double)h, 166 - e));
    tq = fmin(fmax(tq, -32767.0), 32767.0);
    qq = (int)tq;
  }
  q = (int16_t)qq;
}

// FP64 CSR values (vec 3) -> FEM_SSYM_DF48, thread per (group, k, lane).  Each row's upper CSR
// blocks (column >= row) must all be stencil slots; a row with one that is not sets *err.
__global__ void to_ssym_kernel(SsGrid G, const int64_t* __restrict__ bp, const int32_t* __restrict__ bcols,
                               const double* __restrict__ v64, float* __restrict__ hi, int16_t* __restrict__ lo,
                               int* __restrict__ err) {
  const int64_t total = G.groups * G.nz * 32;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int l = (int)(t & 31);
    const int64_t gk = t >> 5;
    const int64_t g = gk / G.nz, k = gk - g * G.nz;
    const int64_t L = g * 32 + l;
    const bool valid = L < G.nl;
    const int64_t i = valid ? L / G.ny : 0, j = valid ? L - i * G.ny : 0;
    const int64_t node = L * G.nz + k;
    const int64_t b0 = valid ? bp[node] : 0;
    const int nb = valid ? (int)(bp[node + 1] - b0) : 0;
    int found = 0;
    for (int s = 0; s < SS_SLOTS; ++s) {
      const int64_t ii = i + ss_di(s), jj = j + ss_dj(s), kk = k + ss_dk(s);
      const bool ok = valid && ii < G.nx && jj >= 0 && jj < G.ny && kk >= 0 && kk < G.nz;
      const int kb = ok ? bsearch_cols<int64_t>(bcols + b0, nb, (ii * G.ny + jj) * G.nz + kk) : -1;
      found += kb >= 0 ? 1 : 0;
      for (int v = 0; v < 9; ++v) {
        const int r = v / 3, d = v - 3 * r;
        const double a = kb >= 0 ? v64[9 * b0 + (int64_t)r * 3 * nb + 3 * kb + d] : 0.0;
        float h;
        int16_t q;
        df48_encode(a, h, q);
        const int64_t o = ss_index(G, g, k, s, v, l);
        hi[o] = h;
        lo[o] = q;
      }
    }
    if (valid) {
      int upper = 0;
      for (int b = 0; b < nb; ++b) upper += bcols[b0 + b] >= node ? 1 : 0;
      if (upper != found) atomicExch(err, 1);
    }
  }
}

template <int N>
struct Df3 {
  float h[N], l[N];
};

struct SsGeom {
  static constexpr uint32_t VB = 9 * 32 * 4;        // value bytes per slot
  static constexpr uint32_t LB = 9 * 32 * 2;        // correction bytes per slot
  static constexpr uint32_t STAGE = SS_STAGE_SLOTS * (VB + LB);
  static constexpr uint32_t BAR_BYTES = 128;
  static constexpr uint32_t WIN = 3 * 2 * SS_WIN_LINES * 16;   // [pos][half][line] float4
  static constexpr uint32_t SMEM = BAR_BYTES + SS_WARPS * (SS_STAGES * STAGE + WIN);
};

__device__ __forceinline__ float df_shfl_down_f(float v) { return __shfl_down_sync(0xffffffffu, v, 1); }
__device__ __forceinline__ float df_shfl_up_f(float v) { return __shfl_up_sync(0xffffffffu, v, 1); }

// dst += (h, l) componentwise in double-float
__device__ __forceinline__ void df3_add(float* dh, float* dl, const float* h, const float* l) {
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const df2 s = df_add(df2{dh[c], dl[c]}, df2{h[c], l[c]});
    dh[c] = s.h;
    dl[c] = s.l;
  }
}

// qT[c][node] += h + l (component stride qt_stride).  For emissions made by every lane of a warp:
// one FP64 add per nonzero component (a warp-wide FP64 instruction serves 32 rows).
__device__ __forceinline__ void ss_atomic3(double* qT, int64_t stride, int64_t node, const float* h, const float* l) {
#pragma unroll
  for (int c = 0; c < 3; ++c)
    if ((__float_as_uint(h[c]) & 0x7FFFFFFFu) != 0u) atomicAdd(qT + (int64_t)c * stride + node, f2d_bits(h[c]) + f2d_bits(l[c]));
}

// The same for emissions made by a single lane (the warp's edge lanes): h and l as two atomics and
// no FP64 arithmetic -- a warp-wide FP64 instruction would cost GB300's FP64 pipe as much for one
// active lane as for 32.
__device__ __forceinline__ void ss_atomic3_lane(double* qT, int64_t stride, int64_t node, const float* h,
                                                const float* l) {
#pragma unroll
  for (int c = 0; c < 3; ++c)
    if ((__float_as_uint(h[c]) & 0x7FFFFFFFu) != 0u) {
      atomicAdd(qT + (int64_t)c * stride + node, f2d_bits(h[c]));
      if ((__float_as_uint(l[c]) & 0x7FFFFFFFu) != 0u) atomicAdd(qT + (int64_t)c * stride + node, f2d_bits(l[c]));
    }
}

// y (double-float, the row parts plus the transposed parts that stayed in the warp) and qT (FP64,
// the rest, added by atomics) with y + qT = A x; fused dot x.(A x) = sum_i 2 x_i.(U x)_i - x_i.A_ii x_i
// (U: the stored upper blocks including the diagonal).  Requires 16-byte aligned vals and vlo.
__global__ void __launch_bounds__(SS_WARPS * 32, 4)   // 4 CTAs (16 warps) per SM
spmv_ssym_bulk_kernel(SsGrid G, const float* __restrict__ vals, const int16_t* __restrict__ vlo,
                      const float2* __restrict__ xp, float* __restrict__ yh, float* __restrict__ yl,
                      double* __restrict__ qT, KCtl* C, int op, double* partials) {
  using Gm = SsGeom;
  extern __shared__ __align__(128) unsigned char smem[];
  if (C->done) return;
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem) + wib * SS_STAGES;
  unsigned char* wbase = smem + Gm::BAR_BYTES + (size_t)wib * (SS_STAGES * Gm::STAGE + Gm::WIN);
  unsigned char* ring = wbase;
  float4* win = reinterpret_cast<float4*>(wbase + SS_STAGES * Gm::STAGE);   // [pos][half][line]
  const int64_t qstride = qt_stride(G.nl * G.nz);   // the component stride of qT
  const int64_t n_items = G.groups * G.chunks;
  const int64_t warp = (int64_t)blockIdx.x * SS_WARPS + wib;
  const int64_t nwarps = (int64_t)gridDim.x * SS_WARPS;
  if (lane == 0) {
#pragma unroll
    for (int j = 0; j < SS_STAGES; ++j) mbar_init(bars + j, 1);
    mbar_init_fence();
  }
  __syncwarp();

  auto item_range = [&](int64_t it, int64_t& g, int64_t& k0, int64_t& k1) {
    g = it / G.chunks;
    const int64_t c = it - g * G.chunks;
    k0 = c * G.nz / G.chunks;
    k1 = (c + 1) * G.nz / G.chunks;
  };
  // producer cursor over slot runs (all lanes track it; lane 0 issues)
  int64_t pit = warp, pk = 0, pe = 0;
  auto prun = [&]() {
    int64_t g, k0, k1;
    item_range(pit, g, k0, k1);
    pk = (g * G.nz + k0) * SS_SLOTS;
    pe = (g * G.nz + k1) * SS_SLOTS;
  };
  if (pit < n_items) prun();
  auto produce = [&](int stage) -> bool {
    while (pit < n_items && pk == pe) {
      pit += nwarps;
      if (pit < n_items) prun();
    }
    if (pit >= n_items) return false;
    if (lane == 0) {
      unsigned char* st = ring + (size_t)stage * Gm::STAGE;
      async_proxy_fence();
      mbar_expect_tx(bars + stage, SS_STAGE_SLOTS * (Gm::VB + Gm::LB));
      const uint64_t pol = l2_evict_first_policy();   // the matrix streams through L2 evict-first
      bulk_load_hint(st, vals + pk * 9 * 32, SS_STAGE_SLOTS * Gm::VB, bars + stage, pol);
      bulk_load_hint(st + SS_STAGE_SLOTS * Gm::VB, vlo + pk * 9 * 32, SS_STAGE_SLOTS * Gm::LB, bars + stage, pol);
    }
    pk += SS_STAGE_SLOTS;
    return true;
  };
  uint32_t parity = 0;
  int inflight = 0;
  for (int j = 0; j < SS_STAGES; ++j) inflight += produce(j) ? 1 : 0;
  int stage = 0;
  bool fault = false;
  float ds = 0.f, de = 0.f;

  // window: line slot w in [0, 67): own lines L0 + w (w <= 32), far lines L0 + ny - 1 + (w - 33)
  // window position of row k: k mod 3, tracked incrementally by the caller (no 64-bit modulo)
  auto load_win = [&](int64_t L0, int64_t k, int pos) {
    auto put = [&](int w, int64_t line) {
      float4 a = make_float4(0.f, 0.f, 0.f, 0.f), b = a;
      if (line >= 0 && line < G.nl && k >= 0 && k < G.nz) {
        const float4* p4 = reinterpret_cast<const float4*>(xp) + 2 * (line * G.nz + k);
        a = __ldg(p4);
        b = __ldg(p4 + 1);
      }
      win[(pos * 2 + 0) * SS_WIN_LINES + w] = a;
      win[(pos * 2 + 1) * SS_WIN_LINES + w] = b;
    };
    put(lane, L0 + lane);                       // own lines
    put(34 + lane, L0 + G.ny + lane);           // far lines L0+ny .. L0+ny+31
    if (lane == 31) {
      put(32, L0 + 32);                         // next warp's first line (lane 31's line + 1)
      put(66, L0 + G.ny + 32);                  // far line L0+ny+32
    }
    if (lane == 0) put(33, L0 + G.ny - 1);      // far line L0+ny-1
  };
  auto get_win = [&](int w, int pos, float* h, float* l) {
    const float4 a = win[(pos * 2 + 0) * SS_WIN_LINES + w];
    const float4 b = win[(pos * 2 + 1) * SS_WIN_LINES + w];
    h[0] = a.x; l[0] = a.y; h[1] = a.z; l[1] = a.w; h[2] = b.x; l[2] = b.y;
  };

  for (int64_t it = warp; it < n_items && !fault; it += nwarps) {
    int64_t g, k0, k1;
    item_range(it, g, k0, k1);
    if (k0 == k1) continue;
    const int64_t L0 = g * 32;
    const int64_t L = L0 + lane;
    const bool lv = L < G.nl;
    const int64_t Lf = L0 + G.ny + lane;        // this lane's far target line
    const bool fv = Lf < G.nl;
    // windows for k0 - 1 and k0 (k0 + 1 is loaded by the first step)
    __syncwarp();
    int pm = (int)((k0 + 2) % 3), p0 = (int)(k0 % 3), pp = (int)((k0 + 1) % 3);   // rows k-1, k, k+1
    load_win(L0, k0 - 1, pm);
    load_win(L0, k0, p0);
    Df3<3> Y0, Y1, Y2, F0, F1, F2;   // own line rows k-1, k, k+1; far line rows k-1, k, k+1
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      Y0.h[c] = Y0.l[c] = Y1.h[c] = Y1.l[c] = Y2.h[c] = Y2.l[c] = 0.f;
      F0.h[c] = F0.l[c] = F1.h[c] = F1.l[c] = F2.h[c] = F2.l[c] = 0.f;
    }
    for (int64_t k = k0; k < k1 && !fault; ++k) {
      load_win(L0, k + 1, pp);
      __syncwarp();
      float xh[3], xl[3];   // the row's own x
      get_win(lane, p0, xh, xl);
      // row part (U x)_row in two banks (the two slots of a stage), two independent chains
      float rh[2][3] = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}}, rl[2][3] = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};
      float dh = 0.f, dl = 0.f;                                  // x.A_ii x
      // The seven stages of a row step share one loop body (kept rolled: unrolling all 14 slots
      // overflowed the instruction cache); slot-dependent routing is warp-uniform branching.
#pragma unroll 1
      for (int sp = 0; sp < SS_SLOTS / SS_STAGE_SLOTS; ++sp) {
        const bool ok = mbar_wait(bars + stage, (parity >> stage) & 1u);
        if (!__all_sync(0xffffffffu, ok)) { fault = true; break; }
        parity ^= 1u << stage;
        --inflight;
        const unsigned char* st = ring + (size_t)stage * Gm::STAGE;
        const float* sv = reinterpret_cast<const float*>(st);
        const int16_t* sq = reinterpret_cast<const int16_t*>(st + SS_STAGE_SLOTS * Gm::VB);
#pragma unroll
        for (int u = 0; u < SS_STAGE_SLOTS; ++u) {
          const int s = sp * SS_STAGE_SLOTS + u;
          float ah[9], al[9];
#pragma unroll
          for (int v = 0; v < 9; ++v) {
            ah[v] = sv[(u * 9 + v) * 32 + lane];
            al[v] = df48_lo(ah[v], sq[(u * 9 + v) * 32 + lane]);
          }
          // neighbour x of this slot from the window
          const int dk = ss_dk(s);
          const bool far = s >= 5;
          const int dj = far ? ss_dj(s) : 1;
          const int w = s < 2 ? lane : far ? 33 + lane + 1 + dj : lane + 1;
          float nh[3], nl[3];
          get_win(w, dk < 0 ? pm : dk > 0 ? pp : p0, nh, nl);
#pragma unroll
          for (int v = 0; v < 9; ++v) df_acc(rh[u][v / 3], rl[u][v / 3], df2{ah[v], al[v]}, df2{nh[v % 3], nl[v % 3]});
          float th[3] = {0.f, 0.f, 0.f}, tl[3] = {0.f, 0.f, 0.f};
          if (s == 0) {   // x.A_ii x for the fused dot
#pragma unroll
            for (int v = 0; v < 9; ++v) df_acc(th[v / 3], tl[v / 3], df2{ah[v], al[v]}, df2{xh[v % 3], xl[v % 3]});
#pragma unroll
            for (int r = 0; r < 3; ++r) df_acc(dh, dl, df2{xh[r], xl[r]}, df_fast(th[r], tl[r]));
            continue;
          }
          // transposed contribution t = A^T x_row to the slot's neighbour
#pragma unroll
          for (int v = 0; v < 9; ++v) df_acc(th[v % 3], tl[v % 3], df2{ah[v], al[v]}, df2{xh[v / 3], xl[v / 3]});
#pragma unroll
          for (int c = 0; c < 3; ++c) { const df2 f = df_fast(th[c], tl[c]); th[c] = f.h; tl[c] = f.l; }
          if (s == 1) {                        // own line, row k+1
            df3_add(Y2.h, Y2.l, th, tl);
            continue;
          }
          // line L+1 (slots 2-4) and plane i+1 lines L+ny+dj (slots 5-13): the receiving lane is
          // lane+1 (shuffle up) for the next line and dj = +1, lane-1 (shuffle down) for dj = -1,
          // the lane itself for dj = 0
          float uh[3], ul[3];
          bool recv = true;
          if (dj > 0) {
#pragma unroll
            for (int c = 0; c < 3; ++c) { uh[c] = df_shfl_up_f(th[c]); ul[c] = df_shfl_up_f(tl[c]); }
            recv = lane > 0;
          } else if (dj < 0) {
#pragma unroll
            for (int c = 0; c < 3; ++c) { uh[c] = df_shfl_down_f(th[c]); ul[c] = df_shfl_down_f(tl[c]); }
            recv = lane < 31;
          } else {
#pragma unroll
            for (int c = 0; c < 3; ++c) { uh[c] = th[c]; ul[c] = tl[c]; }
          }
          if (!recv) {
#pragma unroll
            for (int c = 0; c < 3; ++c) uh[c] = ul[c] = 0.f;
          }
          if (far) {
            if (dk < 0) df3_add(F0.h, F0.l, uh, ul);
            else if (dk == 0) df3_add(F1.h, F1.l, uh, ul);
            else df3_add(F2.h, F2.l, uh, ul);
          } else {
            if (dk < 0) df3_add(Y0.h, Y0.l, uh, ul);
            else if (dk == 0) df3_add(Y1.h, Y1.l, uh, ul);
            else df3_add(Y2.h, Y2.l, uh, ul);
          }
          // the edge lane whose target line lies outside this warp's lines: an atomic
          const int esc = dj > 0 ? 31 : dj < 0 ? 0 : -1;
          if (lane == esc && lv) {
            const int64_t tk = k + dk;
            const int64_t tline = !far ? L0 + 32 : dj < 0 ? L0 + G.ny - 1 : L0 + G.ny + 32;
            if (tline < G.nl && tk >= 0 && tk < G.nz) ss_atomic3_lane(qT, qstride, tline * G.nz + tk, th, tl);
          }
        }
        __syncwarp();
        inflight += produce(stage) ? 1 : 0;
        stage = stage + 1 == SS_STAGES ? 0 : stage + 1;
      }
      if (fault) break;
      // the row part joins row k; fused dot 2 x.(U x) - x.A_ii x
      float yr[3], yrl[3];
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const df2 f = df_add(df_fast(rh[0][c], rl[0][c]), df_fast(rh[1][c], rl[1][c]));
        yr[c] = f.h;
        yrl[c] = f.l;
      }
      df3_add(Y1.h, Y1.l, yr, yrl);
      if (lv) {
        float eh = 0.f, el = 0.f;
#pragma unroll
        for (int c = 0; c < 3; ++c) df_acc(eh, el, df2{xh[c], xl[c]}, df2{yr[c], yrl[c]});
        const df2 two = df_add(df2{2.f * eh, 2.f * el}, df2{-dh, -dl});
        const df2 acc = df_add(df2{ds, de}, two);
        ds = acc.h;
        de = acc.l;
      }
      // row k-1 of the own line is complete: it belongs to this chunk (plain store) or is the
      // previous chunk's last row (its part from this chunk goes to qT)
      const int64_t kp = k - 1;
      if (lv && kp >= 0) {
        const int64_t node = L * G.nz + kp;
        if (kp >= k0) {
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            const df2 f = df_fast(Y0.h[c], Y0.l[c]);
            yh[3 * node + c] = f.h;
            yl[3 * node + c] = f.l;
          }
        } else {
          ss_atomic3(qT, qstride, node, Y0.h, Y0.l);
        }
      }
      // far row k-1 complete (for this warp's sources): one atomic per component
      if (fv && kp >= 0) ss_atomic3(qT, qstride, Lf * G.nz + kp, F0.h, F0.l);
      Y0 = Y1; Y1 = Y2;
      F0 = F1; F1 = F2;
      { const int t = pm; pm = p0; p0 = pp; pp = t; }
#pragma unroll
      for (int c = 0; c < 3; ++c) { Y2.h[c] = Y2.l[c] = F2.h[c] = F2.l[c] = 0.f; }
      __syncwarp();   // window slots of position k-1 are overwritten by the next step's load
    }
    if (fault) break;
    // chunk end: row k1-1 is this chunk's (plain store), row k1 (next chunk) gets this chunk's part
    if (lv) {
      const int64_t node = L * G.nz + (k1 - 1);
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const df2 f = df_fast(Y0.h[c], Y0.l[c]);
        yh[3 * node + c] = f.h;
        yl[3 * node + c] = f.l;
      }
      if (k1 < G.nz) ss_atomic3(qT, qstride, L * G.nz + k1, Y1.h, Y1.l);
    }
    if (fv) {
      ss_atomic3(qT, qstride, Lf * G.nz + (k1 - 1), F0.h, F0.l);
      if (k1 < G.nz) ss_atomic3(qT, qstride, Lf * G.nz + k1, F1.h, F1.l);
    }
  }
  if (fault) {
    for (int j = 0; j < inflight; ++j) {
      (void)mbar_wait(bars + stage, (parity >> stage) & 1u);
      parity ^= 1u << stage;
      stage = stage + 1 == SS_STAGES ? 0 : stage + 1;
    }
    if (lane == 0) {
      atomicExch(&C->fault, 1);
      atomicExch(&C->done, 1);
    }
  }
  df2 dv[1] = {df2{ds, de}};
  reduce_and_finalize_df<1>(dv, C, op, partials, C->ticket, &C->d0);
}

}  // namespace fem
