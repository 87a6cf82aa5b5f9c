// Per-cell weak-form kernel: residual, consistent tangent (CSR values) and
// tangent action, evaluated at quadrature points and scattered into global
// arrays.  Restates the per-cell work of jax_fem/problem.py:189-303
// (laplace kernel + jacfwd tangent) and the scatter :426-437 / PETSc
// setValuesCOO (jax_fem/solver.py:525) as one fused pass.
//
// One CTA processes CPB cells per tile (grid-stride over tiles):
//   A  load connectivity, cell-local coordinates (x - x_node0, in FP64, then T),
//      nodal u (and w) into shared memory                 (thread per cell node)
//   B  geometry at each quadrature point: J, det, J^-1, physical shape grads,
//      JxW; material stress/tangent pre-scaled by JxW    (thread per cell qp)
//   C  element matrix and atomic scatter into the CSR value slots given by the
//      per-cell slot table: isotropic materials one 3x3 node-pair block a <= b
//      and its transpose per item (item per cell node pair); otherwise rows
//      K[(a,i),:]                                          (thread per cell row)
//   D  element residual / tangent action rows, pre-reduced across the warp
//      (lanes hitting the same dof are summed first), then FP64 atomics.
#pragma once

#include "fem_common.cuh"
#include "fem_df.cuh"
#include "fem_elements.cuh"
#include "fem_materials.cuh"

namespace fem {

struct AsmParams {
  VolTables tab;
  MatConsts mc;
  const double* coords;
  const int32_t* conn;
  const double* grads;    // optional cached (n_cells, NQ, NN, 3) physical shape gradients
  const double* jxw;      // and (n_cells, NQ) JxW (fem_cell_geometry); NULL: recomputed
  int64_t n_cells;
  const double* u;
  const double* w;
  const double* qp_params;
  int n_qp;
  const double* hist;
  const int64_t* indptr;
  const uint8_t* slots;
  const uint8_t* bc;
  int bc_mode;
  int outputs;            // FEM_OUT_* bits handled by this launch
  double* res;
  void* vals;
  double* apply_out;
  double* vjp_out;        // fem_param_vjp
  double* hist_out;       // fem_j2_update; fem_j2_history_vjp: history cotangent (C, Q, 18)
  const double* hist_bar; // fem_j2_history_vjp update mode: cotangents of (sigma_new, eps_new)
};

enum { KMODE_ASSEMBLE = 0, KMODE_VJP = 1, KMODE_HIST = 2, KMODE_HVJP = 3 };

template <int NN, int VEC>
struct Cpb {
  static constexpr int value = (192 / (NN * VEC)) > 0 ? (192 / (NN * VEC)) : 1;
};

template <int NN, int NQ, int VEC, int MAT, typename T>
struct AsmLayout {
  static constexpr int CPB = Cpb<NN, VEC>::value;
  static constexpr int THREADS = ((CPB * NN * VEC + 31) / 32) * 32;   // full warps
  static constexpr int NTAN = MatTraits<MAT, VEC>::NTAN;
  static constexpr int NS = VEC * 3;
  // offsets in elements of T
  static constexpr int oN = 0;
  static constexpr int odN = oN + NQ * NN;
  static constexpr int oX = odN + NQ * NN * 3;
  static constexpr int oU = oX + CPB * NN * 3;
  static constexpr int oW = oU + CPB * NN * VEC;
  static constexpr int oG = oW + CPB * NN * VEC;
  static constexpr int oS = oG + CPB * NQ * NN * 3;
  static constexpr int oTan = oS + CPB * NQ * NS;
  static constexpr int nT = oTan + CPB * NQ * NTAN;
  static constexpr size_t bytes = sizeof(T) * (size_t)nT + sizeof(int) * CPB * NN + sizeof(double) * THREADS + 16;
};

// Geometry at one quadrature point from cell-local node coordinates X (x_a - x_0, NN x 3) and the
// reference gradients dN (NN x 3) at that point: J = sum_a X_a (x) dN_a, physical gradients
// G_a = dN_a J^-1 (NN x 3), JxW = det J w.  One routine for the cell kernels and for the cached
// geometry (fem_cell_geometry), so both give the same bits.
template <int NN, typename T>
__device__ __forceinline__ void qp_geometry(const T* X, const T* dN, T w, T* G, T& jxw) {
  T J[3][3] = {};
  for (int n = 0; n < NN; ++n)
    for (int d = 0; d < 3; ++d) {
      const T x = X[n * 3 + d];
      for (int r = 0; r < 3; ++r) J[d][r] += x * dN[n * 3 + r];
    }
  const T det = det3<T>(J);
  T Ji[3][3];
  inv3<T>(J, det, Ji);
  jxw = det * w;
  for (int n = 0; n < NN; ++n) {
    const T* dn = dN + n * 3;
    for (int d = 0; d < 3; ++d) G[n * 3 + d] = dn[0] * Ji[0][d] + dn[1] * Ji[1][d] + dn[2] * Ji[2][d];
  }
}

template <int NN, int NQ, int VEC, int MAT, typename T, int KMODE>
__global__ void __launch_bounds__(AsmLayout<NN, NQ, VEC, MAT, T>::THREADS)
cell_kernel(const AsmParams P) {
  using L = AsmLayout<NN, NQ, VEC, MAT, T>;
  using Mat = Material<MAT, VEC, T>;
  constexpr int CPB = L::CPB, NS = L::NS, NTAN = L::NTAN;
  constexpr int TAN = MatTraits<MAT, VEC>::TAN;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* sm = reinterpret_cast<T*>(smem_raw);
  T* sN = sm + L::oN;
  T* sdN = sm + L::odN;
  T* sX = sm + L::oX;
  T* sU = sm + L::oU;
  T* sW = sm + L::oW;
  T* sG = sm + L::oG;
  T* sS = sm + L::oS;
  T* sTan = sm + L::oTan;
  int* sConn = reinterpret_cast<int*>(sm + L::nT);
  double* sRed = reinterpret_cast<double*>(
      (reinterpret_cast<uintptr_t>(sConn + CPB * NN) + 15) & ~uintptr_t(15));

  const int tid = threadIdx.x;
  for (int k = tid; k < NQ * NN; k += blockDim.x) {
    const int q = k / NN, n = k % NN;
    sN[k] = T(P.tab.N[q][n]);
    for (int d = 0; d < 3; ++d) sdN[k * 3 + d] = T(P.tab.dN[q][n][d]);
  }

  const bool cached = P.grads != nullptr;   // geometry from fem_cell_geometry
  const bool want_res = (KMODE == KMODE_ASSEMBLE) && (P.outputs & FEM_OUT_RESIDUAL);
  const bool want_mat = (KMODE == KMODE_ASSEMBLE) && (P.outputs & FEM_OUT_MATRIX);
  const bool want_app = (KMODE == KMODE_ASSEMBLE) && (P.outputs & FEM_OUT_APPLY);
  const bool need_w = want_app || KMODE == KMODE_VJP || (KMODE == KMODE_HVJP && P.w != nullptr);
  // history VJP in update mode scatters the cotangent of u (residual-style) into P.res
  const bool want_ubar = (KMODE == KMODE_HVJP) && (P.res != nullptr);

  const int64_t n_tiles = (P.n_cells + CPB - 1) / CPB;
  for (int64_t tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
    __syncthreads();
    // ---- A: gather -------------------------------------------------------
    for (int k = tid; k < CPB * NN; k += blockDim.x) {
      const int c = k / NN, n = k % NN;
      const int64_t e = tile * CPB + c;
      int node = -1;
      if (e < P.n_cells) node = P.conn[e * NN + n];
      sConn[k] = node;
      if (node >= 0) {
        if (!cached) {
          const int n0 = P.conn[e * NN];
          for (int d = 0; d < 3; ++d)
            sX[k * 3 + d] = T(P.coords[(int64_t)node * 3 + d] - P.coords[(int64_t)n0 * 3 + d]);
        }
        for (int v = 0; v < VEC; ++v) {
          const int64_t dof = (int64_t)node * VEC + v;
          sU[k * VEC + v] = P.u ? T(P.u[dof]) : T(0);
          if (need_w) {
            T wv = T(P.w[dof]);
            // VJP: multiplier masked on Dirichlet dofs; APPLY with FEM_BC_SYMMETRIC: K_ff w_f
            if (P.bc && P.bc[dof] && (KMODE == KMODE_VJP || KMODE == KMODE_HVJP || P.bc_mode == FEM_BC_SYMMETRIC))
              wv = T(0);
            sW[k * VEC + v] = wv;
          }
        }
      } else {
        for (int d = 0; d < 3; ++d) sX[k * 3 + d] = T(0);
        for (int v = 0; v < VEC; ++v) { sU[k * VEC + v] = T(0); if (need_w) sW[k * VEC + v] = T(0); }
      }
    }
    if (cached) {   // the tile's cached shape gradients, one contiguous run
      constexpr int GT = CPB * NQ * NN * 3;
      const int64_t avail = (P.n_cells - tile * CPB) * (NQ * NN * 3);
      const double* src = P.grads + tile * (int64_t)GT;
      for (int k = tid; k < GT; k += blockDim.x) sG[k] = k < avail ? T(src[k]) : T(0);
    }
    __syncthreads();
    // ---- B: geometry + material at quadrature points ----------------------
    for (int k = tid; k < CPB * NQ; k += blockDim.x) {
      const int c = k / NQ, q = k % NQ;
      const int64_t e = tile * CPB + c;
      if (e >= P.n_cells) continue;
      T* G = sG + (c * NQ + q) * NN * 3;
      T jxw;
      if (cached) jxw = T(P.jxw[e * NQ + q]);
      else qp_geometry<NN, T>(sX + c * NN * 3, sdN + q * NN * 3, T(P.tab.w[q]), G, jxw);
      T gu[NS];
      T gw[NS];
      for (int s = 0; s < NS; ++s) { gu[s] = T(0); gw[s] = T(0); }
      for (int n = 0; n < NN; ++n) {
        const T g[3] = {G[n * 3], G[n * 3 + 1], G[n * 3 + 2]};
        for (int v = 0; v < VEC; ++v) {
          const T un = sU[(c * NN + n) * VEC + v];
          for (int d = 0; d < 3; ++d) gu[v * 3 + d] += un * g[d];
          if (need_w) {
            const T wn = sW[(c * NN + n) * VEC + v];
            for (int d = 0; d < 3; ++d) gw[v * 3 + d] += wn * g[d];
          }
        }
      }
      const double* qp = P.qp_params ? P.qp_params + (e * NQ + q) * P.n_qp : nullptr;
      const double* hs = P.hist ? P.hist + (e * NQ + q) * 18 : nullptr;
      if constexpr (KMODE == KMODE_VJP) {
        T dS[NS];
        Mat::dparam(gu, P.mc, qp, hs, dS);
        T acc = T(0);
        for (int s = 0; s < NS; ++s) acc += dS[s] * gw[s];
        P.vjp_out[(e * NQ + q) * P.n_qp] = -double(acc) * double(jxw);
        continue;
      }
      if constexpr (KMODE == KMODE_HVJP) {
        if constexpr (MAT == FEM_MAT_J2 && VEC == 3) {
          T gs[9], ge[9];
          if (P.w) {  // adjoint mode: cotangent of sigma is -jxw grad(lambda)
            for (int s = 0; s < 9; ++s) { gs[s] = -gw[s] * jxw; ge[s] = T(0); }
          } else {
            const double* hb = P.hist_bar + (e * NQ + q) * 18;
            for (int s = 0; s < 9; ++s) { gs[s] = T(hb[s]); ge[s] = T(hb[9 + s]); }
          }
          T W[9], dso[9], deo[9], dsc;
          Mat::hist_vjp(gu, P.mc, qp, hs, gs, ge, W, dso, deo, dsc);
          double* ho = P.hist_out + (e * NQ + q) * 18;
          for (int s = 0; s < 9; ++s) { ho[s] = double(dso[s]); ho[9 + s] = double(deo[s]); }
          if (P.vjp_out) P.vjp_out[e * NQ + q] = double(dsc);
          if (want_ubar) {
            T* Sq = sS + (c * NQ + q) * NS;
            for (int s = 0; s < 9; ++s) Sq[s] = W[s];
          }
        }
        continue;
      }
      if constexpr (KMODE == KMODE_HIST) {
        if constexpr (VEC == 3) {
          T S[NS];
          Mat::eval(gu, P.mc, qp, hs, S, nullptr, false);
          double* ho = P.hist_out + (e * NQ + q) * 18;
          for (int s = 0; s < 9; ++s) ho[s] = double(S[s]);
          for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) ho[9 + i * 3 + j] = 0.5 * (double(gu[i * 3 + j]) + double(gu[j * 3 + i]));
        }
        continue;
      }
      T S[NS];
      T* tq = sTan + (c * NQ + q) * NTAN;   // tangent is evaluated straight into shared memory
      const bool need_tan = want_mat || want_app;
      Mat::eval(gu, P.mc, qp, hs, S, tq, need_tan);
      T* Sq = sS + (c * NQ + q) * NS;
      if (want_app) {
        // dS = A : grad w  (tangent action), stored in place of the stress
        if constexpr (TAN == TAN_SCALAR) {
          for (int s = 0; s < NS; ++s) Sq[s] = tq[0] * gw[s] * jxw;
        } else if constexpr (TAN == TAN_ISO) {
          T dS[NS];
          iso_stress(gw, tq[0], tq[1], dS);
          for (int s = 0; s < NS; ++s) Sq[s] = dS[s] * jxw;
        } else {
          for (int I = 0; I < NS; ++I) {
            T acc = T(0);
            for (int Jx = 0; Jx < NS; ++Jx) acc += tq[I * NS + Jx] * gw[Jx];
            Sq[I] = acc * jxw;
          }
        }
      } else {
        for (int s = 0; s < NS; ++s) Sq[s] = S[s] * jxw;
      }
      if (want_mat)
        for (int s = 0; s < NTAN; ++s) tq[s] *= jxw;
    }
    if constexpr (KMODE != KMODE_ASSEMBLE && KMODE != KMODE_HVJP) continue;
    if (KMODE == KMODE_HVJP && !want_ubar) continue;
    __syncthreads();
    // ---- C / D: element rows ---------------------------------------------
    const int c = tid / (NN * VEC);
    const int r = tid % (NN * VEC);
    const int a = r / VEC, i = r % VEC;
    const int64_t e = tile * CPB + c;
    const bool active = (c < CPB) && (e < P.n_cells);
    const int na = active ? sConn[c * NN + a] : 0;
    const int64_t row = (int64_t)na * VEC + i;
    const bool row_bc = active && P.bc && P.bc[row];

    if constexpr (TAN == TAN_ISO && VEC == 3) {
      if (want_mat) {
        // K[(a,i),(b,k)] = sum_q lam g_a,i g_b,k + mu g_a,k g_b,i + mu (g_a . g_b) delta_ik.  lam / mu
        // = cr is the same at every point (only E varies), so with M_ab = sum_q mu g_a (x) g_b
        //   K_ab = cr M_ab + M_ab^T + tr(M_ab) I,   K_ba = K_ab^T:
        // one item per cell and node pair a <= b, 9 FMAs per quadrature point; the item scatters
        // block (a, b) into node a's rows and, for a != b, its transpose into node b's rows.
        constexpr int NP = NN * (NN + 1) / 2;
        const T cr = Mat::lam_over_mu(P.mc);
        T* vals = reinterpret_cast<T*>(P.vals);
        for (int t = tid; t < CPB * NP; t += blockDim.x) {
          const int cc = t / NP;
          int pp = t - cc * NP, pa = 0;
          while (pp >= NN - pa) { pp -= NN - pa; ++pa; }
          const int pb = pa + pp;
          const int64_t ee = tile * CPB + cc;
          if (ee >= P.n_cells) continue;
          T M[3][3] = {};
          for (int q = 0; q < NQ; ++q) {
            const T* G = sG + (cc * NQ + q) * NN * 3;
            const T mu = sTan[(cc * NQ + q) * NTAN + 1];
            const T m0 = mu * G[pa * 3], m1 = mu * G[pa * 3 + 1], m2 = mu * G[pa * 3 + 2];
            const T g0 = G[pb * 3], g1 = G[pb * 3 + 1], g2 = G[pb * 3 + 2];
            M[0][0] = fma(m0, g0, M[0][0]); M[0][1] = fma(m0, g1, M[0][1]); M[0][2] = fma(m0, g2, M[0][2]);
            M[1][0] = fma(m1, g0, M[1][0]); M[1][1] = fma(m1, g1, M[1][1]); M[1][2] = fma(m1, g2, M[1][2]);
            M[2][0] = fma(m2, g0, M[2][0]); M[2][1] = fma(m2, g1, M[2][1]); M[2][2] = fma(m2, g2, M[2][2]);
          }
          const T tr = M[0][0] + M[1][1] + M[2][2];
          const int64_t na2 = sConn[cc * NN + pa], nb2 = sConn[cc * NN + pb];
          const int sab = P.slots[(ee * NN + pa) * NN + pb], sba = P.slots[(ee * NN + pb) * NN + pa];
#pragma unroll
          for (int ii = 0; ii < 3; ++ii) {
            const int64_t ra = na2 * 3 + ii;
            const bool abc = P.bc && P.bc[ra];
            T* dst_a = vals + P.indptr[ra] + 3 * sab;
#pragma unroll
            for (int kk = 0; kk < 3; ++kk) {
              const int64_t rb = nb2 * 3 + kk;
              const bool bbc = P.bc && P.bc[rb];
              const T kv = fma(cr, M[ii][kk], M[kk][ii]) + (ii == kk ? tr : T(0));   // K_ab[ii][kk]
              // K[(a,ii),(b,kk)]: row ra, column rb
              if (!(abc && P.bc_mode != FEM_BC_NONE) && !(bbc && P.bc_mode == FEM_BC_SYMMETRIC))
                atomicAdd(dst_a + kk, kv);
              // K[(b,kk),(a,ii)] = K[(a,ii),(b,kk)]: row rb, column ra
              if (pa != pb && !(bbc && P.bc_mode != FEM_BC_NONE) && !(abc && P.bc_mode == FEM_BC_SYMMETRIC))
                atomicAdd(vals + P.indptr[rb] + 3 * sba + ii, kv);
            }
          }
        }
      }
    } else if (want_mat && active && !(row_bc && P.bc_mode != FEM_BC_NONE)) {
      T acc[NN][VEC];
      for (int b = 0; b < NN; ++b)
        for (int k = 0; k < VEC; ++k) acc[b][k] = T(0);
      for (int q = 0; q < NQ; ++q) {
        const T* G = sG + (c * NQ + q) * NN * 3;
        const T ga0 = G[a * 3 + 0], ga1 = G[a * 3 + 1], ga2 = G[a * 3 + 2];
        const T* tq = sTan + (c * NQ + q) * NTAN;
        if constexpr (TAN == TAN_SCALAR) {
          const T t0 = tq[0];
          for (int b = 0; b < NN; ++b)
            acc[b][0] += t0 * (ga0 * G[b * 3] + ga1 * G[b * 3 + 1] + ga2 * G[b * 3 + 2]);
        } else if constexpr (TAN == TAN_ISO) {
          const T lam = tq[0], mu = tq[1];
          const T gai = G[a * 3 + i];
          const T lgi = lam * gai;
          for (int b = 0; b < NN; ++b) {
            const T gb0 = G[b * 3], gb1 = G[b * 3 + 1], gb2 = G[b * 3 + 2];
            const T gbi = G[b * 3 + i];
            const T mdot = mu * (ga0 * gb0 + ga1 * gb1 + ga2 * gb2);
            const T mgbi = mu * gbi;
            acc[b][0] += lgi * gb0 + mgbi * ga0 + (i == 0 ? mdot : T(0));
            if constexpr (VEC == 3) {
              acc[b][1] += lgi * gb1 + mgbi * ga1 + (i == 1 ? mdot : T(0));
              acc[b][2] += lgi * gb2 + mgbi * ga2 + (i == 2 ? mdot : T(0));
            }
          }
        } else {
          // T_kl = sum_j ga_j A[(i,j),(k,l)]
          T Tk[VEC][3];
          for (int k = 0; k < VEC; ++k)
            for (int l = 0; l < 3; ++l)
              Tk[k][l] = ga0 * tq[(i * 3 + 0) * NS + k * 3 + l] + ga1 * tq[(i * 3 + 1) * NS + k * 3 + l] +
                         ga2 * tq[(i * 3 + 2) * NS + k * 3 + l];
          for (int b = 0; b < NN; ++b) {
            const T gb0 = G[b * 3], gb1 = G[b * 3 + 1], gb2 = G[b * 3 + 2];
            for (int k = 0; k < VEC; ++k) acc[b][k] += Tk[k][0] * gb0 + Tk[k][1] * gb1 + Tk[k][2] * gb2;
          }
        }
      }
      T* vals = reinterpret_cast<T*>(P.vals);
      const int64_t rs = P.indptr[row];
      const uint8_t* sl = P.slots + (e * NN + a) * NN;
      for (int b = 0; b < NN; ++b) {
        const int nb = sConn[c * NN + b];
        T* dst = vals + rs + (int64_t)VEC * sl[b];
        for (int k = 0; k < VEC; ++k) {
          if (P.bc_mode == FEM_BC_SYMMETRIC && P.bc[(int64_t)nb * VEC + k]) continue;
          atomicAdd(dst + k, acc[b][k]);
        }
      }
    }

    if (want_res || want_app || want_ubar) {
      double rv = 0.0;
      if (active) {
        T s = T(0);
        for (int q = 0; q < NQ; ++q) {
          const T* G = sG + (c * NQ + q) * NN * 3;
          const T* Sq = sS + (c * NQ + q) * NS;
          s += Sq[i * 3 + 0] * G[a * 3 + 0] + Sq[i * 3 + 1] * G[a * 3 + 1] + Sq[i * 3 + 2] * G[a * 3 + 2];
        }
        rv = double(s);
      }
      // warp-segmented pre-reduction: lanes with the same destination dof are
      // summed (in lane order) before one FP64 atomic per distinct dof
      const bool emit = active && !row_bc;
      const long long key = emit ? (long long)row : -1 - (long long)(tid & 31);
      const unsigned grp = __match_any_sync(0xffffffffu, key);
      sRed[tid] = rv;
      __syncwarp();
      const int lane = tid & 31;
      if (emit && lane == __ffs(grp) - 1) {
        double sum = 0.0;
        for (unsigned m = grp; m; m &= m - 1) sum += sRed[(tid & ~31) + __ffs(m) - 1];
        atomicAdd((want_res || want_ubar) ? (P.res + row) : (P.apply_out + row), sum);
      }
      __syncwarp();
    }
  }
}

// ---- isotropic tangent in double-float (FEM_DF48 matrix assembly) ----------------------------
// The matrix of the linear isotropic laws (linear elastic, SIMP) for the DF48 solver copies, with
// the node-pair form of cell_kernel (K_ab = cr M_ab + M_ab^T + tr(M_ab) I, M_ab = sum_q mu_q JxW_q
// g_qa (x) g_qb, cr = lam / mu the same at every point) evaluated in double-float arithmetic on
// the FP32 pipes: GB300's FP64 pipe (~1/64 of FP32) bounds the FP64 form.  Reads the cached
// geometry (fem_cell_geometry).  Per tile of CPB cells:
//   1  mu_q JxW_q per (cell, qp) in FP64 (the material law, a few flops) and the connectivity;
//   2  the cell's shape gradients and mu JxW g as double-float pairs in shared memory (FP64 ->
//      pair from the bits: integer operations);
//   3  one thread per (cell, node pair a <= b): 9 double-float product-accumulates per qp, then
//      K_ab, each value rounded once to FP64 (one FP64 add) and scattered with FP64 atomics
//      into block (a, b) and, for a != b, its transpose (Dirichlet rules of cell_kernel).
// The values carry ~2^-46 relative rounding against FP64's 2^-53: far below the 2^-40 of the DF48
// copy made from them.
constexpr int DFM_THREADS = 288;
template <int NN>
struct DfmLayout {
  static constexpr int NP = NN * (NN + 1) / 2;
  static constexpr int CPB = DFM_THREADS / NP > 0 ? DFM_THREADS / NP : 1;
};

template <int NN, int NQ, int MAT>
__global__ void __launch_bounds__(DFM_THREADS, 4) cell_matrix_df_kernel(const AsmParams P) {
  using Mat = Material<MAT, 3, double>;
  constexpr int NP = DfmLayout<NN>::NP, CPB = DfmLayout<NN>::CPB, GQ = NN * 3;
  __shared__ float2 sg[CPB * NQ * GQ];   // g_qa (double-float)
  __shared__ float2 sm[CPB * NQ * GQ];   // mu_q JxW_q g_qa (double-float)
  __shared__ float2 smu[CPB * NQ];       // mu_q JxW_q (double-float)
  __shared__ int sconn[CPB * NN];
  const int tid = threadIdx.x;
  const df2 cr = df_from_bits(Mat::lam_over_mu(P.mc));
  double* vals = reinterpret_cast<double*>(P.vals);
  const int64_t n_tiles = (P.n_cells + CPB - 1) / CPB;
  for (int64_t tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
    __syncthreads();
    for (int k = tid; k < CPB * NQ; k += blockDim.x) {
      const int64_t e = tile * CPB + k / NQ;
      double smq = 0.0;
      if (e < P.n_cells) {
        const int q = k % NQ;
        const double* qp = P.qp_params ? P.qp_params + (e * NQ + q) * P.n_qp : nullptr;
        const double g0[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        double S[9], tan[2];
        Mat::eval(g0, P.mc, qp, nullptr, S, tan, true);
        smq = tan[1] * P.jxw[e * NQ + q];
      }
      const df2 sd = df_from_bits(smq);
      smu[k] = make_float2(sd.h, sd.l);
    }
    for (int k = tid; k < CPB * NN; k += blockDim.x) {
      const int64_t e = tile * CPB + k / NN;
      sconn[k] = e < P.n_cells ? P.conn[e * NN + k % NN] : -1;
    }
    __syncthreads();
    {
      constexpr int GT = CPB * NQ * GQ;
      const int64_t avail = (P.n_cells - tile * CPB) * (NQ * GQ);
      const double* src = P.grads + tile * (int64_t)GT;
      for (int k = tid; k < GT; k += blockDim.x) {
        const double g = k < avail ? src[k] : 0.0;
        const df2 gd = df_from_bits(g);
        const float2 mu = smu[k / GQ];
        const df2 md = df_mul(df2{mu.x, mu.y}, gd);
        sg[k] = make_float2(gd.h, gd.l);
        sm[k] = make_float2(md.h, md.l);
      }
    }
    __syncthreads();
    for (int t = tid; t < CPB * NP; t += blockDim.x) {
      const int cc = t / NP;
      int pp = t - cc * NP, pa = 0;
      while (pp >= NN - pa) { pp -= NN - pa; ++pa; }
      const int pb = pa + pp;
      const int64_t ee = tile * CPB + cc;
      if (ee >= P.n_cells) continue;
      // M accumulates on the paired FP32 instructions (df_acc2): rows i of columns (0, 1) as three
      // pairs, (M02, M12) as a fourth, M22 alone -- 4 paired + 1 scalar product-accumulates per qp
      float2 ah[3], al[3], bh = make_float2(0.f, 0.f), bl = bh;
      float ch = 0.f, cl = 0.f;
#pragma unroll
      for (int i = 0; i < 3; ++i) ah[i] = al[i] = make_float2(0.f, 0.f);
#pragma unroll 2
      for (int q = 0; q < NQ; ++q) {
        const float2* ma = sm + (cc * NQ + q) * GQ + pa * 3;
        const float2* gb = sg + (cc * NQ + q) * GQ + pb * 3;
        const float2 m0 = ma[0], m1 = ma[1], m2 = ma[2], g0 = gb[0], g1 = gb[1], g2 = gb[2];
        const float2 gh01 = make_float2(g0.x, g1.x), ngh01 = make_float2(-g0.x, -g1.x), gl01 = make_float2(g0.y, g1.y);
        const float2 mrow[3] = {m0, m1, m2};
#pragma unroll
        for (int i = 0; i < 3; ++i)
          df_acc2(ah[i], al[i], make_float2(mrow[i].x, mrow[i].x), make_float2(mrow[i].y, mrow[i].y), gh01, ngh01,
                  gl01);
        df_acc2(bh, bl, make_float2(m0.x, m1.x), make_float2(m0.y, m1.y), make_float2(g2.x, g2.x),
                make_float2(-g2.x, -g2.x), make_float2(g2.y, g2.y));
        df_acc(ch, cl, df2{m2.x, m2.y}, df2{g2.x, g2.y});
      }
      df2 M[9];
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        M[i * 3 + 0] = df_fast(ah[i].x, al[i].x);
        M[i * 3 + 1] = df_fast(ah[i].y, al[i].y);
      }
      M[2] = df_fast(bh.x, bl.x);
      M[5] = df_fast(bh.y, bl.y);
      M[8] = df_fast(ch, cl);
      const df2 tr = df_add(df_add(M[0], M[4]), M[8]);
      const int64_t na2 = sconn[cc * NN + pa], nb2 = sconn[cc * NN + pb];
      const int sab = P.slots[(ee * NN + pa) * NN + pb], sba = P.slots[(ee * NN + pb) * NN + pa];
      // row pointers and Dirichlet flags of the pair's six rows, read once (byte pointers may
      // alias the values, so they would be re-read after every atomic otherwise)
      double* dst_a[3];
      double* dst_b[3];
      bool abc[3], bbc[3];
#pragma unroll
      for (int r = 0; r < 3; ++r) {
        dst_a[r] = vals + P.indptr[na2 * 3 + r] + 3 * sab;
        dst_b[r] = vals + P.indptr[nb2 * 3 + r] + 3 * sba;
        abc[r] = P.bc && P.bc[na2 * 3 + r];
        bbc[r] = P.bc && P.bc[nb2 * 3 + r];
      }
      const bool keep_rows = P.bc_mode == FEM_BC_NONE, sym = P.bc_mode == FEM_BC_SYMMETRIC;
#pragma unroll
      for (int ii = 0; ii < 3; ++ii) {
#pragma unroll
        for (int kk = 0; kk < 3; ++kk) {
          df2 kv = df_add(df_mul(cr, M[ii * 3 + kk]), M[kk * 3 + ii]);   // K_ab[ii][kk]
          if (ii == kk) kv = df_add(kv, tr);
          const double kd = f2d_bits(kv.h) + f2d_bits(kv.l);
          // K[(a,ii),(b,kk)]: row of a, column of b; K[(b,kk),(a,ii)]: its transpose
          if (!(abc[ii] && !keep_rows) && !(bbc[kk] && sym)) atomicAdd(dst_a[ii] + kk, kd);
          if (pa != pb && !(bbc[kk] && !keep_rows) && !(abc[ii] && sym)) atomicAdd(dst_b[kk] + ii, kd);
        }
      }
    }
  }
}

template <int NN, int NQ, int MAT>
int launch_cell_matrix_df(const AsmParams& P, cudaStream_t stream) {
  using L = DfmLayout<NN>;
  auto kern = cell_matrix_df_kernel<NN, NQ, MAT>;
  const int64_t tiles = (P.n_cells + L::CPB - 1) / L::CPB;
  int blocks_per_sm = 1;
  FEM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm, kern, DFM_THREADS, 0));
  if (blocks_per_sm < 1) blocks_per_sm = 1;
  int64_t grid = (int64_t)sm_count() * blocks_per_sm;
  if (grid > tiles) grid = tiles;
  if (grid < 1) grid = 1;
  kern<<<(unsigned)grid, DFM_THREADS, 0, stream>>>(P);
  note_launches(1);
  return check_launch("cell_matrix_df_kernel");
}

// Host-side launcher for one (element, vec, material, precision, mode).
template <int NN, int NQ, int VEC, int MAT, typename T, int KMODE>
int launch_cell_kernel(const AsmParams& P, cudaStream_t stream) {
  using L = AsmLayout<NN, NQ, VEC, MAT, T>;
  auto kern = cell_kernel<NN, NQ, VEC, MAT, T, KMODE>;
  const size_t smem = L::bytes;
  if (smem > 48 * 1024) FEM_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int64_t tiles = (P.n_cells + L::CPB - 1) / L::CPB;
  int blocks_per_sm = 1;
  FEM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm, kern, L::THREADS, smem));
  if (blocks_per_sm < 1) blocks_per_sm = 1;
  int64_t grid = (int64_t)sm_count() * blocks_per_sm;
  if (grid > tiles) grid = tiles;
  if (grid < 1) grid = 1;
  kern<<<(unsigned)grid, L::THREADS, smem, stream>>>(P);
  note_launches(1);
  return check_launch("cell_kernel");
}

template <int NN, int NQ, int VEC, int MAT>
int dispatch_precision(const AsmParams& P, int precision, int kmode, cudaStream_t s) {
  if (kmode == KMODE_VJP) return launch_cell_kernel<NN, NQ, VEC, MAT, double, KMODE_VJP>(P, s);
  if (kmode == KMODE_HIST) return launch_cell_kernel<NN, NQ, VEC, MAT, double, KMODE_HIST>(P, s);
  if (kmode == KMODE_HVJP) {
    if constexpr (MAT == FEM_MAT_J2 && VEC == 3) return launch_cell_kernel<NN, NQ, VEC, MAT, double, KMODE_HVJP>(P, s);
    return fail(FEM_ERR_UNSUPPORTED, "history VJP is defined for J2 only");
  }
  if (precision == FEM_F32) return launch_cell_kernel<NN, NQ, VEC, MAT, float, KMODE_ASSEMBLE>(P, s);
  if (precision == FEM_DF48) {
    // double-float matrix for the isotropic laws with cached geometry; FP64 otherwise
    if constexpr (VEC == 3 && MatTraits<MAT, VEC>::TAN == TAN_ISO)
      if (P.grads && P.outputs == FEM_OUT_MATRIX) return launch_cell_matrix_df<NN, NQ, MAT>(P, s);
  }
  return launch_cell_kernel<NN, NQ, VEC, MAT, double, KMODE_ASSEMBLE>(P, s);
}

template <int NN, int NQ>
int dispatch_material(const AsmParams& P, int vec, int mat, int precision, int kmode, cudaStream_t s) {
  if (vec == 1) {
    if (mat == FEM_MAT_LAPLACE) return dispatch_precision<NN, NQ, 1, FEM_MAT_LAPLACE>(P, precision, kmode, s);
    if (mat == FEM_MAT_GENERAL_LINEAR) return dispatch_precision<NN, NQ, 1, FEM_MAT_GENERAL_LINEAR>(P, precision, kmode, s);
  } else if (vec == 3) {
    switch (mat) {
      case FEM_MAT_LINEAR_ELASTIC: return dispatch_precision<NN, NQ, 3, FEM_MAT_LINEAR_ELASTIC>(P, precision, kmode, s);
      case FEM_MAT_SIMP: return dispatch_precision<NN, NQ, 3, FEM_MAT_SIMP>(P, precision, kmode, s);
      case FEM_MAT_GENERAL_LINEAR: return dispatch_precision<NN, NQ, 3, FEM_MAT_GENERAL_LINEAR>(P, precision, kmode, s);
      case FEM_MAT_NEO_HOOKEAN: return dispatch_precision<NN, NQ, 3, FEM_MAT_NEO_HOOKEAN>(P, precision, kmode, s);
      case FEM_MAT_J2: return dispatch_precision<NN, NQ, 3, FEM_MAT_J2>(P, precision, kmode, s);
      default: break;
    }
  }
  return fail(FEM_ERR_UNSUPPORTED, "material/vec combination not supported");
}

// per-element-type entry points (one translation unit each, compiled in parallel)
int assemble_hex8(const AsmParams& P, int vec, int mat, int precision, int kmode, cudaStream_t s);
int assemble_tet10(const AsmParams& P, int vec, int mat, int precision, int kmode, cudaStream_t s);
int assemble_tet4(const AsmParams& P, int vec, int mat, int precision, int kmode, cudaStream_t s);

}  // namespace fem
