// Reference-element tables (shape values, reference gradients, quadrature),
// built on the host in double precision and passed to kernels by value.
//
// Reference cells follow basix (jax_fem/basis.py:141-250): [0,1]^3 for the
// hexahedron, the unit simplex for the tetrahedron.  Nodes are in the mesh's
// meshio order, which is what the reference's re_order arrays
// (basis.py:52-84) map basix's tabulation onto.  Default quadrature
// (basis.py:56,83): 2x2x2 Gauss for HEX8, the symmetric 4-point rule for TET10,
// one point for TET4; faces use the same order (2x2 Gauss / 3-point triangle).
#pragma once

#include <cmath>
#include <stdint.h>

namespace fem {

constexpr int MAX_NN = 10;   // nodes per cell
constexpr int MAX_NQ = 8;    // volume quad points
constexpr int MAX_NF = 6;    // faces per cell
constexpr int MAX_NFQ = 4;   // quad points per face
constexpr int MAX_NFV = 4;   // vertices per face

struct VolTables {
  int nn, nq;
  double N[MAX_NQ][MAX_NN];
  double dN[MAX_NQ][MAX_NN][3];
  double w[MAX_NQ];
};

struct FaceTables {
  int nn, nf, nfq, nfv;
  double N[MAX_NF][MAX_NFQ][MAX_NN];
  double dN[MAX_NF][MAX_NFQ][MAX_NN][3];
  double w[MAX_NF][MAX_NFQ];
  double normal[MAX_NF][3];
  int inds[MAX_NF][MAX_NFV];   // local node indices of the face vertices
};

// HEX8 corner coordinates in meshio order.
static const int kHexV[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                                {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};

inline void hex8_eval(const double xi[3], double N[8], double dN[8][3]) {
  for (int n = 0; n < 8; ++n) {
    double f[3], df[3];
    for (int d = 0; d < 3; ++d) {
      f[d] = kHexV[n][d] ? xi[d] : 1.0 - xi[d];
      df[d] = kHexV[n][d] ? 1.0 : -1.0;
    }
    N[n] = f[0] * f[1] * f[2];
    dN[n][0] = df[0] * f[1] * f[2];
    dN[n][1] = f[0] * df[1] * f[2];
    dN[n][2] = f[0] * f[1] * df[2];
  }
}

// TET10 in meshio order: vertices 0..3 then edge midpoints
// (0,1),(1,2),(0,2),(0,3),(1,3),(2,3).
static const int kTetEdges[6][2] = {{0, 1}, {1, 2}, {0, 2}, {0, 3}, {1, 3}, {2, 3}};

inline void tet10_eval(const double xi[3], double N[10], double dN[10][3]) {
  const double L[4] = {1.0 - xi[0] - xi[1] - xi[2], xi[0], xi[1], xi[2]};
  const double dL[4][3] = {{-1, -1, -1}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
  for (int i = 0; i < 4; ++i) {
    N[i] = L[i] * (2.0 * L[i] - 1.0);
    for (int d = 0; d < 3; ++d) dN[i][d] = (4.0 * L[i] - 1.0) * dL[i][d];
  }
  for (int e = 0; e < 6; ++e) {
    const int a = kTetEdges[e][0], b = kTetEdges[e][1];
    N[4 + e] = 4.0 * L[a] * L[b];
    for (int d = 0; d < 3; ++d) dN[4 + e][d] = 4.0 * (L[b] * dL[a][d] + L[a] * dL[b][d]);
  }
}

inline void tet4_eval(const double xi[3], double N[4], double dN[4][3]) {
  const double L[4] = {1.0 - xi[0] - xi[1] - xi[2], xi[0], xi[1], xi[2]};
  const double dL[4][3] = {{-1, -1, -1}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
  for (int i = 0; i < 4; ++i) {
    N[i] = L[i];
    for (int d = 0; d < 3; ++d) dN[i][d] = dL[i][d];
  }
}

inline void eval_shape(int elem, const double xi[3], double* N, double (*dN)[3]) {
  if (elem == 1) hex8_eval(xi, N, dN);
  else if (elem == 2) tet10_eval(xi, N, dN);
  else tet4_eval(xi, N, dN);
}

inline int elem_nn(int elem) { return elem == 1 ? 8 : (elem == 2 ? 10 : (elem == 3 ? 4 : 0)); }
inline int elem_nq(int elem) { return elem == 1 ? 8 : (elem == 2 ? 4 : (elem == 3 ? 1 : 0)); }
inline int elem_nf(int elem) { return elem == 1 ? 6 : (elem == 2 || elem == 3 ? 4 : 0); }
inline int elem_nfq(int elem) { return elem == 1 ? 4 : (elem == 2 ? 3 : (elem == 3 ? 1 : 0)); }
inline int elem_nfv(int elem) { return elem == 1 ? 4 : 3; }

inline VolTables make_vol_tables(int elem) {
  VolTables t{};
  t.nn = elem_nn(elem);
  t.nq = elem_nq(elem);
  double pts[MAX_NQ][3];
  if (elem == 1) {
    const double p[2] = {0.5 - 0.5 / std::sqrt(3.0), 0.5 + 0.5 / std::sqrt(3.0)};
    int q = 0;
    for (int i = 0; i < 2; ++i)
      for (int j = 0; j < 2; ++j)
        for (int k = 0; k < 2; ++k, ++q) {
          pts[q][0] = p[i]; pts[q][1] = p[j]; pts[q][2] = p[k];
          t.w[q] = 0.125;
        }
  } else if (elem == 2) {
    const double a = 0.5854101966249685, b = 0.1381966011250105;
    const double P[4][3] = {{b, b, b}, {a, b, b}, {b, a, b}, {b, b, a}};
    for (int q = 0; q < 4; ++q) {
      for (int d = 0; d < 3; ++d) pts[q][d] = P[q][d];
      t.w[q] = 1.0 / 24.0;
    }
  } else {
    pts[0][0] = pts[0][1] = pts[0][2] = 0.25;
    t.w[0] = 1.0 / 6.0;
  }
  for (int q = 0; q < t.nq; ++q) eval_shape(elem, pts[q], t.N[q], t.dN[q]);
  return t;
}

inline FaceTables make_face_tables(int elem) {
  FaceTables t{};
  t.nn = elem_nn(elem);
  t.nf = elem_nf(elem);
  t.nfq = elem_nfq(elem);
  t.nfv = elem_nfv(elem);
  if (elem == 1) {
    // basix hexahedron vertices (x + 2y + 4z numbering) and facets
    const double BV[8][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {1, 1, 0},
                             {0, 0, 1}, {1, 0, 1}, {0, 1, 1}, {1, 1, 1}};
    const int F[6][4] = {{0, 1, 2, 3}, {0, 1, 4, 5}, {0, 2, 4, 6}, {1, 3, 5, 7}, {2, 3, 6, 7}, {4, 5, 6, 7}};
    const double nrm[6][3] = {{0, 0, -1}, {0, -1, 0}, {-1, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    const int basix_to_meshio[8] = {0, 1, 3, 2, 4, 5, 7, 6};
    const double p[2] = {0.5 - 0.5 / std::sqrt(3.0), 0.5 + 0.5 / std::sqrt(3.0)};
    for (int f = 0; f < 6; ++f) {
      for (int v = 0; v < 4; ++v) t.inds[f][v] = basix_to_meshio[F[f][v]];
      for (int d = 0; d < 3; ++d) t.normal[f][d] = nrm[f][d];
      int q = 0;
      for (int i = 0; i < 2; ++i)
        for (int j = 0; j < 2; ++j, ++q) {
          const double s = p[i], u = p[j];
          const double c[4] = {(1 - s) * (1 - u), s * (1 - u), (1 - s) * u, s * u};
          double xi[3] = {0, 0, 0};
          for (int v = 0; v < 4; ++v)
            for (int d = 0; d < 3; ++d) xi[d] += c[v] * BV[F[f][v]][d];
          eval_shape(elem, xi, t.N[f][q], t.dN[f][q]);
          t.w[f][q] = 0.25;  // facet Jacobian of a unit square face is 1
        }
    }
  } else {
    const double V[4][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    const int F[4][3] = {{1, 2, 3}, {0, 2, 3}, {0, 1, 3}, {0, 1, 2}};
    const double r3 = 1.0 / std::sqrt(3.0);
    const double nrm[4][3] = {{r3, r3, r3}, {-1, 0, 0}, {0, -1, 0}, {0, 0, -1}};
    double P2[3][2];
    double w2[3];
    if (t.nfq == 3) {
      const double P[3][2] = {{1.0 / 6, 1.0 / 6}, {2.0 / 3, 1.0 / 6}, {1.0 / 6, 2.0 / 3}};
      for (int q = 0; q < 3; ++q) { P2[q][0] = P[q][0]; P2[q][1] = P[q][1]; w2[q] = 1.0 / 6.0; }
    } else {
      P2[0][0] = P2[0][1] = 1.0 / 3.0;
      w2[0] = 0.5;
    }
    for (int f = 0; f < 4; ++f) {
      for (int v = 0; v < 3; ++v) t.inds[f][v] = F[f][v];
      for (int d = 0; d < 3; ++d) t.normal[f][d] = nrm[f][d];
      double e1[3], e2[3];
      for (int d = 0; d < 3; ++d) { e1[d] = V[F[f][1]][d] - V[F[f][0]][d]; e2[d] = V[F[f][2]][d] - V[F[f][0]][d]; }
      const double cx = e1[1] * e2[2] - e1[2] * e2[1], cy = e1[2] * e2[0] - e1[0] * e2[2],
                   cz = e1[0] * e2[1] - e1[1] * e2[0];
      const double area = std::sqrt(cx * cx + cy * cy + cz * cz);
      for (int q = 0; q < t.nfq; ++q) {
        const double c[3] = {1 - P2[q][0] - P2[q][1], P2[q][0], P2[q][1]};
        double xi[3] = {0, 0, 0};
        for (int v = 0; v < 3; ++v)
          for (int d = 0; d < 3; ++d) xi[d] += c[v] * V[F[f][v]][d];
        eval_shape(elem, xi, t.N[f][q], t.dN[f][q]);
        t.w[f][q] = w2[q] * area;
      }
    }
  }
  return t;
}

// ---- small dense helpers (device) -------------------------------------------
template <typename T>
__device__ __forceinline__ T det3(const T J[3][3]) {
  return J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) -
         J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
         J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
}

// inverse of a 3x3 matrix given its determinant
template <typename T>
__device__ __forceinline__ void inv3(const T J[3][3], T det, T Ji[3][3]) {
  const T r = T(1) / det;
  Ji[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) * r;
  Ji[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) * r;
  Ji[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * r;
  Ji[1][0] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) * r;
  Ji[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * r;
  Ji[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * r;
  Ji[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) * r;
  Ji[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) * r;
  Ji[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * r;
}

}  // namespace fem
