// C ABI for geometry, loads, assembly, parameter VJP and J2 history update.
#include <cstring>

#include "fem_assemble.cuh"

namespace fem {

static int run_cell_kernel(const fem_mesh_t* mesh, const AsmParams& P, int mat, int precision, int kmode,
                           cudaStream_t s) {
  switch (mesh->elem_type) {
    case FEM_HEX8: return assemble_hex8(P, mesh->vec, mat, precision, kmode, s);
    case FEM_TET10: return assemble_tet10(P, mesh->vec, mat, precision, kmode, s);
    case FEM_TET4: return assemble_tet4(P, mesh->vec, mat, precision, kmode, s);
    default: return fail(FEM_ERR_UNSUPPORTED, "unknown element type");
  }
}

static int check_mesh(const fem_mesh_t* mesh) {
  FEM_REQUIRE(mesh != nullptr, "mesh is NULL");
  FEM_REQUIRE(elem_nn(mesh->elem_type) > 0, "unknown element type");
  FEM_REQUIRE(mesh->vec == 1 || mesh->vec == 3, "vec must be 1 or 3");
  FEM_REQUIRE(mesh->n_cells >= 0 && mesh->n_nodes >= 0, "negative sizes");
  FEM_REQUIRE(mesh->n_cells == 0 || (mesh->coords && mesh->conn), "coords/conn NULL");
  FEM_REQUIRE(mesh->n_nodes < (int64_t(1) << 31) / 3, "too many nodes for 32-bit dof indices in blocks");
  return FEM_OK;
}

static int fill_params(const fem_mesh_t* mesh, const fem_material_t* mat, AsmParams& P) {
  std::memset(&P, 0, sizeof(P));
  P.tab = make_vol_tables(mesh->elem_type);
  P.coords = mesh->coords;
  P.conn = mesh->conn;
  FEM_REQUIRE((mesh->shape_grads == nullptr) == (mesh->jxw == nullptr), "set both or neither of shape_grads / jxw");
  P.grads = mesh->shape_grads;
  P.jxw = mesh->jxw;
  P.n_cells = mesh->n_cells;
  if (mat) {
    FEM_REQUIRE(mat->n_consts >= 0 && mat->n_consts <= 96, "n_consts must be in [0, 96]");
    FEM_REQUIRE(mat->n_consts == 0 || mat->consts, "consts NULL");
    for (int k = 0; k < mat->n_consts; ++k) P.mc.c[k] = mat->consts[k];
    P.mc.n = mat->n_consts;
    P.mc.clamp = (mat->kind == FEM_MAT_NEO_HOOKEAN && mat->n_consts > 2 && mat->consts[2] != 0.0) ? 1 : 0;
    P.qp_params = mat->qp_params;
    P.n_qp = mat->n_qp_params;
    P.hist = mat->history;
    const int need_qp = (mat->kind == FEM_MAT_SIMP) ? 1 : 0;
    FEM_REQUIRE(!need_qp || (mat->qp_params && mat->n_qp_params == 1), "SIMP needs one qp parameter (theta)");
    FEM_REQUIRE(mat->n_qp_params == 0 || mat->n_qp_params == 1, "n_qp_params must be 0 or 1");
    FEM_REQUIRE(mat->n_qp_params == 0 || mat->qp_params, "qp_params NULL");
    const int need_c[7] = {0, 1, 2, 4, 0, 2, 3};
    if (mat->kind >= 1 && mat->kind <= 6) {
      if (mat->kind == FEM_MAT_GENERAL_LINEAR) {
        const int m = mesh->vec * 3;
        FEM_REQUIRE(mat->n_consts == m * m, "GENERAL_LINEAR needs (vec*3)^2 constants");
      } else {
        FEM_REQUIRE(mat->n_consts >= need_c[mat->kind], "too few material constants");
      }
    }
  }
  return FEM_OK;
}

// ---- geometry / load kernels (FP64, setup-time) ------------------------------
__global__ void quad_points_kernel(VolTables tab, const double* coords, const int32_t* conn, int64_t n_cells,
                                   double* x_out, double* jxw_out) {
  const int NN = tab.nn, NQ = tab.nq;
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n_cells * NQ;
       k += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = k / NQ;
    const int q = (int)(k % NQ);
    double J[3][3] = {}, x[3] = {0, 0, 0};
    for (int n = 0; n < NN; ++n) {
      const int node = conn[e * NN + n];
      for (int d = 0; d < 3; ++d) {
        const double X = coords[(int64_t)node * 3 + d];
        x[d] += tab.N[q][n] * X;
        for (int r = 0; r < 3; ++r) J[d][r] += X * tab.dN[q][n][r];
      }
    }
    if (x_out)
      for (int d = 0; d < 3; ++d) x_out[k * 3 + d] = x[d];
    if (jxw_out) jxw_out[k] = det3<double>(J) * tab.w[q];
  }
}

__global__ void face_points_kernel(FaceTables ft, const double* coords, const int32_t* conn,
                                   const int32_t* face_cells, const int32_t* face_ids, int64_t n_faces,
                                   double* x_out, double* nanson_out) {
  const int NN = ft.nn, NFQ = ft.nfq;
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n_faces * NFQ;
       k += (int64_t)gridDim.x * blockDim.x) {
    const int64_t f = k / NFQ;
    const int q = (int)(k % NFQ);
    const int64_t e = face_cells[f];
    const int fid = face_ids[f];
    double J[3][3] = {}, x[3] = {0, 0, 0};
    for (int n = 0; n < NN; ++n) {
      const int node = conn[e * NN + n];
      for (int d = 0; d < 3; ++d) {
        const double X = coords[(int64_t)node * 3 + d];
        x[d] += ft.N[fid][q][n] * X;
        for (int r = 0; r < 3; ++r) J[d][r] += X * ft.dN[fid][q][n][r];
      }
    }
    if (x_out)
      for (int d = 0; d < 3; ++d) x_out[k * 3 + d] = x[d];
    if (nanson_out) {
      const double det = det3<double>(J);
      double Ji[3][3];
      inv3<double>(J, det, Ji);
      double v[3];
      for (int d = 0; d < 3; ++d)
        v[d] = ft.normal[fid][0] * Ji[0][d] + ft.normal[fid][1] * Ji[1][d] + ft.normal[fid][2] * Ji[2][d];
      nanson_out[k] = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]) * det * ft.w[fid][q];
    }
  }
}

// out[dof(a,v)] += sum_q f[e,q,v] N_a(q) JxW(q): thread per (cell, node)
__global__ void body_load_kernel(VolTables tab, int vec, const double* coords, const int32_t* conn, int64_t n_cells,
                                 const double* f_qp, double* out) {
  const int NN = tab.nn, NQ = tab.nq;
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n_cells * NN;
       k += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = k / NN;
    const int a = (int)(k % NN);
    double acc[3] = {0, 0, 0};
    for (int q = 0; q < NQ; ++q) {
      double J[3][3] = {};
      for (int n = 0; n < NN; ++n) {
        const int node = conn[e * NN + n];
        for (int d = 0; d < 3; ++d) {
          const double X = coords[(int64_t)node * 3 + d];
          for (int r = 0; r < 3; ++r) J[d][r] += X * tab.dN[q][n][r];
        }
      }
      const double s = tab.N[q][a] * det3<double>(J) * tab.w[q];
      for (int v = 0; v < vec; ++v) acc[v] += f_qp[(e * NQ + q) * vec + v] * s;
    }
    const int node = conn[e * NN + a];
    for (int v = 0; v < vec; ++v) atomicAdd(out + (int64_t)node * vec + v, acc[v]);
  }
}

__global__ void surface_load_kernel(FaceTables ft, int vec, const double* coords, const int32_t* conn,
                                    const int32_t* face_cells, const int32_t* face_ids, int64_t n_faces,
                                    const double* t_qp, double* out) {
  const int NN = ft.nn, NFQ = ft.nfq;
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n_faces * NN;
       k += (int64_t)gridDim.x * blockDim.x) {
    const int64_t f = k / NN;
    const int a = (int)(k % NN);
    const int64_t e = face_cells[f];
    const int fid = face_ids[f];
    double acc[3] = {0, 0, 0};
    for (int q = 0; q < NFQ; ++q) {
      const double Na = ft.N[fid][q][a];
      if (Na == 0.0) continue;
      double J[3][3] = {};
      for (int n = 0; n < NN; ++n) {
        const int node = conn[e * NN + n];
        for (int d = 0; d < 3; ++d) {
          const double X = coords[(int64_t)node * 3 + d];
          for (int r = 0; r < 3; ++r) J[d][r] += X * ft.dN[fid][q][n][r];
        }
      }
      const double det = det3<double>(J);
      double Ji[3][3];
      inv3<double>(J, det, Ji);
      double v3[3];
      for (int d = 0; d < 3; ++d)
        v3[d] = ft.normal[fid][0] * Ji[0][d] + ft.normal[fid][1] * Ji[1][d] + ft.normal[fid][2] * Ji[2][d];
      const double nanson = sqrt(v3[0] * v3[0] + v3[1] * v3[1] + v3[2] * v3[2]) * det * ft.w[fid][q];
      for (int v = 0; v < vec; ++v) acc[v] += t_qp[(f * NFQ + q) * vec + v] * Na * nanson;
    }
    const int node = conn[e * NN + a];
    for (int v = 0; v < vec; ++v)
      if (acc[v] != 0.0) atomicAdd(out + (int64_t)node * vec + v, acc[v]);
  }
}

}  // namespace fem

using namespace fem;

extern "C" int fem_element_info(int32_t elem_type, int32_t* nodes_per_cell, int32_t* n_quads, int32_t* n_faces,
                                int32_t* n_face_quads) {
  if (elem_nn(elem_type) == 0) return fail(FEM_ERR_ARG, "unknown element type");
  if (nodes_per_cell) *nodes_per_cell = elem_nn(elem_type);
  if (n_quads) *n_quads = elem_nq(elem_type);
  if (n_faces) *n_faces = elem_nf(elem_type);
  if (n_face_quads) *n_face_quads = elem_nfq(elem_type);
  return FEM_OK;
}

extern "C" int fem_element_tables(int32_t elem_type, double* N, double* dN, double* w, double* face_N,
                                  double* face_dN, double* face_w, double* face_normals, int32_t* face_inds) {
  if (elem_nn(elem_type) == 0) return fail(FEM_ERR_ARG, "unknown element type");
  const VolTables t = make_vol_tables(elem_type);
  const FaceTables f = make_face_tables(elem_type);
  for (int q = 0; q < t.nq; ++q) {
    if (w) w[q] = t.w[q];
    for (int n = 0; n < t.nn; ++n) {
      if (N) N[q * t.nn + n] = t.N[q][n];
      if (dN)
        for (int d = 0; d < 3; ++d) dN[(q * t.nn + n) * 3 + d] = t.dN[q][n][d];
    }
  }
  for (int fi = 0; fi < f.nf; ++fi) {
    if (face_normals)
      for (int d = 0; d < 3; ++d) face_normals[fi * 3 + d] = f.normal[fi][d];
    if (face_inds)
      for (int v = 0; v < f.nfv; ++v) face_inds[fi * f.nfv + v] = f.inds[fi][v];
    for (int q = 0; q < f.nfq; ++q) {
      if (face_w) face_w[fi * f.nfq + q] = f.w[fi][q];
      for (int n = 0; n < f.nn; ++n) {
        const int64_t k = ((int64_t)fi * f.nfq + q) * f.nn + n;
        if (face_N) face_N[k] = f.N[fi][q][n];
        if (face_dN)
          for (int d = 0; d < 3; ++d) face_dN[k * 3 + d] = f.dN[fi][q][n][d];
      }
    }
  }
  return FEM_OK;
}

extern "C" int fem_quad_points(const fem_mesh_t* mesh, double* x_out, double* jxw_out, void* stream) {
  int rc = check_mesh(mesh);
  if (rc) return rc;
  if (mesh->n_cells == 0) return FEM_OK;
  VolTables tab = make_vol_tables(mesh->elem_type);
  const int64_t work = mesh->n_cells * tab.nq;
  quad_points_kernel<<<grid_for(work, 256), 256, 0, as_stream(stream)>>>(tab, mesh->coords, mesh->conn,
                                                                         mesh->n_cells, x_out, jxw_out);
  note_launches(1);
  return check_launch("quad_points_kernel");
}

// Cached per-cell geometry: thread per (cell, quadrature point), the cell kernels' own
// arithmetic (qp_geometry on cell-local coordinates) in FP64.
template <int NN, int NQ>
__global__ void cell_geometry_kernel(VolTables tab, const double* coords, const int32_t* conn, int64_t n_cells,
                                     double* grads, double* jxw) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n_cells * NQ;
       k += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = k / NQ;
    const int q = (int)(k % NQ);
    double X[NN * 3], dN[NN * 3];
    const int n0 = conn[e * NN];
    for (int n = 0; n < NN; ++n) {
      const int node = conn[e * NN + n];
      for (int d = 0; d < 3; ++d) {
        X[n * 3 + d] = coords[(int64_t)node * 3 + d] - coords[(int64_t)n0 * 3 + d];
        dN[n * 3 + d] = tab.dN[q][n][d];
      }
    }
    double w;
    qp_geometry<NN, double>(X, dN, tab.w[q], grads + k * (NN * 3), w);
    jxw[k] = w;
  }
}

extern "C" int fem_cell_geometry(const fem_mesh_t* mesh, double* shape_grads, double* jxw, void* stream) {
  int rc = check_mesh(mesh);
  if (rc) return rc;
  FEM_REQUIRE(shape_grads && jxw, "NULL output");
  if (mesh->n_cells == 0) return FEM_OK;
  VolTables tab = make_vol_tables(mesh->elem_type);
  const int64_t work = mesh->n_cells * tab.nq;
  cudaStream_t s = as_stream(stream);
  const int g = grid_for(work, 128);
  switch (mesh->elem_type) {
    case FEM_HEX8:
      cell_geometry_kernel<8, 8><<<g, 128, 0, s>>>(tab, mesh->coords, mesh->conn, mesh->n_cells, shape_grads, jxw);
      break;
    case FEM_TET10:
      cell_geometry_kernel<10, 4><<<g, 128, 0, s>>>(tab, mesh->coords, mesh->conn, mesh->n_cells, shape_grads, jxw);
      break;
    default:
      cell_geometry_kernel<4, 1><<<g, 128, 0, s>>>(tab, mesh->coords, mesh->conn, mesh->n_cells, shape_grads, jxw);
      break;
  }
  note_launches(1);
  return check_launch("cell_geometry_kernel");
}

extern "C" int fem_face_quad_points(const fem_mesh_t* mesh, const int32_t* face_cells, const int32_t* face_ids,
                                    int64_t n_faces, double* x_out, double* nanson_out, void* stream) {
  int rc = check_mesh(mesh);
  if (rc) return rc;
  FEM_REQUIRE(n_faces >= 0, "n_faces < 0");
  if (n_faces == 0) return FEM_OK;
  FEM_REQUIRE(face_cells && face_ids, "face arrays NULL");
  FaceTables ft = make_face_tables(mesh->elem_type);
  const int64_t work = n_faces * ft.nfq;
  face_points_kernel<<<grid_for(work, 128), 128, 0, as_stream(stream)>>>(ft, mesh->coords, mesh->conn, face_cells,
                                                                         face_ids, n_faces, x_out, nanson_out);
  note_launches(1);
  return check_launch("face_points_kernel");
}

extern "C" int fem_body_load(const fem_mesh_t* mesh, const double* f_qp, double* out, void* stream) {
  int rc = check_mesh(mesh);
  if (rc) return rc;
  if (mesh->n_cells == 0) return FEM_OK;
  FEM_REQUIRE(f_qp && out, "f_qp/out NULL");
  VolTables tab = make_vol_tables(mesh->elem_type);
  const int64_t work = mesh->n_cells * tab.nn;
  body_load_kernel<<<grid_for(work, 256), 256, 0, as_stream(stream)>>>(tab, mesh->vec, mesh->coords, mesh->conn,
                                                                       mesh->n_cells, f_qp, out);
  note_launches(1);
  return check_launch("body_load_kernel");
}

extern "C" int fem_surface_load(const fem_mesh_t* mesh, const int32_t* face_cells, const int32_t* face_ids,
                                int64_t n_faces, const double* t_qp, double* out, void* stream) {
  int rc = check_mesh(mesh);
  if (rc) return rc;
  FEM_REQUIRE(n_faces >= 0, "n_faces < 0");
  if (n_faces == 0) return FEM_OK;
  FEM_REQUIRE(face_cells && face_ids && t_qp && out, "NULL argument");
  FaceTables ft = make_face_tables(mesh->elem_type);
  const int64_t work = n_faces * ft.nn;
  surface_load_kernel<<<grid_for(work, 128), 128, 0, as_stream(stream)>>>(
      ft, mesh->vec, mesh->coords, mesh->conn, face_cells, face_ids, n_faces, t_qp, out);
  note_launches(1);
  return check_launch("surface_load_kernel");
}

extern "C" int fem_assemble(const fem_mesh_t* mesh, const fem_material_t* mat, const fem_pattern_t* pat,
                            int32_t outputs, int32_t precision, const double* u, const double* w,
                            const uint8_t* bc_mask, int32_t bc_mode, double* residual, void* vals,
                            double* apply_out, void* stream) {
  int rc = check_mesh(mesh);
  if (rc) return rc;
  FEM_REQUIRE(mat != nullptr, "material NULL");
  FEM_REQUIRE((outputs & ~7) == 0 && outputs != 0, "outputs must be a non-empty FEM_OUT_* mask");
  FEM_REQUIRE(precision == FEM_F32 || precision == FEM_F64 || precision == FEM_DF48,
              "precision must be FEM_F32, FEM_F64 or FEM_DF48");
  FEM_REQUIRE(bc_mode >= FEM_BC_NONE && bc_mode <= FEM_BC_SYMMETRIC, "bad bc_mode");
  FEM_REQUIRE(bc_mode == FEM_BC_NONE || bc_mask, "bc_mode needs bc_mask");
  if (outputs & FEM_OUT_RESIDUAL) FEM_REQUIRE(residual && u, "residual output needs u and residual");
  if (outputs & FEM_OUT_MATRIX) {
    FEM_REQUIRE(pat && pat->indptr && pat->slots && vals, "matrix output needs pattern (indptr, slots) and vals");
    FEM_REQUIRE(elem_nn(mesh->elem_type) <= 255, "slots are 8-bit");
  }
  if (outputs & FEM_OUT_APPLY) FEM_REQUIRE(w && apply_out, "apply output needs w and apply_out");
  if (mesh->n_cells == 0) return FEM_OK;
  AsmParams P;
  rc = fill_params(mesh, mat, P);
  if (rc) return rc;
  P.u = u;
  P.w = w;
  P.bc = bc_mask;
  P.bc_mode = bc_mode;
  P.res = residual;
  P.vals = vals;
  P.apply_out = apply_out;
  if (pat) {
    P.indptr = pat->indptr;
    P.slots = pat->slots;
  }
  cudaStream_t s = as_stream(stream);
  if ((precision == FEM_F32 || precision == FEM_DF48) && (outputs & FEM_OUT_MATRIX)) {
    // FP32 / double-float matrix, FP64 residual / tangent action in a separate pass
    AsmParams Pm = P;
    Pm.outputs = FEM_OUT_MATRIX;
    rc = run_cell_kernel(mesh, Pm, mat->kind, precision, KMODE_ASSEMBLE, s);
    if (rc) return rc;
    const int rest = outputs & ~FEM_OUT_MATRIX;
    if (!rest) return FEM_OK;
    P.outputs = rest;
    return run_cell_kernel(mesh, P, mat->kind, FEM_F64, KMODE_ASSEMBLE, s);
  }
  P.outputs = outputs;
  return run_cell_kernel(mesh, P, mat->kind, FEM_F64, KMODE_ASSEMBLE, s);
}

extern "C" int fem_param_vjp(const fem_mesh_t* mesh, const fem_material_t* mat, const double* u, const double* lam,
                             const uint8_t* bc_mask, double* grad_qp, void* stream) {
  int rc = check_mesh(mesh);
  if (rc) return rc;
  FEM_REQUIRE(mat && u && lam && grad_qp, "NULL argument");
  FEM_REQUIRE(mat->n_qp_params == 1 && mat->qp_params, "parameter VJP needs one qp parameter per point");
  FEM_REQUIRE(mat->kind == FEM_MAT_SIMP || mat->kind == FEM_MAT_NEO_HOOKEAN || mat->kind == FEM_MAT_J2,
              "parameter VJP is defined for SIMP theta, Neo-Hookean rho and J2 modulus scale");
  if (mesh->n_cells == 0) return FEM_OK;
  AsmParams P;
  rc = fill_params(mesh, mat, P);
  if (rc) return rc;
  P.u = u;
  P.w = lam;
  P.bc = bc_mask;
  P.vjp_out = grad_qp;
  return run_cell_kernel(mesh, P, mat->kind, FEM_F64, KMODE_VJP, as_stream(stream));
}

extern "C" int fem_j2_update(const fem_mesh_t* mesh, const fem_material_t* mat, const double* u,
                             double* history_out, void* stream) {
  int rc = check_mesh(mesh);
  if (rc) return rc;
  FEM_REQUIRE(mat && mat->kind == FEM_MAT_J2 && mesh->vec == 3, "J2 update needs a J2 material on vec=3");
  FEM_REQUIRE(u && history_out, "NULL argument");
  FEM_REQUIRE(history_out != mat->history, "history_out must not alias the input history");
  if (mesh->n_cells == 0) return FEM_OK;
  AsmParams P;
  rc = fill_params(mesh, mat, P);
  if (rc) return rc;
  P.u = u;
  P.hist_out = history_out;
  return run_cell_kernel(mesh, P, mat->kind, FEM_F64, KMODE_HIST, as_stream(stream));
}

extern "C" int fem_j2_history_vjp(const fem_mesh_t* mesh, const fem_material_t* mat, const double* u,
                                  const double* lam, const uint8_t* bc_mask, const double* hist_bar,
                                  double* hist_grad, double* scale_grad, double* u_grad, void* stream) {
  int rc = check_mesh(mesh);
  if (rc) return rc;
  FEM_REQUIRE(mat && mat->kind == FEM_MAT_J2 && mesh->vec == 3, "history VJP needs a J2 material on vec=3");
  FEM_REQUIRE(u && hist_grad, "NULL argument");
  FEM_REQUIRE((lam == nullptr) != (hist_bar == nullptr), "give exactly one of lam (adjoint) and hist_bar (update)");
  FEM_REQUIRE(!(lam && u_grad), "u_grad is only produced in update mode (hist_bar)");
  FEM_REQUIRE(!scale_grad || (mat->n_qp_params == 1 && mat->qp_params), "scale_grad needs the modulus-scale field");
  if (mesh->n_cells == 0) return FEM_OK;
  AsmParams P;
  rc = fill_params(mesh, mat, P);
  if (rc) return rc;
  P.u = u;
  P.w = lam;
  P.bc = lam ? bc_mask : nullptr;
  P.hist_bar = hist_bar;
  P.hist_out = hist_grad;
  P.vjp_out = scale_grad;
  P.res = u_grad;
  return run_cell_kernel(mesh, P, mat->kind, FEM_F64, KMODE_HVJP, as_stream(stream));
}

// ---- u-dependent (Robin) surface maps -------------------------------------------------
// Surface map t_v(u, x) = h_v(x) + sum_{k=1..deg} c[v][k] u_v^k on the selected faces
// (problem.py:238-259 with a u-dependent surface_map; applications/robin_bc/example.py:64-80).
// The x-only part h goes into the load vector (fem_surface_load); this kernel adds the
// u-dependent part to the residual, its tangent dt/du N_a N_b nanson to the CSR values (same
// slots as the cell kernel) and/or its action on w.  Thread per (face, node, component).
namespace fem {

struct RobinCoef {
  double c[3][5];
  int deg;
};

template <typename T>
__global__ void robin_kernel(FaceTables ft, int vec, const double* coords, const int32_t* conn,
                             const int32_t* face_cells, const int32_t* face_ids, int64_t n_faces, RobinCoef rc,
                             const double* u, const double* w, const uint8_t* bc, int bc_mode, int outputs,
                             double* res, T* vals, double* apply_out, const int64_t* indptr, const uint8_t* slots) {
  const int NN = ft.nn, NFQ = ft.nfq;
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n_faces * NN * vec;
       k += (int64_t)gridDim.x * blockDim.x) {
    const int v = (int)(k % vec);
    const int a = (int)((k / vec) % NN);
    const int64_t f = k / ((int64_t)vec * NN);
    const int64_t e = face_cells[f];
    const int fid = face_ids[f];
    const int na = conn[e * NN + a];
    const int64_t row = (int64_t)na * vec + v;
    const bool row_bc = bc && bc[row];
    double r = 0.0, ap = 0.0, kb[MAX_NN];
    for (int b = 0; b < NN; ++b) kb[b] = 0.0;
    bool on_face = false;
    for (int q = 0; q < NFQ; ++q) {
      const double Na = ft.N[fid][q][a];
      if (Na == 0.0) continue;
      on_face = true;
      double J[3][3] = {}, uq = 0.0, wq = 0.0;
      for (int n = 0; n < NN; ++n) {
        const int node = conn[e * NN + n];
        for (int d = 0; d < 3; ++d) {
          const double X = coords[(int64_t)node * 3 + d];
          for (int s = 0; s < 3; ++s) J[d][s] += X * ft.dN[fid][q][n][s];
        }
        const double Nn = ft.N[fid][q][n];
        const int64_t dof = (int64_t)node * vec + v;
        uq += Nn * u[dof];
        if (w) wq += Nn * ((bc && bc[dof] && bc_mode == FEM_BC_SYMMETRIC) ? 0.0 : w[dof]);
      }
      const double det = det3<double>(J);
      double Ji[3][3];
      inv3<double>(J, det, Ji);
      double v3[3];
      for (int d = 0; d < 3; ++d)
        v3[d] = ft.normal[fid][0] * Ji[0][d] + ft.normal[fid][1] * Ji[1][d] + ft.normal[fid][2] * Ji[2][d];
      const double nanson = sqrt(v3[0] * v3[0] + v3[1] * v3[1] + v3[2] * v3[2]) * det * ft.w[fid][q];
      double t = 0.0, dt = 0.0, pk = 1.0;   // pk = u^(k-1)
      for (int p = 1; p <= rc.deg; ++p) {
        dt += p * rc.c[v][p] * pk;
        pk *= uq;
        t += rc.c[v][p] * pk;
      }
      r += t * Na * nanson;
      ap += dt * wq * Na * nanson;
      for (int b = 0; b < NN; ++b) kb[b] += dt * Na * ft.N[fid][q][b] * nanson;
    }
    if (!on_face) continue;
    if ((outputs & FEM_OUT_RESIDUAL) && res) atomicAdd(res + row, r);
    if ((outputs & FEM_OUT_APPLY) && apply_out && !row_bc) atomicAdd(apply_out + row, ap);
    if ((outputs & FEM_OUT_MATRIX) && vals && !(row_bc && bc_mode != FEM_BC_NONE)) {
      const int64_t rs = indptr[row];
      const uint8_t* sl = slots + (e * NN + a) * NN;
      for (int b = 0; b < NN; ++b) {
        if (kb[b] == 0.0) continue;
        const int nb = conn[e * NN + b];
        if (bc_mode == FEM_BC_SYMMETRIC && bc && bc[(int64_t)nb * vec + v]) continue;
        atomicAdd(vals + rs + (int64_t)vec * sl[b] + v, T(kb[b]));
      }
    }
  }
}

}  // namespace fem

extern "C" int fem_surface_robin(const fem_mesh_t* mesh, const fem_pattern_t* pat, const int32_t* face_cells,
                                 const int32_t* face_ids, int64_t n_faces, int32_t degree, const double* coeffs,
                                 int32_t outputs, int32_t precision, const double* u, const double* w,
                                 const uint8_t* bc_mask, int32_t bc_mode, double* residual, void* vals,
                                 double* apply_out, void* stream) {
  int rc = check_mesh(mesh);
  if (rc) return rc;
  FEM_REQUIRE(n_faces >= 0 && degree >= 1 && degree <= 4, "need n_faces >= 0 and 1 <= degree <= 4");
  FEM_REQUIRE(coeffs && u, "NULL argument");
  FEM_REQUIRE(!(outputs & FEM_OUT_MATRIX) || (pat && vals && pat->indptr && pat->slots), "matrix output needs a pattern");
  FEM_REQUIRE(!(outputs & FEM_OUT_APPLY) || (w && apply_out), "APPLY needs w and apply_out");
  FEM_REQUIRE(precision == FEM_F32 || precision == FEM_F64, "values must be FEM_F32 or FEM_F64");
  if (n_faces == 0) return FEM_OK;
  FEM_REQUIRE(face_cells && face_ids, "face arrays NULL");
  RobinCoef co{};
  co.deg = degree;
  for (int v = 0; v < mesh->vec; ++v)
    for (int p = 0; p <= degree; ++p) co.c[v][p] = coeffs[v * (degree + 1) + p];
  FaceTables ft = make_face_tables(mesh->elem_type);
  const int64_t work = n_faces * ft.nn * mesh->vec;
  cudaStream_t s = as_stream(stream);
  if (precision == FEM_F32)
    robin_kernel<float><<<grid_for(work, 128), 128, 0, s>>>(
        ft, mesh->vec, mesh->coords, mesh->conn, face_cells, face_ids, n_faces, co, u, w, bc_mask, bc_mode, outputs,
        residual, static_cast<float*>(vals), apply_out, pat ? pat->indptr : nullptr, pat ? pat->slots : nullptr);
  else
    robin_kernel<double><<<grid_for(work, 128), 128, 0, s>>>(
        ft, mesh->vec, mesh->coords, mesh->conn, face_cells, face_ids, n_faces, co, u, w, bc_mask, bc_mode, outputs,
        residual, static_cast<double*>(vals), apply_out, pat ? pat->indptr : nullptr, pat ? pat->slots : nullptr);
  note_launches(1);
  return check_launch("robin_kernel");
}
