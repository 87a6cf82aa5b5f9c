/*
 * jaxfem_gb300.h -- C ABI of the GB300 (sm_103a) implementation of jax-fem's
 * hot path: per-cell weak form at quadrature points, scatter-add assembly of
 * the residual and the CSR Jacobian, the Krylov solve and the implicit adjoint.
 *
 * The reference (deepmodeling/jax-fem) is pure Python on JAX/PETSc and has no
 * native FFI of its own; each entry point below replaces the reference
 * function(s) cited beside it (paths relative to the jax-fem repository).
 *
 * Conventions (all entry points):
 *   - return an int status: FEM_OK (0) or an FEM_ERR_* code; the message is
 *     available from fem_last_error() on the calling thread;
 *   - take raw DEVICE pointers, sizes and an opaque CUDA stream (`void*`,
 *     a cudaStream_t; NULL = legacy default stream); work is enqueued on that
 *     stream and nothing is synchronised unless stated (calls that return a
 *     host-side count or status synchronise the stream);
 *   - never allocate device memory: every workspace is caller-owned, sized by
 *     the matching *_workspace() query;
 *   - degrees of freedom are ordered dof = node*vec + component
 *     (jax_fem/problem.py:86-92), matrices are CSR with rows sorted by column.
 *   - not re-entrant on the same workspace; one stream per problem.
 */
#ifndef JAXFEM_GB300_H
#define JAXFEM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes -------------------------------------------------------- */
enum {
  FEM_OK = 0,
  FEM_ERR_ARG = 1,         /* invalid argument (null pointer, bad size, bad enum) */
  FEM_ERR_CUDA = 2,        /* a CUDA runtime call or kernel launch failed        */
  FEM_ERR_UNSUPPORTED = 3, /* element / material / precision combination absent  */
  FEM_ERR_CAPACITY = 4,    /* workspace too small or a row exceeds 255 blocks    */
  FEM_ERR_DEVICE = 5       /* a kernel reported invalid data (e.g. bad node id)  */
};

/* ---- enumerations -------------------------------------------------------- */
enum { FEM_HEX8 = 1, FEM_TET10 = 2, FEM_TET4 = 3 };          /* jax_fem/basis.py:19-114 */
enum {
  FEM_F32 = 0,
  FEM_F64 = 1,
  FEM_DF48 = 2,  /* matrix values as FP32 hi + int16 correction q (a = hi + q*ulp(hi)/2^16, a
                    40-bit mantissa in 6 bytes): hi[m] floats, then at byte offset
                    round_up(4*m, 256) q[m] int16.  Vectors for DF48 SpMV: x is the
                    (hi[n], lo[n]) float pair of fem_vector_split, y is FP64.  Arithmetic is
                    double-float on FP32 pipes (error-free two-product / two-sum). */
  /* Sliced node-block layouts (solver copies; built by fem_matrix_convert from FP64 CSR
   * values): node rows in slices of 32, slice s owning block slots slice_ptr[s] ..
   * slice_ptr[s+1]; value v (= r*vec + d) of slot k for the node in lane l sits at
   * (k*vec*vec + v)*32 + l.  One warp per slice, one lane per node row, every load a
   * full coalesced line and no cross-lane reduction.  Vectors as for the unsliced type. */
  FEM_SLICED_F32 = 3,
  FEM_SLICED_F64 = 4,
  FEM_SLICED_DF48 = 5,
  /* Symmetric sliced DF48: only the upper node blocks (block column >= row, diagonal first)
   * of a symmetric matrix, in the sliced layout of fem_pattern_slices_upper (slice_ptr_u,
   * slice_cols_u; padding slots point at the row itself with zero values).  The SpMV adds
   * A_ij x_j to row i and A_ij^T x_i to row j (FP64 atomics into a separate FP64 vector),
   * so it reads about half the bytes; its result is not bitwise reproducible. */
  FEM_SYM_DF48 = 6,
  /* Structured symmetric DF48 (vec 3): for a node grid numbered node = (i*ny + j)*nz + k
   * (fem_pattern_t.grid_nx/ny/nz set), the diagonal and the 13 upper neighbours of the 27-point
   * stencil per node row with implicit columns, value v of slot s of row (line L, k) at
   * (((L/32)*nz + k)*14 + s)*288 + v*32 + L%32 (hi floats, then the int16 corrections at
   * round_up(4*m, 256); 256 bytes more hold the converter's pattern check).  The SpMV keeps the
   * transposed half in registers and warp shuffles and sends the rest (plane i+1 and the warp
   * edges) to an FP64 vector by atomics, so its result is not bitwise reproducible. */
  FEM_SSYM_DF48 = 7
};
enum {                                                       /* built-in tensor maps     */
  FEM_MAT_LAPLACE = 1,        /* consts: [k]                      test_linear_poisson.py:15-17 */
  FEM_MAT_LINEAR_ELASTIC = 2, /* consts: [E, nu]                  test_linear_elasticity_cube.py:15-26 */
  FEM_MAT_SIMP = 3,           /* consts: [Emax, Emin, nu, penal]; qp param theta */
  FEM_MAT_GENERAL_LINEAR = 4, /* consts: C ((vec*3)^2, row-major) sigma_I = C_IJ grad_J */
  FEM_MAT_NEO_HOOKEAN = 5,    /* consts: [E, nu, clampJ]; optional qp param rho (E*rho)
                                 test_hyper_elasticity.py:15-34, hyperelastic3d_common.py:45-70 */
  FEM_MAT_J2 = 6              /* consts: [E, nu, sig0]; history sigma_old|eps_old (18/qp);
                                 optional qp param s scaling E      test_plasticity.py:32-78 */
};
enum { FEM_OUT_RESIDUAL = 1, FEM_OUT_MATRIX = 2, FEM_OUT_APPLY = 4,
       FEM_OUT_PARAM_VJP = 8 /* run-time compiled kernels only: -lam^T dR/d(internal vars) */ };
enum {
  FEM_BC_NONE = 0,
  FEM_BC_ROWS = 1,      /* skip Dirichlet rows (PETSc zeroRows semantics, solver.py:527-528) */
  FEM_BC_SYMMETRIC = 2  /* skip Dirichlet rows and columns (symmetric elimination for CG) */
};
enum { FEM_PC_NONE = 0, FEM_PC_JACOBI = 1, FEM_PC_BJACOBI = 2 };
/* FEM_SOLVE_STAGNATED (solvers with FP64 reliable updates): the FP64 true residual stopped falling
 * above the target -- the attainable accuracy of the arithmetic; x holds the last iterate. */
enum { FEM_SOLVE_CONVERGED = 0, FEM_SOLVE_MAXITER = 1, FEM_SOLVE_BREAKDOWN = 2, FEM_SOLVE_NAN = 3,
       FEM_SOLVE_STAGNATED = 4 };

/* ---- plain descriptor structs (pointers are device pointers) ------------- */
typedef struct fem_mesh_t {
  int32_t elem_type;        /* FEM_HEX8 / FEM_TET10 / FEM_TET4                   */
  int32_t vec;              /* components per node: 1 or 3                        */
  int64_t n_nodes;
  int64_t n_cells;
  const double* coords;     /* (n_nodes, 3)                                       */
  const int32_t* conn;      /* (n_cells, nodes_per_cell), meshio node order       */
  /* Optional per-cell geometry from fem_cell_geometry (both or neither): the
   * (n_cells, nq, nodes_per_cell, 3) physical shape gradients and (n_cells, nq) JxW.
   * When set, the cell kernels read them instead of recomputing the Jacobians;
   * NULL: recomputed in every launch.  Replaces nothing: the reference keeps the
   * same arrays (problem.py:130-147, fe.shape_grads / fe.JxW). */
  const double* shape_grads;
  const double* jxw;
} fem_mesh_t;

typedef struct fem_pattern_t {
  int64_t nnzb;             /* number of node-pair blocks                         */
  const int64_t* block_ptr; /* (n_nodes+1)                                        */
  const int32_t* block_cols;/* (nnzb), sorted within each node row               */
  const int64_t* indptr;    /* scalar CSR row pointers (n_nodes*vec+1)            */
  const int64_t* diag;      /* (n_nodes*vec) offset of each row's diagonal entry  */
  const uint8_t* slots;     /* (n_cells, npc, npc): position of conn[b] in row conn[a] */
  int64_t n_slices;         /* sliced layout (fem_pattern_slices); 0 when not built  */
  int64_t n_slots;          /* total block slots of the sliced layout (host value)    */
  const int64_t* slice_ptr; /* (n_slices+1) first block slot of each 32-node slice    */
  const int32_t* slice_cols;/* (n_slots*32) block column of slot k, lane l (padding: 0; */
                            /* grid layout: node + stencil offset, clamped)           */
  int64_t n_slots_u;        /* upper-block sliced layout (fem_pattern_slices_upper)  */
  const int64_t* slice_ptr_u;
  const int32_t* slice_cols_u;/* padding: the row's own node                         */
  int64_t grid_nx, grid_ny, grid_nz; /* node grid of a structured box numbering          */
                            /* node = (i*ny + j)*nz + k, or 0 when not structured   */
  int64_t slices_grid;      /* 1: slice_ptr / slice_cols are the grid layout of      */
                            /* fem_pattern_slices_grid (slot k = stencil offset k)  */
} fem_pattern_t;

typedef struct fem_material_t {
  int32_t kind;             /* FEM_MAT_*                                          */
  int32_t n_consts;         /* <= 96                                              */
  const double* consts;     /* HOST pointer, copied at call time                  */
  int32_t n_qp_params;      /* per quadrature point parameters (0 or 1)           */
  const double* qp_params;  /* (n_cells, nq, n_qp_params) or NULL                 */
  const double* history;    /* J2: (n_cells, nq, 18) = sigma_old(9) | eps_old(9)  */
} fem_material_t;

/* Parameter block of the run-time compiled (user) kernels, fem_jit_launch.  Every field is 8 bytes
 * wide so the generated kernel's copy of the struct has the same layout.
 *   coords/conn: the mesh; n_items: cells (cell kernel) or faces (face kernel);
 *   face_cells/face_ids: the faces' cell and local face (face kernels);
 *   u: dofs; w: direction of FEM_OUT_APPLY; lam: multiplier of FEM_OUT_PARAM_VJP;
 *   iv: per-cell internal variables, iv_stride doubles per cell (per face for face kernels);
 *   indptr/slots: CSR rows and per-cell slot table (FEM_OUT_MATRIX); bc/bc_mode: Dirichlet mask
 *   and handling as fem_assemble; outputs: FEM_OUT_* bits;
 *   res/vals/apply_out: atomically accumulated FP64 outputs; vjp_out: iv_stride values per item. */
typedef struct fem_jit_params_t {
  const double* coords;
  const int32_t* conn;
  int64_t n_items;
  const int32_t* face_cells;
  const int32_t* face_ids;
  const double* u;
  const double* w;
  const double* lam;
  const double* iv;
  int64_t iv_stride;
  const int64_t* indptr;
  const uint8_t* slots;
  const uint8_t* bc;
  int64_t bc_mode;
  int64_t outputs;
  double* res;
  double* vals;
  double* apply_out;
  double* vjp_out;
} fem_jit_params_t;

/* ---- library ------------------------------------------------------------- */
const char* fem_last_error(void);
int fem_version(void);
/* Number of kernels this library has launched in the process (diagnostic counter; no
 * counterpart in the reference). */
uint64_t fem_kernel_launches(void);
/* Element sizes: nodes per cell, volume quad points, faces, face quad points. */
int fem_element_info(int32_t elem_type, int32_t* nodes_per_cell, int32_t* n_quads,
                     int32_t* n_faces, int32_t* n_face_quads);

/* Reference-element tables in double precision, written to HOST arrays (any may be NULL):
 * N (nq,nn), dN (nq,nn,3), w (nq), face_N (nf,nfq,nn), face_dN (nf,nfq,nn,3), face_w (nf,nfq),
 * face_normals (nf,3), face_inds (nf,nfv).  Replaces jax_fem/basis.py:141-250 (basix tabulation). */
int fem_element_tables(int32_t elem_type, double* N, double* dN, double* w, double* face_N, double* face_dN,
                       double* face_w, double* face_normals, int32_t* face_inds);

/* ---- sparsity pattern ----------------------------------------------------
 * Replaces the COO index build jax_fem/problem.py:86-107 and PETSc's COO
 * preallocation jax_fem/solver.py:474-478: the pattern is the sorted union of
 * every cell's dof pairs, kept as node-pair blocks (each block is vec x vec
 * and fully populated) plus the equivalent scalar CSR row pointers.  */
int fem_pattern_workspace(int64_t n_cells, int32_t nodes_per_cell, int64_t n_nodes, size_t* bytes);
/* Builds node->cell incidence in ws, writes block_ptr and the total block count (host). Syncs. */
int fem_pattern_count(int32_t elem_type, const int32_t* conn, int64_t n_cells, int64_t n_nodes,
                      void* ws, size_t ws_bytes, int64_t* block_ptr, int64_t* nnzb_out, void* stream);
/* Fills block_cols (nnzb); ws must hold what fem_pattern_count left there. */
int fem_pattern_fill(int32_t elem_type, const int32_t* conn, int64_t n_cells, int64_t n_nodes,
                     void* ws, size_t ws_bytes, const int64_t* block_ptr, int32_t* block_cols, void* stream);
/* Per-cell block slots: slots[c][a][b] = position of conn[c][b] in row conn[c][a]. */
int fem_pattern_slots(int32_t elem_type, const int32_t* conn, int64_t n_cells,
                      const int64_t* block_ptr, const int32_t* block_cols, uint8_t* slots, void* stream);
/* Scalar CSR view: indptr (n_nodes*vec+1), diag (n_nodes*vec), indices (nnzb*vec*vec, may be NULL). */
int fem_pattern_scalar(int64_t n_nodes, int32_t vec, const int64_t* block_ptr, const int32_t* block_cols,
                       int64_t* indptr, int64_t* diag, int32_t* indices, void* stream);

/* ---- geometry and loads ---------------------------------------------------
 * Replaces jax_fem/fe.py:112-218 (shape grads, JxW, physical quad points,
 * face Nanson scale) and the u-independent parts of the mass / surface
 * kernels jax_fem/problem.py:216-259. */
int fem_quad_points(const fem_mesh_t* mesh, double* x_out /* (n_cells,nq,3) or NULL */,
                    double* jxw_out /* (n_cells,nq) or NULL */, void* stream);
/* Physical shape gradients (n_cells, nq, nodes_per_cell, 3) and JxW (n_cells, nq) in FP64
 * (fe.py:112-141 get_shape_grads, kept by problem.py:130-147 initialize_geometric_quantities):
 * J = sum_a (x_a - x_0) (x) dN_a/dxi, grads = dN/dxi J^-1, JxW = det J w_q.  Store the two
 * pointers in fem_mesh_t.shape_grads / .jxw to let the cell kernels reuse them. */
int fem_cell_geometry(const fem_mesh_t* mesh, double* shape_grads, double* jxw, void* stream);
int fem_face_quad_points(const fem_mesh_t* mesh, const int32_t* face_cells, const int32_t* face_ids,
                         int64_t n_faces, double* x_out /* (n_faces,nfq,3) */,
                         double* nanson_out /* (n_faces,nfq) or NULL */, void* stream);
/* out[dof] += sum_q f_qp[c,q,:] N_a(q) JxW  (mass_map evaluated at quad points) */
int fem_body_load(const fem_mesh_t* mesh, const double* f_qp, double* out, void* stream);
/* out[dof] += sum_q t_qp[f,q,:] N_a(q) nanson  (surface_map at face quad points) */
int fem_surface_load(const fem_mesh_t* mesh, const int32_t* face_cells, const int32_t* face_ids,
                     int64_t n_faces, const double* t_qp, double* out, void* stream);
/* u-dependent surface maps (problem.py:238-259 with a u-dependent surface_map; Robin,
 * applications/robin_bc/example.py:64-80): t_v(u, x) = h_v(x) + sum_{k=1..degree} c[v][k] u_v^k,
 * coeffs (host) = c as vec x (degree+1) (column 0 unused: h goes through fem_surface_load).
 * outputs: FEM_OUT_RESIDUAL adds sum_q t N_a nanson to residual; FEM_OUT_MATRIX adds
 * dt/du N_a N_b nanson to vals (FEM_F32 / FEM_F64, BC rows / columns as fem_assemble's bc_mode);
 * FEM_OUT_APPLY adds the tangent action on w to apply_out.  1 <= degree <= 4. */
int fem_surface_robin(const fem_mesh_t* mesh, const fem_pattern_t* pat, const int32_t* face_cells,
                      const int32_t* face_ids, int64_t n_faces, int32_t degree, const double* coeffs,
                      int32_t outputs, int32_t precision, const double* u, const double* w, const uint8_t* bc_mask,
                      int32_t bc_mode, double* residual, void* vals, double* apply_out, void* stream);

/* ---- per-cell weak form and assembly --------------------------------------
 * Replaces the cell kernels and their jacfwd tangents jax_fem/problem.py:189-303,
 * the batched evaluation split_and_compute_cell :359-396, the residual scatter
 * compute_residual_vars_helper :426-437, compute_newton_vars :447-460 and the
 * PETSc setValuesCOO/assemble jax_fem/solver.py:522-526.
 * outputs: FEM_OUT_RESIDUAL  residual += R_int(u)           (FP64 always)
 *          FEM_OUT_MATRIX    vals += K(u) in `precision`    (consistent hand-derived tangent;
 *                            FEM_F32 / FEM_F64 values; FEM_DF48: FP64 values computed in
 *                            double-float arithmetic on the FP32 pipes, ~2^-46 relative, for
 *                            the DF48 solver copies -- isotropic materials (linear elastic,
 *                            SIMP) with the mesh's geometry cache; others assemble in FP64)
 *          FEM_OUT_APPLY     apply_out += K(u) w            (FP64 always)
 * Outputs are accumulated (the caller zeroes them).  bc_mode controls which
 * matrix entries are skipped (FEM_BC_*); bc_mask is one byte per dof.  With a
 * bc_mask, FEM_OUT_RESIDUAL / FEM_OUT_APPLY skip Dirichlet rows too, and
 * FEM_OUT_APPLY with FEM_BC_SYMMETRIC also treats w as zero on Dirichlet dofs
 * (the action of the eliminated operator K_ff). */
int fem_assemble(const fem_mesh_t* mesh, const fem_material_t* mat, const fem_pattern_t* pat,
                 int32_t outputs, int32_t precision, const double* u, const double* w,
                 const uint8_t* bc_mask, int32_t bc_mode, double* residual, void* vals,
                 double* apply_out, void* stream);

/* Parameter VJP (replaces the jax.vjp of the BC-applied residual w.r.t. params in
 * implicit_vjp, jax_fem/solver.py:1386-1416):
 *   grad_qp[c,q,k] = - sum_a lam_a . dR_a/dp_{c,q,k}   (lam masked to 0 on Dirichlet dofs). */
int fem_param_vjp(const fem_mesh_t* mesh, const fem_material_t* mat, const double* u,
                  const double* lam, const uint8_t* bc_mask, double* grad_qp, void* stream);

/* J2 history update (tests/benchmarks/plasticity/test_plasticity.py:73-78):
 * history_out[c,q] = (return_map(grad u, history), strain(grad u)). */
int fem_j2_update(const fem_mesh_t* mesh, const fem_material_t* mat, const double* u,
                  double* history_out, void* stream);

/* Reverse mode of the J2 material through its history, for gradients over several load steps
 * (the reference takes jax.grad over a loop of fwd_pred and update_int_vars_gp:
 * applications/crystal_plasticity/volume_sensitivity.py:89-107; return map and update
 * test_plasticity.py:54-78).  Exactly one of:
 *   lam (adjoint mode): cotangents of -lam^T R(u; history, scale) (lam masked on Dirichlet dofs);
 *   hist_bar (update mode, (cells, nq, 18)): cotangents of fem_j2_update's outputs
 *     (sigma_new 9 | eps_new 9); u_grad (n_dofs, accumulated: +=) receives the cotangent of u.
 * hist_grad (cells, nq, 18) receives the cotangents of the input history (sigma_old | eps_old);
 * scale_grad (cells, nq), optional, those of the modulus-scale field. */
int fem_j2_history_vjp(const fem_mesh_t* mesh, const fem_material_t* mat, const double* u, const double* lam,
                       const uint8_t* bc_mask, const double* hist_bar, double* hist_grad, double* scale_grad,
                       double* u_grad, void* stream);

/* ---- Dirichlet rows -------------------------------------------------------
 * fem_zero_rows: PETSc zeroRows with KEEP_NONZERO_PATTERN (solver.py:477,527-528):
 *   every entry of each listed row := 0, then the diagonal := diag_value.
 * fem_apply_bc_vec: apply_bc_vec (solver.py:290-304): res[r] = dofs[r] - scale*vals[i]. */
int fem_zero_rows(const fem_pattern_t* pat, int32_t vec, int32_t precision, void* vals,
                  const int32_t* rows, int64_t n_rows, double diag_value, void* stream);
int fem_apply_bc_vec(double* res, const double* dofs, const int32_t* rows, const double* values,
                     int64_t n_rows, double scale, void* stream);
/* fem_matrix_transpose: vals_t := A^T in the same CSR pattern (out of place; FP32 / FP64 CSR
 * order).  Replaces the PETSc transpose of the adjoint (solver.py:1405-1409: A_T =
 * A.transpose(); the adjoint solves A_T lam = v).  ws: >= 4 bytes of device scratch (a pattern
 * error flag).  Fails with FEM_ERR_ARG if a block (I, J) has no (J, I) partner.  Syncs. */
int fem_matrix_transpose(const fem_pattern_t* pat, int64_t n_nodes, int32_t vec, int32_t precision,
                         const void* vals, void* vals_t, void* ws, size_t ws_bytes, void* stream);

/* ---- sparse linear algebra ------------------------------------------------
 * Replaces jax.scipy.sparse.linalg.bicgstab on the BCOO matrix (solver.py:63-92)
 * and PETSc KSPCG/KSPBCGS with PCJACOBI / PCBJACOBI (solver.py:109-134). */
int fem_spmv(const fem_pattern_t* pat, int64_t n_nodes, int32_t vec, int32_t precision,
             const void* vals, const void* x, void* y, void* stream);
/* Sliced layout of the pattern: with slice_cols == NULL writes slice_ptr (n_slices+1, where
 * n_slices = ceil(n_nodes/32)) and the slot count (host; syncs); otherwise fills slice_cols. */
int fem_pattern_slices(int64_t n_nodes, const int64_t* block_ptr, const int32_t* block_cols,
                       int64_t* slice_ptr, int32_t* slice_cols, int64_t* n_slots, void* stream);
/* Sliced layout of a pattern on the node grid nx x ny x nz (node = (i*ny + j)*nz + k, the
 * numbering of box_mesh) whose node rows hold only 27-point-stencil neighbours (HEX8, TET4): every
 * slice has 27 slots, slot k = (di+1)*9 + (dj+1)*3 + (dk+1) holding the block of neighbour
 * (i+di, j+dj, k+dk), a zero block where that neighbour is outside the grid or not coupled.
 * slice_ptr (n_slices+1) = 27 s; slice_cols (27*n_slices*32) = node + offset of slot k, clamped
 * to [0, n_nodes).  n_slots = 27*n_slices.  The column of every slot follows from the grid, so the
 * mixed CG's SpMV streams no block columns.  Fails with FEM_ERR_ARG (slice_ptr then undefined)
 * when a row holds a block outside the stencil.  Set fem_pattern_t.slices_grid = 1 with these
 * arrays.  Syncs. */
int fem_pattern_slices_grid(int64_t n_nodes, const int64_t* block_ptr, const int32_t* block_cols, int64_t nx,
                            int64_t ny, int64_t nz, int64_t* slice_ptr, int32_t* slice_cols, void* stream);
/* The same for the upper node blocks of each row (block column >= row): slice_ptr_u,
 * slice_cols_u and n_slots_u of the FEM_SYM_DF48 layout. */
int fem_pattern_slices_upper(int64_t n_nodes, const int64_t* block_ptr, const int32_t* block_cols,
                             int64_t* slice_ptr_u, int32_t* slice_cols_u, int64_t* n_slots_u, void* stream);
/* Bytes of a value buffer for `pat` in `precision` (any FEM_F32 .. FEM_SLICED_DF48). */
int fem_matrix_bytes(const fem_pattern_t* pat, int32_t vec, int32_t precision, size_t* bytes);
/* FP64 CSR values -> values in `precision` (FEM_F32, FEM_DF48 or a sliced type). */
int fem_matrix_convert(const fem_pattern_t* pat, int64_t n_nodes, int32_t vec, const double* vals64,
                       int32_t precision, void* out, void* stream);
/* FP64 vector -> (hi[n], lo[n]) float pair, the FEM_DF48 SpMV input. */
int fem_vector_split(const double* x, int64_t n, float* x_df, void* stream);
/* The mixed CG's SpMV (no counterpart in the reference: the inner operator of
 * fem_pcg_refined with FEM_SLICED_DF48 / FEM_SYM_DF48).  y = A x with A in `precision`
 * (FEM_SLICED_DF48, or FEM_SYM_DF48 whose transposed half is folded into y); x is a
 * node-interleaved double-float vector: component c of node i is the float pair
 * (hi, lo) at pair index i*pad + c, pad = 4 for vec 3 (32 bytes per node) and 1 for vec 1;
 * y is written as y_hi[n] + y_lo[n] (scalar row order).  When xy_dot (device) is non-NULL it
 * receives the dot x.y.  ws: at least fem_krylov_workspace(n_dofs, FEM_SLICED_DF48) bytes.
 * For vec 3 with 16-byte aligned vals and slice_cols the slices are streamed through
 * shared memory by bulk copies (cp.async.bulk + mbarrier); a barrier wait that exceeds
 * its limit returns FEM_ERR_DEVICE. */
int fem_spmv_dfx(const fem_pattern_t* pat, int64_t n_nodes, int32_t vec, int32_t precision, const void* vals,
                 const void* x_df, float* y_hi, float* y_lo, double* xy_dot, void* ws, size_t ws_bytes, void* stream);
/* Jacobi: pc = 1/diag (n_dofs values); block Jacobi: inverse node blocks (n_nodes*vec*vec). */
int fem_precond_setup(const fem_pattern_t* pat, int64_t n_nodes, int32_t vec, int32_t precision,
                      const void* vals, int32_t pc_kind, void* pc, void* stream);
int fem_krylov_workspace(int64_t n_dofs, int32_t precision, size_t* bytes);
/* Preconditioned CG on an SPD matrix.  Stops when ||r||_2 <= max(rtol*||b||_2, atol)
 * (checked every iteration on the device; dots and norms in FP64).  Syncs. */
int fem_pcg(const fem_pattern_t* pat, int64_t n_nodes, int32_t vec, int32_t precision,
            const void* vals, int32_t pc_kind, const void* pc, const void* b, void* x,
            double rtol, double atol, int64_t maxiter, void* ws, size_t ws_bytes,
            int64_t* iterations, double* res_norm, int32_t* status, void* stream);
/* Allocation-free PCG (no counterpart in the reference).  Same method, arguments and result
 * as fem_pcg, for callers that cannot allocate device memory: host frameworks whose device
 * allocator is closed to plug-ins, and embeddings that reserve all device memory up front and
 * forbid allocation after start-up.  Its scratch is a fixed file-scope device array of
 * about 8.6 MB that every GPU loading the library keeps until the process exits; systems of
 * more than 262144 dofs (n_nodes*vec) are rejected with FEM_ERR_CAPACITY.  The first call on a
 * device looks up the array's device address and caches it for that device.  The cached
 * address belongs to the CUDA context of that
 * first call: after cudaDeviceReset on a device, the next call would hand the kernels a stale
 * address, so a process that resets a device must not call this entry point on it again.
 * Every call shares the array, so calls that overlap on the GPU (two streams, two threads)
 * race: serialise them.  Allocates nothing (no cudaMalloc / cudaFree).  Like fem_pcg it
 * synchronises with the host while it runs: it reads the convergence flag back every 16
 * iterations. */
int fem_pcg_static(const fem_pattern_t* pat, int64_t n_nodes, int32_t vec, int32_t precision,
                   const void* vals, int32_t pc_kind, const void* pc, const void* b, void* x,
                   double rtol, double atol, int64_t maxiter, int64_t* iterations, double* res_norm,
                   int32_t* status, void* stream);
/* BiCGStab with jax.scipy.sparse.linalg.bicgstab's iteration and stopping rule
 * ||r||^2 <= max(tol^2 ||b||^2, atol^2) (solver.py:78-84).  Syncs. */
int fem_bicgstab(const fem_pattern_t* pat, int64_t n_nodes, int32_t vec, int32_t precision,
                 const void* vals, int32_t pc_kind, const void* pc, const void* b, void* x,
                 double tol, double atol, int64_t maxiter, void* ws, size_t ws_bytes,
                 int64_t* iterations, double* res_norm, int32_t* status, void* stream);

/* Mixed-precision PCG with FP64 reliable updates.  precision FEM_F32 / FEM_SLICED_F32: FP32
 * matrix, FP32 vectors; FEM_DF48 / FEM_SLICED_DF48 / FEM_SYM_DF48 / FEM_SSYM_DF48: DF48 matrix
 * (double-float SpMV on FP32 pipes), double-float vectors, dot partials reduced in double-float,
 * FP64 scalars.  The preconditioner pc32 is FP32 in all cases (Jacobi: one float per dof; block
 * Jacobi: the VEC x VEC inverse blocks, VEC^2 floats per node).  CG takes the matrix and the
 * preconditioner as symmetric: with FEM_SLICED_DF48 and vec 3 the block inverses are applied
 * through their upper triangles.
 * Solves the Dirichlet-eliminated system K_ff x_f = b_f (x_b = b_b on Dirichlet dofs)
 * where K is the tangent of `mat` at u_lin.  x (FP64, in/out) holds the initial guess.
 * When the FP32 recursive residual has fallen by `delta` since the last replacement,
 * the FP32 increment is added into x in FP64 and the residual is replaced by the true
 * residual b - K x computed in FP64 -- by SpMV with vals_ref (the FP64 Dirichlet-eliminated
 * matrix, FEM_F64 or FEM_SLICED_F64) when given, else by the matrix-free tangent action of
 * mesh / mat at u_lin; the search direction is kept.  Stops when the FP64 true residual satisfies
 * ||b - K x||_2 <= max(rtol ||b||_2, atol).  ws >= fem_krylov_workspace(n, FEM_F64).
 * Replaces the reference's FP64-only linear solve in newton_step / implicit_vjp
 * (jax_fem/solver.py:390-421, 1399-1409) for the mixed-precision path.  Syncs. */
int fem_pcg_refined(const fem_pattern_t* pat, int64_t n_nodes, int32_t vec, int32_t precision, const void* vals32,
                    int32_t pc_kind, const void* pc32, const fem_mesh_t* mesh, const fem_material_t* mat,
                    const double* u_lin, const void* vals_ref, int32_t ref_precision,
                    const uint8_t* bc_mask, const double* b, double* x,
                    double rtol, double atol, double delta, int64_t maxiter, void* ws, size_t ws_bytes,
                    int64_t* iterations, int64_t* updates, double* res_norm, int32_t* status, void* stream);

/* ---- vector helpers for refinement / Newton ------------------------------ */
/* dst32[i] = mask[i] ? 0 : (float)src64[i]  (mask may be NULL) */
int fem_cast_f64_f32(const double* src, float* dst, int64_t n, const uint8_t* mask, void* stream);
/* y64[i] += alpha * (double)x32[i] */
int fem_axpy_f32_f64(double alpha, const float* x, double* y, int64_t n, void* stream);
/* Deterministic FP64 dot product written to *out (device); ws >= fem_krylov_workspace bytes. */
int fem_dot(int32_t precision, const void* x, const void* y, int64_t n, double* out,
            void* ws, size_t ws_bytes, void* stream);
/* Measurement hook (no reference counterpart): between start and stop, the mixed CG
 * (fem_pcg_refined with a DF48 format) brackets the second SpMV of every 16-iteration chunk
 * (the first follows the host's poll) with CUDA events on its stream; stop returns the summed SpMV time and the
 * number of timed launches.  Process-wide state: not for concurrent solves. */
int fem_spmv_timing_start(void);
int fem_spmv_timing_stop(double* seconds, int64_t* samples);
/* Failure-detection self-test (no reference counterpart; the reference's solvers do not wait on
 * the device): one warp waits, through the bounded mbarrier wait of the bulk-copy kernels, on a
 * phase that never completes; the wait gives up after its limit (~2 s) and the call returns
 * FEM_ERR_DEVICE exactly as a solver whose copy never landed would.  The context stays usable.
 * ws >= fem_krylov_workspace(0, FEM_F64) bytes. */
int fem_selftest_bounded_wait(void* ws, size_t ws_bytes, void* stream);

/* ---- topology-optimisation update (jax_fem/mma.py) ------------------------------------ */
/* Workspace bytes of fem_mma_update for n design variables and m constraints (1 <= m <= 4). */
int fem_mma_workspace(int64_t n, int32_t m, size_t* bytes);
/* One MMA update (MMA.mmasub, mma.py:113-206, with subsolv, mma.py:209-405), all per-variable
 * work on the GPU.  Device arrays (n): xval, xold1, xold2, xmin, xmax, df0dx; dfdx (m x n,
 * row-major); low / upp are read (iter > 2) and written; xmma receives the new design.  Host
 * arrays (m): fval, a, c, d.  iter is the reference's epoch (asymptotes re-initialised while
 * iter <= 2).  newton_steps (host, optional) receives the interior-point Newton step count. */
int fem_mma_update(int64_t n, int32_t m, int32_t iter, const double* xval, const double* xold1,
                   const double* xold2, double* low, double* upp, const double* xmin, const double* xmax,
                   double move, const double* df0dx, const double* fval, const double* dfdx, double a0,
                   const double* a, const double* c, const double* d, double* xmma, void* ws, size_t ws_bytes,
                   int32_t* newton_steps, void* stream);
/* Filter of compute_filter_kd_tree (mma.py:27-57): for each of n centroids (device, n x 3) the
 * at most nnb nearest centroids closer than rmin, weights rmin - distance, stored nnb per row
 * (cols = -1 in unused slots), hs = row sums.  Ties at the nnb-th distance keep lower indices. */
int fem_filter_workspace(int64_t n, size_t* bytes);
int fem_filter_build(int64_t n, const double* centroids, double rmin, int32_t nnb, int32_t* cols, double* vals,
                     double* hs, void* ws, size_t ws_bytes, void* stream);
/* mode 0: applySensitivityFilter (mma.py:59-62) on nr rows g (nr x n): H (rho g / max(1e-3, rho) / Hs);
 * mode 1: applyDensityFilter (mma.py:64-66): H g / Hs. */
int fem_filter_apply(int64_t n, int32_t nnb, const int32_t* cols, const double* vals, const double* hs,
                     const double* rho, const double* g, int32_t nr, int32_t mode, double* out, void* stream);

/* ---- dynamic relaxation (jax_fem/solver.py:918-1049) --------------------------------- */
/* out[r] = scale * sum_k |vals[k]| over scalar CSR row r (lumped mass of assembleCSR's matrix,
 * solver.py:959-961, with scale = h~^2/4). */
int fem_row_abs_sum(int64_t n_rows, const int64_t* indptr, const double* vals, double scale, double* out,
                    void* stream);
/* q_old = q; R_old = R; q += h qdot (solver.py:983-985). */
int fem_dr_march(int64_t n, double h, double* q, double* q_old, const double* qdot, const double* R, double* R_old,
                 void* stream);
/* out4 (host) = [max|R|, sum (R - R_old)/h qdot, sum qdot M qdot,
 *                max h~^2/4 |(qdd - qdd_old)/(q - q_old)| over q != q_old] (solver.py:991-1002);
 * ws: device scratch of at least 8*(4*2048+4) bytes.  Synchronises the stream. */
int fem_dr_measure(int64_t n, double h, double h_tilde, const double* R, const double* R_old, const double* qdot,
                   const double* M, const double* q, const double* q_old, const double* qdd, const double* qdd_old,
                   double* out4, double* ws, size_t ws_bytes, void* stream);
/* qdot_old = qdot; qdd_old = qdd; qdot = (2 - c h)/(2 + c h) qdot_old - 2h/(2 + c h) R/M;
 * qdd = (qdot - qdot_old)/h (solver.py:1020-1022). */
int fem_dr_velocity(int64_t n, double h, double c, const double* R, const double* M, double* qdot, double* qdot_old,
                    double* qdd, double* qdd_old, void* stream);

/* ---- run-time compiled user kernels ---------------------------------------
 * The reference compiles the user's weak-form functions with XLA (jax.jit(jax.vmap(kernel)),
 * problem.py:335-338, including get_universal_kernel at :289-294 and
 * get_universal_kernels_surface at :318-323).  Here the Python layer traces such a function
 * into CUDA C++ and these two calls compile and run it.
 * fem_jit_load: compile `source` with NVRTC for the current device and load it (cached per
 *   source and device); *module receives an opaque handle.  FEM_ERR_ARG carries the compiler log.
 * fem_jit_launch: run the generated kernel `kernel` over n_items cells or faces with the
 *   parameter block P (copied at call time) on `stream`. */
int fem_jit_load(const char* source, void** module);
int fem_jit_launch(void* module, const char* kernel, const fem_jit_params_t* params, int64_t n_items, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* JAXFEM_GB300_H */
