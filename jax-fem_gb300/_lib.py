"""ctypes binding of libjaxfem_gb300.so (the C ABI in include/jaxfem_gb300.h).

The library is loaded from this package directory; if it is missing the import
fails loudly -- there is no CPU fallback for any hot-path operation.
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libjaxfem_gb300.so")

# ---- constants mirrored from the header --------------------------------------
FEM_OK, FEM_ERR_ARG, FEM_ERR_CUDA, FEM_ERR_UNSUPPORTED, FEM_ERR_CAPACITY, FEM_ERR_DEVICE = range(6)
FEM_HEX8, FEM_TET10, FEM_TET4 = 1, 2, 3
FEM_F32, FEM_F64, FEM_DF48, FEM_SLICED_F32, FEM_SLICED_F64, FEM_SLICED_DF48, FEM_SYM_DF48, FEM_SSYM_DF48 = range(8)
(FEM_MAT_LAPLACE, FEM_MAT_LINEAR_ELASTIC, FEM_MAT_SIMP, FEM_MAT_GENERAL_LINEAR,
 FEM_MAT_NEO_HOOKEAN, FEM_MAT_J2) = range(1, 7)
FEM_OUT_RESIDUAL, FEM_OUT_MATRIX, FEM_OUT_APPLY, FEM_OUT_PARAM_VJP = 1, 2, 4, 8
FEM_BC_NONE, FEM_BC_ROWS, FEM_BC_SYMMETRIC = 0, 1, 2
FEM_PC_NONE, FEM_PC_JACOBI, FEM_PC_BJACOBI = 0, 1, 2
FEM_SOLVE_CONVERGED, FEM_SOLVE_MAXITER, FEM_SOLVE_BREAKDOWN, FEM_SOLVE_NAN, FEM_SOLVE_STAGNATED = range(5)
SOLVE_STATUS = {0: "converged", 1: "maxiter", 2: "breakdown", 3: "nan", 4: "stagnated"}

ELEM_IDS = {"HEX8": FEM_HEX8, "TET10": FEM_TET10, "TET4": FEM_TET4}


class FemError(RuntimeError):
    """Raised when a C-ABI call returns a non-zero status."""

    def __init__(self, code, func, msg):
        super().__init__(f"{func} failed (code {code}): {msg}")
        self.code = code


class FemMesh(C.Structure):
    _fields_ = [("elem_type", C.c_int32), ("vec", C.c_int32), ("n_nodes", C.c_int64), ("n_cells", C.c_int64),
                ("coords", C.c_void_p), ("conn", C.c_void_p), ("shape_grads", C.c_void_p), ("jxw", C.c_void_p)]


class FemPattern(C.Structure):
    _fields_ = [("nnzb", C.c_int64), ("block_ptr", C.c_void_p), ("block_cols", C.c_void_p),
                ("indptr", C.c_void_p), ("diag", C.c_void_p), ("slots", C.c_void_p),
                ("n_slices", C.c_int64), ("n_slots", C.c_int64), ("slice_ptr", C.c_void_p),
                ("slice_cols", C.c_void_p), ("n_slots_u", C.c_int64), ("slice_ptr_u", C.c_void_p),
                ("slice_cols_u", C.c_void_p), ("grid_nx", C.c_int64), ("grid_ny", C.c_int64),
                ("grid_nz", C.c_int64), ("slices_grid", C.c_int64)]


class FemJitParams(C.Structure):
    _fields_ = [("coords", C.c_void_p), ("conn", C.c_void_p), ("n_items", C.c_int64), ("face_cells", C.c_void_p),
                ("face_ids", C.c_void_p), ("u", C.c_void_p), ("w", C.c_void_p), ("lam", C.c_void_p),
                ("iv", C.c_void_p), ("iv_stride", C.c_int64), ("indptr", C.c_void_p), ("slots", C.c_void_p),
                ("bc", C.c_void_p), ("bc_mode", C.c_int64), ("outputs", C.c_int64), ("res", C.c_void_p),
                ("vals", C.c_void_p), ("apply_out", C.c_void_p), ("vjp_out", C.c_void_p)]


class FemMaterial(C.Structure):
    _fields_ = [("kind", C.c_int32), ("n_consts", C.c_int32), ("consts", C.POINTER(C.c_double)),
                ("n_qp_params", C.c_int32), ("qp_params", C.c_void_p), ("history", C.c_void_p)]


P = C.c_void_p
I32, I64, F64, SZ = C.c_int32, C.c_int64, C.c_double, C.c_size_t
PI64 = C.POINTER(C.c_int64)
PI32 = C.POINTER(C.c_int32)
PF64 = C.POINTER(C.c_double)
PSZ = C.POINTER(C.c_size_t)
PMESH, PPAT, PMAT = C.POINTER(FemMesh), C.POINTER(FemPattern), C.POINTER(FemMaterial)

SIGNATURES = {
    "fem_last_error": ([], C.c_char_p),
    "fem_version": ([], C.c_int),
    "fem_kernel_launches": ([], C.c_uint64),
    "fem_element_info": ([I32, PI32, PI32, PI32, PI32], C.c_int),
    "fem_element_tables": ([I32, PF64, PF64, PF64, PF64, PF64, PF64, PF64, PI32], C.c_int),
    "fem_pattern_workspace": ([I64, I32, I64, PSZ], C.c_int),
    "fem_pattern_count": ([I32, P, I64, I64, P, SZ, P, PI64, P], C.c_int),
    "fem_pattern_fill": ([I32, P, I64, I64, P, SZ, P, P, P], C.c_int),
    "fem_pattern_slots": ([I32, P, I64, P, P, P, P], C.c_int),
    "fem_pattern_scalar": ([I64, I32, P, P, P, P, P, P], C.c_int),
    "fem_quad_points": ([PMESH, P, P, P], C.c_int),
    "fem_cell_geometry": ([PMESH, P, P, P], C.c_int),
    "fem_face_quad_points": ([PMESH, P, P, I64, P, P, P], C.c_int),
    "fem_body_load": ([PMESH, P, P, P], C.c_int),
    "fem_surface_load": ([PMESH, P, P, I64, P, P, P], C.c_int),
    "fem_surface_robin": ([PMESH, PPAT, P, P, I64, I32, PF64, I32, I32, P, P, P, I32, P, P, P, P], C.c_int),
    "fem_assemble": ([PMESH, PMAT, PPAT, I32, I32, P, P, P, I32, P, P, P, P], C.c_int),
    "fem_param_vjp": ([PMESH, PMAT, P, P, P, P, P], C.c_int),
    "fem_j2_update": ([PMESH, PMAT, P, P, P], C.c_int),
    "fem_j2_history_vjp": ([PMESH, PMAT, P, P, P, P, P, P, P, P], C.c_int),
    "fem_zero_rows": ([PPAT, I32, I32, P, P, I64, F64, P], C.c_int),
    "fem_apply_bc_vec": ([P, P, P, P, I64, F64, P], C.c_int),
    "fem_matrix_transpose": ([PPAT, I64, I32, I32, P, P, P, SZ, P], C.c_int),
    "fem_spmv": ([PPAT, I64, I32, I32, P, P, P, P], C.c_int),
    "fem_precond_setup": ([PPAT, I64, I32, I32, P, I32, P, P], C.c_int),
    "fem_krylov_workspace": ([I64, I32, PSZ], C.c_int),
    "fem_pcg": ([PPAT, I64, I32, I32, P, I32, P, P, P, F64, F64, I64, P, SZ, PI64, PF64, PI32, P], C.c_int),
    "fem_pcg_static": ([PPAT, I64, I32, I32, P, I32, P, P, P, F64, F64, I64, PI64, PF64, PI32, P], C.c_int),
    "fem_bicgstab": ([PPAT, I64, I32, I32, P, I32, P, P, P, F64, F64, I64, P, SZ, PI64, PF64, PI32, P], C.c_int),
    "fem_pcg_refined": ([PPAT, I64, I32, I32, P, I32, P, PMESH, PMAT, P, P, I32, P, P, P, F64, F64, F64, I64, P, SZ,
                         PI64, PI64, PF64, PI32, P], C.c_int),
    "fem_pattern_slices": ([I64, P, P, P, P, PI64, P], C.c_int),
    "fem_pattern_slices_grid": ([I64, P, P, I64, I64, I64, P, P, P], C.c_int),
    "fem_matrix_bytes": ([PPAT, I32, I32, PSZ], C.c_int),
    "fem_matrix_convert": ([PPAT, I64, I32, P, I32, P, P], C.c_int),
    "fem_vector_split": ([P, I64, P, P], C.c_int),
    "fem_spmv_dfx": ([PPAT, I64, I32, I32, P, P, P, P, P, P, SZ, P], C.c_int),
    "fem_pattern_slices_upper": ([I64, P, P, P, P, PI64, P], C.c_int),
    "fem_cast_f64_f32": ([P, P, I64, P, P], C.c_int),
    "fem_axpy_f32_f64": ([F64, P, P, I64, P], C.c_int),
    "fem_dot": ([I32, P, P, I64, P, P, SZ, P], C.c_int),
    "fem_selftest_bounded_wait": ([P, SZ, P], C.c_int),
    "fem_spmv_timing_start": ([], C.c_int),
    "fem_spmv_timing_stop": ([PF64, PI64], C.c_int),
    "fem_row_abs_sum": ([I64, P, P, F64, P, P], C.c_int),
    "fem_dr_march": ([I64, F64, P, P, P, P, P, P], C.c_int),
    "fem_dr_measure": ([I64, F64, F64, P, P, P, P, P, P, P, P, PF64, P, SZ, P], C.c_int),
    "fem_dr_velocity": ([I64, F64, F64, P, P, P, P, P, P, P], C.c_int),
    "fem_mma_workspace": ([I64, I32, PSZ], C.c_int),
    "fem_mma_update": ([I64, I32, I32, P, P, P, P, P, P, P, F64, P, PF64, P, F64, PF64, PF64, PF64, P, P, SZ, PI32, P],
                       C.c_int),
    "fem_filter_workspace": ([I64, PSZ], C.c_int),
    "fem_filter_build": ([I64, P, F64, I32, P, P, P, P, SZ, P], C.c_int),
    "fem_filter_apply": ([I64, I32, P, P, P, P, P, I32, I32, P, P], C.c_int),
    "fem_jit_load": ([C.c_char_p, C.POINTER(C.c_void_p)], C.c_int),
    "fem_jit_launch": ([P, C.c_char_p, C.POINTER(FemJitParams), I64, P], C.c_int),
}

_lib = None


def load():
    """Load the library (once) and attach argument types. Raises if it is absent."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(
            f"{LIB_PATH} is missing: build the sm_103a library first "
            "(python -c 'import __graft_entry__ as g; g.build()'); there is no CPU fallback.")
    lib = C.CDLL(LIB_PATH)
    for name, (args, res) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    _lib = lib
    return lib


def last_error():
    return load().fem_last_error().decode(errors="replace")


def call(name, *args):
    """Call a C-ABI entry point and raise FemError on a non-zero status."""
    lib = load()
    rc = getattr(lib, name)(*args)
    if rc != FEM_OK:
        raise FemError(rc, name, last_error())
    return rc


def ptr(t):
    """Raw device (or host) pointer of a torch tensor, or None."""
    return None if t is None else C.c_void_p(t.data_ptr())


def stream_handle(stream=None):
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    return C.c_void_p(s.cuda_stream)
