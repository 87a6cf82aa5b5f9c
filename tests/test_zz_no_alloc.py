"""fem_pcg_static: the allocation-free PCG entry point.

It exists for callers that cannot call cudaMalloc themselves: a host framework whose device
allocator is closed to plug-ins, or an embedding that reserves device memory at start-up and
forbids allocation afterwards.  Its scratch is a fixed device array inside the library, so
this file checks it against the workspace-taking fem_pcg on the same system, twice in a row
(the second call reuses the array the first one left behind), for every matrix format and
preconditioner the entry point accepts, and checks that a call leaves the device's free
memory unchanged.  It lives in a file of its own that pytest collects last.
"""
import ctypes as C

import pytest
import torch

pytestmark = pytest.mark.gpu


def _system(cuda, precision=None, nx=8, ny=4, nz=3):
    import cases
    import jax_fem_gb300 as jf
    prob, _, theta_np = cases.simp_box(nx, ny, nz)
    prob.set_params(torch.tensor(theta_np, device=cuda))
    eng = prob._engine
    z = torch.zeros(eng.num_dofs, dtype=torch.float64, device=cuda)
    A = eng.tangent(z, jf._lib.FEM_F64 if precision is None else precision, jf._lib.FEM_BC_SYMMETRIC, cache=False)
    b = (-eng.residual(z, apply_bc=True)).to(A.vector_dtype)
    return jf, eng, A, b


def _static_call(eng, A, pc_kind, pc, b, x, rtol, maxiter=10000):
    from jax_fem_gb300._lib import call, ptr, stream_handle
    it, rn, st = C.c_int64(), C.c_double(), C.c_int32()
    call("fem_pcg_static", C.byref(eng.pattern), eng.num_nodes, eng.vec, A.precision, ptr(A.data), pc_kind,
         ptr(pc), ptr(b), ptr(x), rtol, 0.0, maxiter, C.byref(it), C.byref(rn), C.byref(st), stream_handle())
    return it.value, rn.value, st.value


# (matrix precision, preconditioner, rtol, relative tolerance on x against fem_pcg)
VARIANTS = [
    ("FEM_F64", "FEM_PC_BJACOBI", 1e-12, 1e-12),
    ("FEM_F64", "FEM_PC_JACOBI", 1e-12, 1e-12),
    ("FEM_F64", "FEM_PC_NONE", 1e-12, 1e-12),
    ("FEM_SLICED_F64", "FEM_PC_BJACOBI", 1e-12, 1e-12),
    ("FEM_F32", "FEM_PC_JACOBI", 1e-5, 1e-6),
    ("FEM_SLICED_F32", "FEM_PC_BJACOBI", 1e-5, 1e-6),
]


@pytest.mark.parametrize("prec_name,pc_name,rtol,tol", VARIANTS)
def test_static_pcg_matches_workspace_pcg_twice(cuda, prec_name, pc_name, rtol, tol):
    import jax_fem_gb300 as jf
    jf, eng, A, b = _system(cuda, getattr(jf._lib, prec_name))
    pc_kind = getattr(jf._lib, pc_name)
    x_ref = torch.zeros_like(b)
    it_ref, rn_ref, st_ref = eng.krylov("cg", A, b, x_ref, pc_kind, rtol, 0.0, 10000)
    assert st_ref == jf._lib.FEM_SOLVE_CONVERGED
    pc = A.preconditioner(pc_kind)
    for call_no in range(2):
        x = torch.zeros_like(b)
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info()[0]
        it, rn, st = _static_call(eng, A, pc_kind, pc, b, x, rtol)
        torch.cuda.synchronize()
        free1 = torch.cuda.mem_get_info()[0]
        if call_no == 1:   # the first call may still load kernel modules; the second must allocate nothing
            assert free1 == free0, f"fem_pcg_static changed free device memory by {free0 - free1} bytes"
        assert st == jf._lib.FEM_SOLVE_CONVERGED and it == it_ref
        assert (x - x_ref).abs().max().item() <= tol * x_ref.abs().max().item()
        assert abs(rn - rn_ref) <= tol * max(rn_ref, 1e-300) + 1e-30


def test_static_pcg_rejects_oversize(cuda):
    jf, eng, A, b = _system(cuda, None, 60, 40, 40)          # 61*41*41*3 = 307,623 dofs > 262,144
    assert eng.num_dofs > 262144
    x = torch.zeros_like(b)
    with pytest.raises(jf._lib.FemError) as e:
        _static_call(eng, A, jf._lib.FEM_PC_JACOBI, A.preconditioner(jf._lib.FEM_PC_JACOBI), b, x, 1e-8)
    assert e.value.code == jf._lib.FEM_ERR_CAPACITY and "262144" in str(e.value)
