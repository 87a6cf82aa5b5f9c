"""fem_pcg_static: the allocation-free PCG entry point.

It exists for callers that cannot call cudaMalloc themselves (a stream under CUDA-graph
capture, a host framework with a closed allocator, an embedding that forbids allocation
after start-up).  Its scratch is a fixed device array inside the library, so this file
checks it against the workspace-taking fem_pcg on the same system, twice in a row (the
second call reuses the array the first one left behind).  It lives in a file of its own
that pytest collects last.
"""
import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _system(cuda, nx=8, ny=4, nz=3):
    import cases
    import jax_fem_gb300 as jf
    prob, _, theta_np = cases.simp_box(nx, ny, nz)
    prob.set_params(torch.tensor(theta_np, device=cuda))
    eng = prob._engine
    z = torch.zeros(eng.num_dofs, dtype=torch.float64, device=cuda)
    A = eng.tangent(z, jf._lib.FEM_F64, jf._lib.FEM_BC_SYMMETRIC, cache=False)
    b = -eng.residual(z, apply_bc=True)
    return jf, eng, A, b


def _static_solve(jf, eng, A, b, pc_kind, rtol, maxiter=10000):
    from jax_fem_gb300._lib import call, ptr, stream_handle
    x = torch.zeros_like(b)
    pc = A.preconditioner(pc_kind)
    it, rn, st = C.c_int64(), C.c_double(), C.c_int32()
    call("fem_pcg_static", C.byref(eng.pattern), eng.num_nodes, eng.vec, A.precision, ptr(A.data), pc_kind,
         ptr(pc), ptr(b), ptr(x), rtol, 0.0, maxiter, C.byref(it), C.byref(rn), C.byref(st), stream_handle())
    return x, it.value, rn.value, st.value


def test_static_pcg_matches_workspace_pcg_twice(cuda):
    jf, eng, A, b = _system(cuda)
    pc_kind = jf._lib.FEM_PC_BJACOBI
    x_ref = torch.zeros_like(b)
    it_ref, rn_ref, st_ref = eng.krylov("cg", A, b, x_ref, pc_kind, 1e-12, 0.0, 10000)
    assert st_ref == jf._lib.FEM_SOLVE_CONVERGED
    for _ in range(2):
        x, it, rn, st = _static_solve(jf, eng, A, b, pc_kind, 1e-12)
        assert st == jf._lib.FEM_SOLVE_CONVERGED and it == it_ref
        assert (x - x_ref).abs().max().item() <= 1e-12 * x_ref.abs().max().item()
        assert abs(rn - rn_ref) <= 1e-12 * max(rn_ref, 1e-300) + 1e-30


def test_static_pcg_rejects_oversize(cuda):
    jf, eng, A, b = _system(cuda, 60, 40, 40)          # 61*41*41*3 = 307,623 dofs > 262,144
    assert eng.num_dofs > 262144
    with pytest.raises(jf._lib.FemError) as e:
        _static_solve(jf, eng, A, b, jf._lib.FEM_PC_JACOBI, 1e-8)
    assert e.value.code == jf._lib.FEM_ERR_CAPACITY and "262144" in str(e.value)
