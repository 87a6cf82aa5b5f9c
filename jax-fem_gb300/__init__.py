"""jax_fem_gb300 -- jax-fem's hot path (per-cell weak form, CSR assembly, Krylov solve,
implicit adjoint) written for one NVIDIA GB300 (sm_103a).

Public API mirrors jax_fem: Problem, solver, ad_wrapper, Mesh, box_mesh, ...
The native library libjaxfem_gb300.so (C ABI in include/jaxfem_gb300.h) must be
built first (build.build()); importing the package loads it and fails loudly if
it is absent.
"""
from . import _lib
from .build import build
from .generate_mesh import Mesh, box_mesh, box_mesh_tet10, get_meshio_cell_type
from .materials import (GeneralLinear, J2Plasticity, Laplace, LinearElastic, Material, NeoHookean,
                        SIMPElastic)
from .logger import logger
from .problem import Problem
from .utils import read_vtu, save_sol
from .solver import (ad_wrapper, adjoint_solve, apply_bc_vec, assign_bc, copy_bc, get_A, implicit_vjp,
                     linear_solver, solver, update_j2_history, get_q_vec)

__all__ = ["save_sol", "read_vtu", "Problem", "solver", "ad_wrapper", "implicit_vjp", "update_j2_history", "get_q_vec", "linear_solver", "get_A", "apply_bc_vec",
           "assign_bc", "copy_bc", "adjoint_solve", "Mesh", "box_mesh", "box_mesh_tet10", "get_meshio_cell_type",
           "Laplace", "LinearElastic", "SIMPElastic", "GeneralLinear", "NeoHookean", "J2Plasticity", "Material",
           "logger", "build"]
