"""CPU tests: the C-ABI library loads and exports every declared symbol, argument checks
fail loudly without touching a GPU, and the host-side logic (options, Dirichlet / face
detection, user-map probing, meshes) matches the reference's rules."""
import os
import re

import numpy as np
import pytest
import torch

from conftest import ROOT, golden


def _declared():
    names = set()
    for f in os.listdir(os.path.join(ROOT, "include")):
        if f.endswith(".h"):
            src = open(os.path.join(ROOT, "include", f)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names |= set(re.findall(r"\b(fem_[a-z0-9_]+)\s*\(", src))
    return names


def _header_enums():
    """Every `FEM_NAME = value` enumerator in include/*.h (comments stripped)."""
    vals = {}
    for f in os.listdir(os.path.join(ROOT, "include")):
        if f.endswith(".h"):
            src = re.sub(r"/\*.*?\*/", "", open(os.path.join(ROOT, "include", f)).read(), flags=re.S)
            for body in re.findall(r"enum\s*\{(.*?)\}", src, flags=re.S):
                for name, v in re.findall(r"\b(FEM_[A-Z0-9_]+)\s*=\s*(\d+)", body):
                    vals[name] = int(v)
    return vals


def test_python_constants_match_header_enums():
    """The ctypes layer's FEM_* constants equal the header's enumerators (no ABI drift)."""
    import jax_fem_gb300 as jf
    vals = _header_enums()
    assert len(vals) >= 30 and vals["FEM_SOLVE_STAGNATED"] == 4
    for name, v in vals.items():
        assert getattr(jf._lib, name) == v, name
    assert set(jf._lib.SOLVE_STATUS) == {v for k, v in vals.items() if k.startswith("FEM_SOLVE_")}


def test_library_exports_every_declared_symbol(lib):
    names = _declared()
    assert len(names) >= 25
    for n in sorted(names):
        assert hasattr(lib, n), f"{n} declared in include/ but not exported"


def test_signatures_cover_declared(lib):
    import jax_fem_gb300 as jf
    assert _declared() == set(jf._lib.SIGNATURES)


def test_argument_errors_without_gpu(lib):
    import ctypes as C
    import jax_fem_gb300 as jf
    rc = lib.fem_element_info(99, None, None, None, None)
    assert rc == jf._lib.FEM_ERR_ARG
    assert "unknown element" in jf._lib.last_error()
    nb = C.c_size_t()
    jf._lib.call("fem_krylov_workspace", 1000, jf._lib.FEM_F32, C.byref(nb))
    assert nb.value > 8 * 4000
    with pytest.raises(jf._lib.FemError):
        jf._lib.call("fem_krylov_workspace", -1, jf._lib.FEM_F32, C.byref(nb))
    assert lib.fem_version() >= 100
    # in-solve SpMV timing: nothing recorded without a solve; NULL outputs rejected
    sec, cnt = C.c_double(-1.0), C.c_int64(-1)
    assert lib.fem_spmv_timing_start() == jf._lib.FEM_OK
    assert lib.fem_spmv_timing_stop(C.byref(sec), C.byref(cnt)) == jf._lib.FEM_OK
    assert sec.value == 0.0 and cnt.value == 0
    assert lib.fem_spmv_timing_stop(None, None) == jf._lib.FEM_ERR_ARG


def test_widened_entry_points_validate_arguments(lib):
    """The MMA, filter, Robin, history-VJP and driver entry points reject bad arguments with
    FEM_ERR_ARG before touching the device (no GPU needed)."""
    import ctypes as C
    import jax_fem_gb300 as jf
    L = jf._lib
    nb = C.c_size_t()
    L.call("fem_mma_workspace", 1000, 1, C.byref(nb))
    assert nb.value > 8 * 1000 * 17
    assert lib.fem_mma_workspace(1000, 5, C.byref(nb)) == L.FEM_ERR_ARG          # m <= 4
    assert lib.fem_mma_workspace(0, 1, C.byref(nb)) == L.FEM_ERR_ARG
    f = C.c_double(0.0)
    rc = lib.fem_mma_update(3, 4, 1, *([None] * 7), 0.1, None, C.byref(f), None, 1.0, C.byref(f), C.byref(f),
                            C.byref(f), None, None, 0, None, None)
    assert rc == L.FEM_ERR_ARG                                                  # n must exceed m
    L.call("fem_filter_workspace", 100, C.byref(nb))
    assert lib.fem_filter_build(100, None, 0.1, 20, None, None, None, None, 0, None) == L.FEM_ERR_ARG
    assert lib.fem_filter_apply(100, 40, None, None, None, None, None, 1, 0, None, None) == L.FEM_ERR_ARG
    assert lib.fem_dr_march(0, 1.0, None, None, None, None, None, None) == L.FEM_ERR_ARG
    assert lib.fem_row_abs_sum(10, None, None, 1.0, None, None) == L.FEM_ERR_ARG
    mesh = L.FemMesh(L.FEM_HEX8, 3, 8, 1, None, None)
    assert lib.fem_surface_robin(C.byref(mesh), None, None, None, 0, 5, None, 1, L.FEM_F64, None, None, None, 0,
                                 None, None, None, None) == L.FEM_ERR_ARG         # degree <= 4
    assert lib.fem_j2_history_vjp(C.byref(mesh), None, None, None, None, None, None, None, None,
                                  None) == L.FEM_ERR_ARG
    assert "J2" in L.last_error() or "NULL" in L.last_error() or "mesh" in L.last_error()


def test_geometry_cache_and_df_assembly_validate_arguments(lib):
    """fem_cell_geometry and the FEM_DF48 assembly precision reject bad arguments before touching
    the device: NULL outputs, a mesh whose geometry cache sets only one of its two arrays, an
    assembly precision outside FP32 / FP64 / DF48."""
    import ctypes as C
    import jax_fem_gb300 as jf
    L = jf._lib
    empty = L.FemMesh(L.FEM_HEX8, 3, 0, 0, None, None)
    assert lib.fem_cell_geometry(C.byref(empty), None, None, None) == L.FEM_ERR_ARG
    assert "NULL" in L.last_error()
    buf = (C.c_double * 8)()
    assert lib.fem_cell_geometry(C.byref(empty), buf, buf, None) == L.FEM_OK    # no cells: nothing to do
    half = L.FemMesh(L.FEM_HEX8, 3, 8, 1, C.addressof(buf), C.addressof(buf), C.addressof(buf), None)
    mat = L.FemMaterial() if hasattr(L, "FemMaterial") else None
    if mat is not None:
        rc = lib.fem_assemble(C.byref(half), C.byref(mat), None, L.FEM_OUT_RESIDUAL, L.FEM_F64, buf, None, None,
                              L.FEM_BC_NONE, buf, None, None, None)
        assert rc == L.FEM_ERR_ARG and "shape_grads" in L.last_error()
        rc = lib.fem_assemble(C.byref(empty), C.byref(mat), None, L.FEM_OUT_MATRIX, L.FEM_SLICED_DF48, None, None,
                              None, L.FEM_BC_NONE, None, None, None, None)
        assert rc == L.FEM_ERR_ARG and "precision" in L.last_error()


def test_grid_slices_validate_arguments(lib):
    """fem_pattern_slices_grid rejects NULL arrays and a node grid that does not hold n_nodes
    nodes, and the solvers reject a pattern flagged with the grid layout whose slot count or grid
    does not match it, all before touching the device."""
    import ctypes as C
    import jax_fem_gb300 as jf
    L = jf._lib
    buf = (C.c_int64 * 64)()
    a = C.addressof(buf)
    assert lib.fem_pattern_slices_grid(8, a, a, 2, 2, 2, a, None, None) == L.FEM_ERR_ARG
    assert lib.fem_pattern_slices_grid(8, a, a, 2, 2, 3, a, a, None) == L.FEM_ERR_ARG
    assert "grid" in L.last_error()
    pat = L.FemPattern(1, a, a, a, a, a, 1, 26, a, a, 0, None, None, 2, 2, 2, 1)
    y = (C.c_double * 24)()
    assert lib.fem_spmv(C.byref(pat), 8, 3, L.FEM_SLICED_F64, a, y, y, None) == L.FEM_ERR_ARG
    assert "slices_grid" in L.last_error()


def test_structured_grid_detection():
    """structured_grid (the host test behind the grid slice layout and FEM_SSYM_DF48) finds the
    node grid of box_mesh's numbering (z fastest), including one-cell-thick boxes, and refuses
    moved nodes, a permuted numbering and x-fastest numbering."""
    import importlib
    import jax_fem_gb300 as jf
    D = importlib.import_module("jax_fem_gb300.device")
    for n in ((4, 3, 2), (1, 1, 1), (5, 1, 7), (2, 6, 1)):
        m = jf.box_mesh(*n, 2.0, 1.0, 0.5)
        assert D.structured_grid(m.points) == tuple(k + 1 for k in n), n
    pts = np.array(jf.box_mesh(4, 3, 2, 2.0, 1.0, 0.5).points)
    moved = pts.copy()
    moved[7] += 0.01
    assert D.structured_grid(moved) is None
    perm = np.random.default_rng(0).permutation(len(pts))
    assert D.structured_grid(pts[perm]) is None
    g = pts.reshape(5, 4, 3, 3).transpose(2, 1, 0, 3).reshape(-1, 3)   # x fastest
    assert D.structured_grid(g) is None


def test_element_tables_match_oracle(lib):
    from jax_fem_gb300 import basis
    from oracle import basis as ob
    for e in ("HEX8", "TET10", "TET4"):
        t, o = basis.element_tables(e), ob.element_tables(e)
        for k in ("shape_vals", "shape_grads_ref", "quad_weights", "face_shape_vals", "face_shape_grads_ref",
                  "face_quad_weights", "face_normals", "face_inds"):
            np.testing.assert_allclose(t[k], o[k], atol=1e-14)
        # quadrature exactness: weights sum to the reference volume, shape functions partition unity
        assert abs(t["quad_weights"].sum() - (1.0 if e == "HEX8" else 1.0 / 6.0)) < 1e-15
        np.testing.assert_allclose(t["shape_vals"].sum(1), 1.0, atol=1e-14)
        np.testing.assert_allclose(t["shape_grads_ref"].sum(1), 0.0, atol=1e-13)


def test_resolve_solver_options_rules(lib):
    import importlib
    S = importlib.import_module("jax_fem_gb300.solver")
    assert S._resolve_solver_options({}) == ("newton", {})
    m, cfg = S._resolve_solver_options({"petsc_solver": {}, "tol": 1e-5})
    assert m == "newton" and cfg == {"linear": {"petsc_solver": {}}, "tol": 1e-5}
    with pytest.raises(ValueError):
        S._resolve_solver_options({"newton": {}, "arc_length": {}})
    with pytest.raises(ValueError):
        S._resolve_solver_options({"newton": 3})
    spec = S.resolve_linear({})
    assert spec.method == "bicgstab" and spec.rtol == 1e-10 and spec.atol == 1e-10 and spec.maxiter == 10000
    spec = S.resolve_linear({"petsc_solver": {"ksp_type": "cg", "pc_type": "jacobi"}})
    assert spec.method == "cg" and spec.rtol == 1e-5
    with pytest.raises(NotImplementedError):
        S.resolve_linear({"amgx_solver": {}})


def test_dirichlet_and_faces_match_oracle(lib):
    from jax_fem_gb300.fe import FiniteElement
    from jax_fem_gb300.generate_mesh import Mesh
    from oracle import fem as ofem
    g = golden("plasticity")
    top = lambda p: np.isclose(p[2], 10.0, atol=1e-5)
    bottom = lambda p: np.isclose(p[2], 0.0, atol=1e-5)
    both = lambda p, i: np.logical_and(np.isclose(p[2], 0.0, atol=1e-5), i % 2 == 0)
    bc = [[bottom, top, both], [0, 2, 1], [lambda p: 0.0, lambda p: 0.1 * p[0], lambda p: 2.0]]
    fe = FiniteElement(Mesh(g["points"], g["cells"]), 3, 3, "HEX8", dirichlet_bc_info=bc)
    ofe = ofem.OracleFE(g["points"], g["cells"], 3, "HEX8", dirichlet_bc_info=bc)
    for a, b in zip(fe.node_inds_list, ofe.node_inds_list):
        np.testing.assert_array_equal(a, b)
    for a, b in zip(fe.vals_list, ofe.vals_list):
        np.testing.assert_allclose(a, b, rtol=0, atol=0)
    for a, b in zip(fe.get_boundary_conditions_inds([top, bottom]), ofe.get_boundary_conditions_inds([top, bottom])):
        np.testing.assert_array_equal(a, b)


def test_probe_tensor_map(lib):
    import jax_fem_gb300 as jf
    from jax_fem_gb300.materials import probe_tensor_map

    def elastic(u_grad):
        E, nu = 70e3, 0.3
        mu = E / (2 * (1 + nu))
        lm = E * nu / ((1 + nu) * (1 - 2 * nu))
        eps = 0.5 * (u_grad + u_grad.T)
        return lm * np.trace(eps) * np.eye(3) + 2 * mu * eps

    m = probe_tensor_map(elastic, 3)
    assert isinstance(m, jf.LinearElastic)
    assert abs(m.E - 70e3) < 1e-9 and abs(m.nu - 0.3) < 1e-14
    assert isinstance(probe_tensor_map(lambda x: x, 1), jf.Laplace)
    aniso = np.diag([1.0, 2.0, 3.0])
    assert isinstance(probe_tensor_map(lambda g: (aniso @ g.T).T, 1), jf.GeneralLinear)
    with pytest.raises(NotImplementedError):
        probe_tensor_map(lambda g: g ** 3, 3)
    with pytest.raises(NotImplementedError):
        probe_tensor_map(lambda g, theta: g * theta, 3)


def test_box_meshes(lib):
    import jax_fem_gb300 as jf
    from oracle import fem as ofem
    m = jf.box_mesh(3, 4, 5, 1.0, 2.0, 3.0)
    p, c = ofem.box_mesh(3, 4, 5, 1.0, 2.0, 3.0)
    np.testing.assert_array_equal(m.points, p)
    np.testing.assert_array_equal(m.cells_dict["hexahedron"], c)
    t = jf.box_mesh_tet10(2, 2, 2, 1.0, 1.0, 1.0)
    pts, cells = t.points, t.cells_dict["tetra10"]
    assert cells.shape == (48, 10) and len(pts) == 27 + 98
    P = pts[cells]
    vol = np.einsum("ij,ij->i", np.cross(P[:, 1] - P[:, 0], P[:, 2] - P[:, 0]), P[:, 3] - P[:, 0]) / 6
    assert np.all(vol > 0) and abs(vol.sum() - 1.0) < 1e-12
    # midpoints lie halfway along their edges
    for k, (a, b) in enumerate([(0, 1), (1, 2), (0, 2), (0, 3), (1, 3), (2, 3)]):
        np.testing.assert_allclose(P[:, 4 + k], 0.5 * (P[:, a] + P[:, b]), atol=1e-15)


def test_pointwise_eval_falls_back(lib):
    from jax_fem_gb300.fe import eval_pointwise
    x = np.random.default_rng(0).standard_normal((20, 3))
    f1 = lambda p: np.linalg.norm(p)                    # not vectorisable by axis trick
    np.testing.assert_allclose(eval_pointwise(f1, [x]), np.linalg.norm(x, axis=1))
    f2 = lambda p: -np.array([1e3 * p[0], 2e3 * p[1], 3e3 * p[2]])
    np.testing.assert_allclose(eval_pointwise(f2, [x], (3,)), -x * np.array([1e3, 2e3, 3e3]))
    f3 = lambda p: np.array([0.0, 10.0, 10.0])
    assert eval_pointwise(f3, [x], (3,)).shape == (20, 3)


def test_surface_map_split_probe():
    """u-dependent surface maps: component-wise polynomials (here the Robin example's 5 u^2 and a
    linear spring with an x-dependent load) are split into h(x) + sum_k c_k u^k; non-polynomial
    or coupled u-dependence is refused loudly."""
    import importlib
    import numpy as np
    import pytest
    P = importlib.import_module("jax_fem_gb300.problem")
    x = np.random.default_rng(0).uniform(0, 1, (12, 3))
    h, c = P._surface_map_split(lambda u, xx: 5.0 * u ** 2, x, 1)
    assert np.allclose(h, 0.0) and c.shape == (1, 3) and np.allclose(c, [[0, 0, 5.0]])
    h, c = P._surface_map_split(lambda u, xx: 100.0 * u + np.array([0.0, 0.0, -xx[0]]), x, 3)
    assert np.allclose(h.reshape(-1, 3)[:, 2], -x[:, 0]) and c.shape == (3, 2) and np.allclose(c[:, 1], 100.0)
    h, c = P._surface_map_split(lambda u, xx: np.array([0.0, 1.0, 2.0]), x, 3)
    assert c is None and np.allclose(h.reshape(-1, 3), [0.0, 1.0, 2.0])
    with pytest.raises(NotImplementedError):
        P._surface_map_split(lambda u, xx: np.sin(u), x, 1)
    with pytest.raises(NotImplementedError):
        P._surface_map_split(lambda u, xx: np.array([u[0] * u[1], 0.0, 0.0]), x, 3)


def test_map_probes_see_local_u_dependence():
    """A mass or surface map that depends on u only on part of the domain (here x < 0.5) must be
    refused, not integrated as a constant load: the probes check every quadrature point.  Maps
    written with per-point branching (not vectorisable) and vectorised ones are both covered."""
    import importlib
    P = importlib.import_module("jax_fem_gb300.problem")
    x = np.random.default_rng(1).uniform(0, 1, (400, 3))
    loc_branch = lambda u, xx: np.array([0.0, 0.0, 1.0]) + (u if xx[0] < 0.5 else 0.0 * u)
    loc_vector = lambda u, xx: np.array([0.0 * u[0], 0.0 * u[1], 1.0 + 0.0 * u[2]]) + u * (xx[0] < 0.5)
    for fn in (loc_branch, loc_vector):
        with pytest.raises(NotImplementedError):
            P._u_independent(fn, x, 3, "mass map")
    # u only on half of the faces, linear there: not x-independent, so refused as a Robin map too
    with pytest.raises(NotImplementedError):
        P._surface_map_split(loc_branch, x, 3)
    # genuinely u-independent maps still pass and return their values at every point
    val = P._u_independent(lambda u, xx: np.array([xx[0], 0.0, -1.0]), x, 3, "mass map").reshape(-1, 3)
    assert np.allclose(val[:, 0], x[:, 0]) and np.allclose(val[:, 2], -1.0)


@pytest.mark.parametrize("binary", [True, False])
def test_save_sol_vtu_round_trip(tmp_path, binary):
    """save_sol (utils.py:13-57) writes a VTU whose points, cells, 'sol' (float32) and cell /
    point data read back unchanged, for HEX8 and TET10 meshes."""
    import importlib
    import numpy as np
    jf = importlib.import_module("jax_fem_gb300")
    U = importlib.import_module("jax_fem_gb300.utils")
    FE = importlib.import_module("jax_fem_gb300.fe")
    for m, et, key in ((jf.box_mesh(3, 2, 2, 1.0, 1.0, 1.0), "HEX8", "hexahedron"),
                       (jf.box_mesh_tet10(2, 2, 1, 1.0, 1.0, 1.0), "TET10", "tetra10")):
        fe = FE.FiniteElement(jf.Mesh(m.points, m.cells_dict[key]), vec=3, dim=3, ele_type=et)
        rng = np.random.default_rng(0)
        sol = rng.standard_normal((fe.num_total_nodes, 3))
        theta = rng.uniform(size=fe.num_cells)
        T = rng.uniform(size=fe.num_total_nodes)
        path = tmp_path / f"{et}_{binary}.vtu"
        U.save_sol(fe, sol, str(path), cell_infos=[("theta", theta)], point_infos=[("T", T)], binary=binary)
        pts, cells, pd, cd = U.read_vtu(str(path))
        np.testing.assert_array_equal(pts, fe.points)
        np.testing.assert_array_equal(cells[key], fe.cells)
        np.testing.assert_array_equal(pd["sol"], sol.astype(np.float32))
        np.testing.assert_array_equal(pd["T"], T.astype(np.float32))
        np.testing.assert_array_equal(cd["theta"], theta.astype(np.float32))
