"""Cached per-cell geometry (fem_cell_geometry) and the double-float matrix assembly (fem_assemble
with FEM_DF48), against the oracle and the FP64 kernels:
- the cached physical shape gradients and JxW equal the oracle's restatement of
  get_shape_grads (fe.py:112-141, kept by problem.py:130-147) on a distorted HEX8 mesh (1e-12);
- the cell kernels give the same residual, FP64 tangent, tangent action and parameter VJP with
  and without the cache (1e-13);
- the double-float isotropic tangent (SIMP and linear elastic; HEX8, TET10 and TET4; every
  Dirichlet mode) equals the FP64 tangent to 1e-13 of max|K| (its values carry ~2^-46 rounding
  against FP64's 2^-53), and a mixed solve whose DF48 copy comes from it matches FP64."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _distorted_simp(nx=6, ny=4, nz=3, seed=0):
    """SIMP cantilever on a box mesh whose nodes off the x = 0 and x = Lx planes are moved by up to
    20% of the cell size in every direction."""
    import jax_fem_gb300 as jf
    from oracle import fem as ofem, materials as omat
    Lx, Ly, Lz = 2.0, 1.0, 0.5
    m = jf.box_mesh(nx, ny, nz, Lx, Ly, Lz)
    pts = np.array(m.points, dtype=np.float64)
    cells = m.cells_dict["hexahedron"]
    rng = np.random.default_rng(seed)
    inner = (pts[:, 0] > 1e-9) & (pts[:, 0] < Lx - 1e-9)
    h = np.array([Lx / nx, Ly / ny, Lz / nz])
    pts[inner] += rng.uniform(-0.2, 0.2, (inner.sum(), 3)) * h
    left = lambda p: np.isclose(p[0], 0.0, atol=1e-5)
    right = lambda p: np.isclose(p[0], Lx, atol=1e-5)
    bc = [[left] * 3, [0, 1, 2], [lambda p: 0.0] * 3]

    class P(jf.Problem):
        def get_tensor_map(self):
            return jf.SIMPElastic(1.0, 1e-3, 0.3, 3.0)

        def get_surface_maps(self):
            return [lambda u, x: np.array([0.0, 0.0, 1.0])]

        def set_params(self, params):
            self.internal_vars = [params]

    prob = P(jf.Mesh(pts, cells), vec=3, dim=3, dirichlet_bc_info=bc, location_fns=[right])
    theta = 0.5 + np.random.default_rng(seed + 1).uniform(-0.3, 0.3, (len(cells), 8, 1))
    return prob, pts, cells, theta


def _without_cache(eng, fn):
    """fn() evaluated with the mesh's geometry cache detached (the kernels recompute it)."""
    sg, jw = eng.mesh.shape_grads, eng.mesh.jxw
    eng.mesh.shape_grads = eng.mesh.jxw = None
    try:
        return fn()
    finally:
        eng.mesh.shape_grads, eng.mesh.jxw = sg, jw


def test_cell_geometry_matches_oracle(cuda):
    from oracle import fem as ofem
    prob, pts, cells, _ = _distorted_simp()
    eng = prob._engine
    assert eng.shape_grads is not None, "geometry cache not built"
    fe = ofem.OracleFE(pts, cells, 3)
    g = eng.shape_grads.view(eng.num_cells, eng.num_quads, eng.nn, 3).cpu().numpy()
    j = eng.jxw.view(eng.num_cells, eng.num_quads).cpu().numpy()
    assert np.abs(g - fe.shape_grads).max() <= 1e-12 * np.abs(fe.shape_grads).max()
    assert np.abs(j - fe.JxW).max() <= 1e-12 * np.abs(fe.JxW).max()


def test_cached_geometry_gives_the_same_kernels(cuda):
    import jax_fem_gb300 as jf
    L = jf._lib
    prob, _, _, theta = _distorted_simp(seed=2)
    prob.set_params(torch.tensor(theta, device=cuda))
    eng = prob._engine
    rng = np.random.default_rng(5)
    u = torch.tensor(rng.standard_normal(eng.num_dofs) * 1e-2, device=cuda)
    w = torch.tensor(rng.standard_normal(eng.num_dofs), device=cuda)

    def evaluate():
        r = prob.compute_residual([u.reshape(-1, 3)])[0].reshape(-1).clone()
        K = eng.tangent(u, L.FEM_F64, L.FEM_BC_ROWS, cache=False).data.clone()
        a = eng.apply(u, w).clone()
        v = eng.param_vjp(u, w).clone() if hasattr(eng, "param_vjp") else None
        return r, K, a, v

    cached = evaluate()
    plain = _without_cache(eng, evaluate)
    for x, y, name in zip(cached, plain, ("residual", "tangent", "apply", "vjp")):
        if x is None:
            continue
        assert (x - y).abs().max().item() <= 1e-13 * y.abs().max().item(), name


@pytest.mark.parametrize("bc_mode", [0, 1, 2])
def test_df_tangent_simp_hex8(cuda, bc_mode):
    import jax_fem_gb300 as jf
    L = jf._lib
    prob, _, _, theta = _distorted_simp(seed=3)
    prob.set_params(torch.tensor(theta, device=cuda))
    eng = prob._engine
    z = torch.zeros(eng.num_dofs, dtype=torch.float64, device=cuda)
    K64 = eng.tangent(z, L.FEM_F64, bc_mode, cache=False).data
    Kdf = eng.tangent(z, L.FEM_F64, bc_mode, cache=False, df_source=True).data
    assert Kdf.data_ptr() != K64.data_ptr()
    err = (Kdf - K64).abs().max().item() / K64.abs().max().item()
    assert 0 < err <= 1e-13, err     # computed differently (0 would mean the FP64 kernel ran)
    # without the geometry cache (a mesh too large for it) the double-float request falls back to
    # the FP64 kernel and still gives the tangent (the atomics' order makes equality bitwise loose)
    Kfb = _without_cache(eng, lambda: eng.tangent(z, L.FEM_F64, bc_mode, cache=False, df_source=True).data.clone())
    assert (Kfb - K64).abs().max().item() <= 1e-13 * K64.abs().max().item()


def test_df_tangent_linear_elastic_tet10_tet4(cuda):
    import jax_fem_gb300 as jf
    L = jf._lib
    m = jf.box_mesh_tet10(3, 3, 2, 1.0, 1.0, 0.5)
    pts10, cells10 = np.asarray(m.points), np.asarray(m.cells_dict["tetra10"])
    nv = 4 * 4 * 3
    x0 = lambda p: np.isclose(p[0], 0.0, atol=1e-5)
    bc = [[x0] * 3, [0, 1, 2], [lambda p: 0.0] * 3]

    class P(jf.Problem):
        def get_tensor_map(self):
            return jf.LinearElastic(70e3, 0.3)

    for pts, cells, ele in ((pts10, cells10, "TET10"), (pts10[:nv], cells10[:, :4], "TET4")):
        prob = P(jf.Mesh(pts, cells), vec=3, dim=3, ele_type=ele, dirichlet_bc_info=bc)
        eng = prob._engine
        z = torch.zeros(eng.num_dofs, dtype=torch.float64, device=cuda)
        for mode in (L.FEM_BC_NONE, L.FEM_BC_SYMMETRIC):
            K64 = eng.tangent(z, L.FEM_F64, mode, cache=False).data
            Kdf = eng.tangent(z, L.FEM_F64, mode, cache=False, df_source=True).data
            err = (Kdf - K64).abs().max().item() / K64.abs().max().item()
            assert 0 < err <= 1e-13, (ele, mode, err)


def test_mixed_solve_with_df_assembled_copy(cuda):
    """The mixed path now splits its DF48 copy from the double-float tangent: solution, objective
    and gradient still match FP64 on the distorted mesh (as test_mixed_precision_matches_fp64)."""
    import jax_fem_gb300 as jf
    prob, _, _, theta = _distorted_simp(8, 4, 4, seed=4)
    eng = prob._engine

    def run(prec):
        o = {"petsc_solver": {"ksp_type": "cg", "pc_type": "bjacobi", "rtol": 1e-12}, "rel_tol": 1e-12, "tol": 0.0,
             "precision": prec}
        a = {"petsc_solver": {"ksp_type": "cg", "pc_type": "bjacobi", "rtol": 1e-12}, "precision": prec}
        fwd = jf.ad_wrapper(prob, o, a)
        th = torch.tensor(theta, device=cuda, requires_grad=True)
        sol = fwd(th)[0]
        J = torch.dot(eng.f_ext, sol.reshape(-1))
        J.backward()
        return sol.detach(), J.item(), th.grad.cpu().numpy()

    s64, J64, g64 = run("fp64")
    eng.solve_log.clear()
    smx, Jmx, gmx = run("mixed")
    assert any(r["method"] == "cg-refined" for r in eng.solve_log)
    assert (smx - s64).abs().max().item() <= 1e-9 * s64.abs().max().item()
    assert abs(Jmx - J64) <= 1e-10 * abs(J64)
    assert np.abs(gmx - g64).max() <= 1e-8 * np.abs(g64).max()
