"""Reference-element tables, read from the native library (the single source of the
tables the kernels use).  Replaces jax_fem/basis.py:19-250 (basix tabulation) for the
element types built here; node order is meshio's, as in the reference's re_order maps."""
import ctypes as C
import functools

import numpy as np

from . import _lib

# default quadrature orders of jax_fem/basis.py:52-84
DEFAULT_ORDER = {"HEX8": 2, "TET10": 2, "TET4": 0}
MESHIO_TYPE = {"HEX8": "hexahedron", "TET10": "tetra10", "TET4": "tetra"}


@functools.lru_cache(maxsize=None)
def element_tables(ele_type):
    if ele_type not in _lib.ELEM_IDS:
        raise NotImplementedError(f"element type {ele_type!r} is not built on GB300 "
                                  f"(available: {sorted(_lib.ELEM_IDS)})")
    eid = _lib.ELEM_IDS[ele_type]
    nn, nq, nf, nfq = (C.c_int32() for _ in range(4))
    _lib.call("fem_element_info", eid, C.byref(nn), C.byref(nq), C.byref(nf), C.byref(nfq))
    nn, nq, nf, nfq = nn.value, nq.value, nf.value, nfq.value
    nfv = 4 if ele_type == "HEX8" else 3
    N = np.zeros((nq, nn)); dN = np.zeros((nq, nn, 3)); w = np.zeros(nq)
    fN = np.zeros((nf, nfq, nn)); fdN = np.zeros((nf, nfq, nn, 3)); fw = np.zeros((nf, nfq))
    fn = np.zeros((nf, 3)); finds = np.zeros((nf, nfv), dtype=np.int32)
    d = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
    _lib.call("fem_element_tables", eid, d(N), d(dN), d(w), d(fN), d(fdN), d(fw), d(fn),
              finds.ctypes.data_as(C.POINTER(C.c_int32)))
    return dict(shape_vals=N, shape_grads_ref=dN, quad_weights=w, face_shape_vals=fN,
                face_shape_grads_ref=fdN, face_quad_weights=fw, face_normals=fn,
                face_inds=finds.astype(np.int64), elem_id=eid)


def get_elements(ele_type):
    """Subset of jax_fem/basis.py:get_elements: (default quadrature order, meshio cell type)."""
    if ele_type not in DEFAULT_ORDER:
        raise NotImplementedError(ele_type)
    return DEFAULT_ORDER[ele_type], MESHIO_TYPE[ele_type]
