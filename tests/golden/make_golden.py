"""Extract the reference's own FEniCSx gold fixtures into small compressed npz files.

Run, where a checkout of the reference (deepmodeling/jax-fem) is available, with

    python tests/golden/make_golden.py <path to the reference checkout>

It reads the ASCII VTU files and .npy arrays that the reference's regression
tests compare against (tests/benchmarks/*/fenicsx/) and writes
tests/golden/<case>.npz holding the mesh (points, cells), the gold solution
and the scalar gold quantities.  Nothing else from the reference is copied.

Reference tests that consume these files:
  tests/benchmarks/linear_poisson/test_linear_poisson.py:27-65
  tests/benchmarks/linear_elasticity_cube/test_linear_elasticity_cube.py:45-83
  tests/benchmarks/linear_elasticity_cylinder/test_linear_elasticity_cylinder.py:85-132
  tests/benchmarks/hyperelasticity/test_hyper_elasticity.py:79-127
  tests/benchmarks/plasticity/test_plasticity.py:96-161
"""
import os
import sys
import xml.etree.ElementTree as ET

import numpy as np

CASES = {
    "linear_poisson": [],
    "linear_elasticity_cube": [],
    "linear_elasticity_cylinder": ["surface_area.npy"],
    "hyperelasticity": ["traction.npy"],
    "plasticity": ["disps.npy", "avg_stresses.npy"],
}


def read_vtu(path):
    root = ET.parse(path).getroot()
    piece = root.find("UnstructuredGrid/Piece")
    pts = piece.find("Points/DataArray")
    points = np.array(pts.text.split(), dtype=np.float64).reshape(-1, 3)
    arrays = {da.get("Name"): da for da in piece.find("Cells").findall("DataArray")}
    conn = np.array(arrays["connectivity"].text.split(), dtype=np.int64)
    offsets = np.array(arrays["offsets"].text.split(), dtype=np.int64)
    types = np.array(arrays["types"].text.split(), dtype=np.int64)
    nper = np.diff(np.concatenate([[0], offsets]))
    assert np.all(nper == 8), "expected 8-node hexahedra"
    # VTK_LAGRANGE_HEXAHEDRON (72) with 8 nodes has the VTK hexahedron corner order
    assert np.all(types == 72)
    cells = conn.reshape(-1, 8)
    sol = None
    for da in piece.find("PointData").findall("DataArray"):
        if da.get("Name") == "sol":
            ncomp = int(da.get("NumberOfComponents", "1"))
            sol = np.array(da.text.split(), dtype=np.float64).reshape(-1, ncomp)
    return points, cells, sol


def main(ref_root):
    out_dir = os.path.dirname(os.path.abspath(__file__))
    for case, extras in CASES.items():
        d = os.path.join(ref_root, "tests", "benchmarks", case, "fenicsx")
        points, cells, sol = read_vtu(os.path.join(d, "sol_p0_000000.vtu"))
        payload = dict(points=points, cells=cells.astype(np.int32), sol=sol)
        for e in extras:
            payload[e[:-4]] = np.atleast_1d(np.load(os.path.join(d, e)))
        np.savez_compressed(os.path.join(out_dir, case + ".npz"), **payload)
        print(case, points.shape, cells.shape, None if sol is None else sol.shape,
              {k: v for k, v in payload.items() if k not in ("points", "cells", "sol")})


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path to the reference checkout>")
    main(sys.argv[1])
