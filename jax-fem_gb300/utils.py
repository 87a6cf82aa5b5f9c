"""Solution output (jax_fem/utils.py:13-57): VTK XML unstructured-grid files without meshio.

``save_sol`` keeps the reference's signature and data layout (point data 'sol' as float32,
optional cell / point data as float32); the file is written directly as VTU XML, inline
base64 'binary' (UInt32 length headers) or ASCII.  ``read_vtu`` reads both back.
"""
import base64
import os
import struct
import xml.etree.ElementTree as ET

import numpy as np

# meshio cell type -> (VTK cell type id, nodes per cell); node order of meshio = VTK order
VTK_TYPES = {"hexahedron": (12, 8), "tetra": (10, 4), "tetra10": (24, 10), "quad": (9, 4), "triangle": (5, 3),
             "hexahedron27": (29, 27), "hexahedron20": (25, 20)}
_VTK_BY_ID = {v[0]: (k, v[1]) for k, v in VTK_TYPES.items()}
_VTK_DT = {np.dtype(np.float32): "Float32", np.dtype(np.float64): "Float64", np.dtype(np.int64): "Int64",
           np.dtype(np.int32): "Int32", np.dtype(np.uint8): "UInt8"}
_NP_DT = {v: k for k, v in _VTK_DT.items()}


def _to_numpy(a):
    try:
        import torch
        if torch.is_tensor(a):
            return a.detach().cpu().numpy()
    except ImportError:  # pragma: no cover
        pass
    return np.asarray(a)


def _data_array(parent, name, arr, ncomp, binary):
    arr = np.ascontiguousarray(arr)
    da = ET.SubElement(parent, "DataArray", type=_VTK_DT[arr.dtype], Name=name,
                       format="binary" if binary else "ascii")
    if ncomp > 1:
        da.set("NumberOfComponents", str(ncomp))
    if binary:
        raw = arr.astype(arr.dtype.newbyteorder("<"), copy=False).tobytes()
        da.text = base64.b64encode(struct.pack("<I", len(raw)) + raw).decode("ascii")
    else:
        fmt = "%.9g" if arr.dtype == np.float32 else ("%.17g" if arr.dtype == np.float64 else "%d")
        da.text = " ".join(fmt % v for v in arr.reshape(-1))
    return da


def save_sol(fe, sol, sol_file, cell_infos=None, point_infos=None, binary=True):
    """utils.py:13-57: write the mesh of fe with point data 'sol' (num_total_nodes, vec) and the
    optional [(name, data)] cell data (num_cells,) and point data (num_total_nodes, ...)."""
    from .generate_mesh import get_meshio_cell_type
    cell_type = get_meshio_cell_type(fe.ele_type)
    vtk_id, npc = VTK_TYPES[cell_type]
    sol = _to_numpy(sol)
    points = np.asarray(fe.points, dtype=np.float64)
    cells = np.asarray(fe.cells, dtype=np.int64)
    assert cells.shape[1] == npc
    d = os.path.dirname(sol_file)
    if d:
        os.makedirs(d, exist_ok=True)
    root = ET.Element("VTKFile", type="UnstructuredGrid", version="1.0", byte_order="LittleEndian",
                      header_type="UInt32")
    grid = ET.SubElement(root, "UnstructuredGrid")
    piece = ET.SubElement(grid, "Piece", NumberOfPoints=str(len(points)), NumberOfCells=str(len(cells)))
    pts3 = np.zeros((len(points), 3))
    pts3[:, :points.shape[1]] = points
    _data_array(ET.SubElement(piece, "Points"), "Points", pts3, 3, binary)
    cel = ET.SubElement(piece, "Cells")
    _data_array(cel, "connectivity", cells.reshape(-1), 1, binary)
    _data_array(cel, "offsets", np.arange(1, len(cells) + 1, dtype=np.int64) * npc, 1, binary)
    _data_array(cel, "types", np.full(len(cells), vtk_id, dtype=np.uint8), 1, binary)
    pd = ET.SubElement(piece, "PointData")
    s = np.asarray(sol, dtype=np.float32)
    _data_array(pd, "sol", s, 1 if s.ndim == 1 else s.shape[1], binary)
    for name, data in (point_infos or []):
        data = np.asarray(_to_numpy(data), dtype=np.float32)
        assert len(data) == len(s), "point data wrong shape!"
        _data_array(pd, name, data, 1 if data.ndim == 1 else int(np.prod(data.shape[1:])), binary)
    if cell_infos:
        cd = ET.SubElement(piece, "CellData")
        for name, data in cell_infos:
            data = np.asarray(_to_numpy(data), dtype=np.float32)
            assert data.shape == (len(cells),), \
                f"cell data wrong shape, get {data.shape}, while num_cells = {len(cells)}"
            _data_array(cd, name, data, 1, binary)
    ET.ElementTree(root).write(sol_file, xml_declaration=True, encoding="utf-8")


def _read_array(da):
    dt = _NP_DT[da.get("type")]
    ncomp = int(da.get("NumberOfComponents", "1"))
    if da.get("format", "ascii") == "binary":
        raw = base64.b64decode(da.text.strip())
        n = struct.unpack("<I", raw[:4])[0]
        arr = np.frombuffer(raw[4:4 + n], dtype=dt.newbyteorder("<")).astype(dt)
    else:
        arr = np.array(da.text.split(), dtype=dt)
    return arr.reshape(-1, ncomp) if ncomp > 1 else arr


def read_vtu(path):
    """Read a VTU written by save_sol (binary or ASCII; single piece, one cell type):
    returns (points, {cell_type: cells}, point_data, cell_data)."""
    piece = ET.parse(path).getroot().find("UnstructuredGrid/Piece")
    points = _read_array(piece.find("Points/DataArray"))
    arrs = {da.get("Name"): _read_array(da) for da in piece.find("Cells").findall("DataArray")}
    types = arrs["types"].astype(np.int64)
    name, npc = _VTK_BY_ID[int(types[0])]
    cells = {name: arrs["connectivity"].astype(np.int64).reshape(-1, npc)}
    pdn, cdn = piece.find("PointData"), piece.find("CellData")
    pd = {da.get("Name"): _read_array(da) for da in (pdn.findall("DataArray") if pdn is not None else [])}
    cd = {da.get("Name"): _read_array(da) for da in (cdn.findall("DataArray") if cdn is not None else [])}
    return points, cells, pd, cd
