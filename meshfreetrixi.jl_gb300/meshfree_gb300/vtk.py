"""VTK output of point-cloud solutions: trixi2vtk (src/visualization/write2vtk.jl:113-248).

Writes what the reference's WriteVTK-based writer writes: one unstructured-grid file
(.vtu) per call with every node as a VTK_VERTEX cell, the point data of
write2vtk!(vtk, u, t, ::CompressibleEulerEquations2D) (:310-326: density, density_energy,
momentum, pressure, velocity) or the scalar field of other equations, the viscosity of a
residual/upwind viscosity source when the engine holds one (:328-341, `eps`), the node
`index`, the field data `time`, and a ParaView collection (.pvd) that gains one entry
per call (reset when iter == 0).  File names follow system_names (:38-43):
"[prefix_]<EquationsType>_1[_iter].vtu".  Arrays are stored as raw appended binary
(little endian, UInt64 block headers), which ParaView and VTK read directly.
"""
from __future__ import annotations

import os
import xml.etree.ElementTree as ET

import numpy as np

_VTK_VERTEX = 1


def _system_name(equations) -> str:
    return type(equations).__name__ + "_1"


class _Appended:
    def __init__(self):
        self.blocks = []
        self.offset = 0

    def add(self, arr) -> int:
        raw = np.ascontiguousarray(arr).astype(np.asarray(arr).dtype.newbyteorder("<"),
                                               copy=False).tobytes()
        off = self.offset
        self.blocks.append(np.uint64(len(raw)).tobytes() + raw)
        self.offset += 8 + len(raw)
        return off


_TYPES = {np.dtype(np.float64): "Float64", np.dtype(np.float32): "Float32",
          np.dtype(np.int64): "Int64", np.dtype(np.int32): "Int32", np.dtype(np.uint8): "UInt8"}


def _data_array(parent, app, name, arr, ncomp=1):
    arr = np.asarray(arr)
    el = ET.SubElement(parent, "DataArray", type=_TYPES[arr.dtype], Name=name,
                       NumberOfComponents=str(ncomp), format="appended",
                       offset=str(app.add(arr)))
    return el


def write_vtu(path, points, point_data, field_data=None):
    """points: (n, dim) with dim <= 3; point_data: {name: (n,) or (n, c)} arrays."""
    pts = np.asarray(points, dtype=np.float64)
    n, dim = pts.shape
    p3 = np.zeros((n, 3))
    p3[:, :dim] = pts
    root = ET.Element("VTKFile", type="UnstructuredGrid", version="1.0",
                      byte_order="LittleEndian", header_type="UInt64")
    grid = ET.SubElement(root, "UnstructuredGrid")
    app = _Appended()
    if field_data:
        fd = ET.SubElement(grid, "FieldData")
        for name, val in field_data.items():
            a = np.atleast_1d(np.asarray(val, dtype=np.float64))
            el = _data_array(fd, app, name, a)
            el.set("NumberOfTuples", str(a.size))
    piece = ET.SubElement(grid, "Piece", NumberOfPoints=str(n), NumberOfCells=str(n))
    pd = ET.SubElement(piece, "PointData")
    for name, arr in point_data.items():
        a = np.asarray(arr)
        if a.dtype not in _TYPES:
            a = a.astype(np.float64)
        _data_array(pd, app, name, a, 1 if a.ndim == 1 else a.shape[1])
    pe = ET.SubElement(piece, "Points")
    _data_array(pe, app, "Points", p3, 3)
    cells = ET.SubElement(piece, "Cells")
    _data_array(cells, app, "connectivity", np.arange(n, dtype=np.int64))
    _data_array(cells, app, "offsets", np.arange(1, n + 1, dtype=np.int64))
    _data_array(cells, app, "types", np.full(n, _VTK_VERTEX, dtype=np.uint8))
    ET.SubElement(root, "AppendedData", encoding="raw").text = "_"
    head = ET.tostring(root, encoding="unicode")
    cut = head.rindex("_</AppendedData>")
    with open(path, "wb") as f:
        f.write(b'<?xml version="1.0" encoding="utf-8"?>\n')
        f.write(head[:cut + 1].encode())
        for b in app.blocks:
            f.write(b)
        f.write(head[cut + 1:].encode())
    return path


def _pvd_add(pvd_path, vtu_path, t, reset):
    entries = []
    if not reset and os.path.exists(pvd_path):
        for ds in ET.parse(pvd_path).getroot().iter("DataSet"):
            entries.append((ds.get("timestep"), ds.get("file")))
    entries.append((repr(float(t)), os.path.basename(vtu_path)))
    root = ET.Element("VTKFile", type="Collection", version="1.0", byte_order="LittleEndian")
    col = ET.SubElement(root, "Collection")
    for ts, fn in entries:
        ET.SubElement(col, "DataSet", timestep=ts, part="0", file=fn)
    ET.ElementTree(root).write(pvd_path, encoding="utf-8", xml_declaration=True)


def read_vtu_point_data(path):
    """{name: array} of a file written by write_vtu (used by the tests)."""
    data = open(path, "rb").read()
    start = data.index(b'<AppendedData encoding="raw">_') + len(b'<AppendedData encoding="raw">_')
    root = ET.fromstring(data[:start].decode() + "</AppendedData></VTKFile>")
    inv = {v: k for k, v in _TYPES.items()}
    out = {}
    for el in root.iter("DataArray"):
        off = start + int(el.get("offset"))
        nbytes = int(np.frombuffer(data[off:off + 8], dtype="<u8")[0])
        a = np.frombuffer(data[off + 8:off + 8 + nbytes], dtype=inv[el.get("type")].newbyteorder("<"))
        nc = int(el.get("NumberOfComponents", "1"))
        out[el.get("Name")] = a.reshape(-1, nc) if nc > 1 else a
    return out


def trixi2vtk(u, semi, t, iter=None, output_directory="out", prefix=""):
    """trixi2vtk(u_ode, semi, t; iter, output_directory, prefix) for a solution u of shape
    (nvars, n).  Returns the .vtu path."""
    os.makedirs(output_directory, exist_ok=True)
    eq = semi.equations
    name = _system_name(eq)
    pre = "" if prefix == "" else prefix + "_"
    post = "" if iter is None else "_%d" % iter
    path = os.path.join(output_directory, pre + name + post + ".vtu")
    u = np.asarray(u, dtype=np.float64)
    pdata = {}
    if u.shape[0] == 4 and hasattr(eq, "cons2prim"):
        prim = eq.cons2prim(u)
        pdata["density"] = u[0]
        pdata["density_energy"] = u[3]
        pdata["momentum"] = np.stack([u[1], u[2]], axis=1)
        pdata["pressure"] = prim[3]
        pdata["velocity"] = np.stack([prim[1], prim[2]], axis=1)
    else:
        for v in range(u.shape[0]):
            pdata["scalar" if u.shape[0] == 1 else "u%d" % (v + 1)] = u[v]
    from ._lib import MFTError
    try:
        pdata["eps"] = semi.domain.ctx.viscosity()
    except MFTError:  # no viscosity source evaluated yet: nothing to write
        pass
    pdata["index"] = np.arange(1, u.shape[1] + 1, dtype=np.int64)
    field = {"time": t}
    write_vtu(path, semi.domain.pd.points, pdata, field)
    _pvd_add(os.path.join(output_directory, pre + name + ".pvd"), path, t,
             reset=(iter is None or iter == 0))
    return path
