"""VTK writer (trixi2vtk, write2vtk.jl:113-248, 310-341): the arrays written read back
exactly, the file names follow the reference's system naming, and the ParaView
collection gains one entry per call (CPU only)."""
import types
import xml.etree.ElementTree as ET

import numpy as np


class _NoVisc:
    def viscosity(self):
        from meshfree_gb300._lib import MFTError
        raise MFTError(5, "no viscosity")


def test_trixi2vtk_roundtrip(tmp_path):
    import meshfree_gb300 as M
    from meshfree_gb300 import vtk
    from meshfree_gb300 import workloads as W
    pts, per, h = W.vortex_cloud(8)
    u = W.isentropic_vortex(pts, 0.0)
    eq = M.CompressibleEulerEquations2D(1.4)
    semi = types.SimpleNamespace(equations=eq, domain=types.SimpleNamespace(
        pd=types.SimpleNamespace(points=pts), ctx=_NoVisc()))
    p0 = vtk.trixi2vtk(u, semi, 0.0, iter=0, output_directory=str(tmp_path), prefix="run")
    p1 = vtk.trixi2vtk(u * 1.5, semi, 0.25, iter=1, output_directory=str(tmp_path), prefix="run")
    assert p0.endswith("run_CompressibleEulerEquations2D_1_0.vtu")
    d = vtk.read_vtu_point_data(p1)
    u1 = u * 1.5
    prim = eq.cons2prim(u1)
    assert np.array_equal(d["density"], u1[0])
    assert np.array_equal(d["density_energy"], u1[3])
    assert np.array_equal(d["momentum"], np.stack([u1[1], u1[2]], 1))
    assert np.array_equal(d["pressure"], prim[3])
    assert np.array_equal(d["velocity"], np.stack([prim[1], prim[2]], 1))
    assert np.array_equal(d["index"], np.arange(1, pts.shape[0] + 1))
    assert np.array_equal(d["Points"][:, :2], pts) and not d["Points"][:, 2].any()
    assert np.array_equal(d["types"], np.ones(pts.shape[0], np.uint8))
    assert d["time"][0] == 0.25
    pvd = ET.parse(str(tmp_path / "run_CompressibleEulerEquations2D_1.pvd")).getroot()
    files = [ds.get("file") for ds in pvd.iter("DataSet")]
    assert files == ["run_CompressibleEulerEquations2D_1_0.vtu",
                     "run_CompressibleEulerEquations2D_1_1.vtu"]
