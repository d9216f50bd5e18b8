"""Generates tests/golden/cyl_0_05.npz from the reference's own fixture.

Reads the Medusa point cloud test/data/cyl_0_05_* of MeshfreeTrixi.jl (2154 nodes,
boundary groups inlet/outlet/bottom/top/cyl = types -1..-5) and stores it together
with outputs of the CPU oracle on it, so that tests on machines without the
reference checkout can use the same inputs:

  positions, boundary groups and normals (the fixture itself)
  knn (nv = 20, the reference default for 2D degree 3) and dx_min / dx_avg
  weights Dx, Dy for PHS r^3 with degree-3 polynomials

Usage: python tests/golden/make_golden.py <reference checkout>/test/data/cyl_0_05
(the case prefix of the Medusa files; required).
"""
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "meshfreetrixi.jl_gb300"))

from meshfree_gb300.medusa import read_medusa_file  # noqa: E402
from oracle import oracle as o  # noqa: E402


def main(casename):
    pos, interior, b_idx, b_nrm, normals, types = read_medusa_file(casename)
    n = pos.shape[0]
    k = 20
    idx, dists, dx_min, dx_avg = o.knn(pos, k)
    rowptr = np.arange(n + 1, dtype=np.int64) * k
    st = idx.ravel()
    w3 = o.weights(pos, rowptr, st, rbf_pow=3, polydeg=3, deriv_order=1)
    out = dict(positions=pos, interior=interior, types=types, normals=normals,
               knn=idx, dx=np.array([dx_min, dx_avg]), w_r3=w3)
    for g, (ii, nn) in enumerate(zip(b_idx, b_nrm)):
        out["bidx_%d" % (g + 1)] = ii
        out["bnrm_%d" % (g + 1)] = nn
    dst = Path(__file__).resolve().parent / "cyl_0_05.npz"
    np.savez_compressed(dst, **out)
    print("wrote", dst, "nodes", n)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden.py <reference checkout>/test/data/cyl_0_05")
    main(sys.argv[1])
