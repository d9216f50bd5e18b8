"""Medusa point-cloud reader (read_medusa_file, src/auxiliary/medusa/read_medusa_file.jl:2-64).

* The reference's own fixture files test/data/cyl_0_05_* read through
  meshfree_gb300.medusa.read_medusa_file give the committed fixture tests/golden/cyl_0_05.npz
  (positions, types, interior list, boundary groups and their normals).  The reference
  checkout is located by the environment variable MFT_REFERENCE_ROOT; the test is skipped
  where it is not set.
* Everywhere: the fixture written out in the Medusa text layout (comma-separated rows,
  whitespace-separated integer lists) and read back gives the same arrays, which exercises
  the group splitting by the negative type codes.
"""
import os
from pathlib import Path

import numpy as np
import pytest

from meshfree_gb300.medusa import read_medusa_file


def _compare(cyl, got):
    pos, interior, b_idx, b_nrm, normals, types = got
    assert np.array_equal(pos, cyl["positions"])
    assert np.array_equal(types, cyl["types"])
    assert np.array_equal(interior, cyl["interior"])
    assert np.array_equal(normals, cyl["normals"])
    groups = sorted(k for k in cyl if k.startswith("bidx_"))
    assert len(b_idx) == len(groups)
    for g, key in enumerate(groups):
        assert np.array_equal(b_idx[g], cyl[key])
        assert np.array_equal(b_nrm[g], cyl["bnrm_%d" % (g + 1)])


def _write_medusa(prefix, cyl):
    """The fixture in the Medusa layout: the boundary list in type order (groups -1, -2,
    ...), one normal per boundary-list entry."""
    bidx = np.concatenate([cyl["bidx_%d" % g] for g in range(1, 6)])
    bnrm = np.concatenate([cyl["bnrm_%d" % g] for g in range(1, 6)])
    rows = lambda a: "\n".join("%r , %r" % (float(x), float(y)) for x, y in a) + "\n"
    ints = lambda a: "\n".join(str(int(v)) for v in a) + "\n"
    Path(str(prefix) + "_positions.txt").write_text(rows(cyl["positions"]))
    Path(str(prefix) + "_types.txt").write_text(ints(cyl["types"]))
    Path(str(prefix) + "_boundary.txt").write_text(ints(bidx))
    Path(str(prefix) + "_interior.txt").write_text(ints(cyl["interior"]))
    Path(str(prefix) + "_normals.txt").write_text(rows(bnrm))
    return bidx, bnrm


def test_reader_round_trip_of_the_fixture(cyl, tmp_path):
    bidx, bnrm = _write_medusa(tmp_path / "cyl", cyl)
    pos, interior, b_idx, b_nrm, normals, types = read_medusa_file(tmp_path / "cyl")
    assert np.array_equal(pos, cyl["positions"])
    assert np.array_equal(types, cyl["types"])
    assert np.array_equal(interior, cyl["interior"])
    assert np.array_equal(normals, bnrm)
    for g in range(5):
        assert np.array_equal(b_idx[g], cyl["bidx_%d" % (g + 1)])
        assert np.array_equal(b_nrm[g], cyl["bnrm_%d" % (g + 1)])


def test_reader_on_the_reference_fixture_files(cyl):
    root = os.environ.get("MFT_REFERENCE_ROOT")
    if not root:
        pytest.skip("MFT_REFERENCE_ROOT (a MeshfreeTrixi.jl checkout) is not set")
    prefix = Path(root) / "test" / "data" / "cyl_0_05"
    if not Path(str(prefix) + "_positions.txt").exists():
        pytest.skip("no test/data/cyl_0_05_* under MFT_REFERENCE_ROOT")
    _compare(cyl, read_medusa_file(prefix))
