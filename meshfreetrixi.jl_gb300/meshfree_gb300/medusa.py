"""Medusa point-cloud files, the only on-disk domain format of the reference.

Restates read_medusa_file (src/auxiliary/medusa/read_medusa_file.jl:2-64):
<case>_positions.txt (x , y rows), <case>_types.txt (0 interior, -i boundary
group i), <case>_boundary.txt / _interior.txt (0-based node lists) and
<case>_normals.txt (one outward normal per boundary-list entry).  Indices stay
0-based here.
"""
from __future__ import annotations

from pathlib import Path

import numpy as np


def _read_rows(path, sep=","):
    rows = []
    for line in Path(path).read_text().splitlines():
        line = line.strip()
        if not line:
            continue
        rows.append([float(v) for v in line.split(sep)])
    return np.asarray(rows, dtype=np.float64)


def _read_ints(path):
    return np.asarray([int(v) for v in Path(path).read_text().split()], dtype=np.int64)


def read_medusa_file(casename):
    """Returns positions (n,2), interior_idx, boundary_idxs (list per group),
    boundary_normals (list per group, (m,2)), normals (nb,2), types (n,)."""
    positions = _read_rows(str(casename) + "_positions.txt")
    types = _read_ints(str(casename) + "_types.txt")
    boundary_idx = _read_ints(str(casename) + "_boundary.txt")
    interior_idx = _read_ints(str(casename) + "_interior.txt")
    normals = _read_rows(str(casename) + "_normals.txt")
    num_bound = -int(types.min()) if types.size else 0
    b_idx = [[] for _ in range(num_bound)]
    b_nrm = [[] for _ in range(num_bound)]
    for j, b in enumerate(boundary_idx):
        for i in range(1, num_bound + 1):
            if types[b] == -i:
                b_idx[i - 1].append(int(b))
                b_nrm[i - 1].append(normals[j])
    # groups without nodes are dropped from the index lists (as the reference does)
    boundary_idxs = [np.asarray(g, dtype=np.int64) for g in b_idx if len(g)]
    boundary_normals = [np.asarray(g, dtype=np.float64).reshape(-1, 2) for g in b_nrm]
    return positions, interior_idx, boundary_idxs, boundary_normals, normals, types
