"""TEST INFRASTRUCTURE - canonical forms of mapper state for parity checks.

The reference numbers occupied voxels with an atomic counter
(gvom.py:1238, 1031, 1059), so compact indices differ run to run and are not
observable.  These helpers re-key every per-voxel quantity by the voxel's
linear index (x + y*X + z*X*X, gvom.py:1167) so two implementations can be
compared exactly.
"""
from __future__ import annotations

import numpy as np


def canonical_map(index, **per_voxel):
    """Return {'occ': occupied voxel ids (ascending), 'free': dense int32 map with
    occupied voxels set to 0 (free/unknown values are <= -1), and each keyword
    array re-ordered to canonical occupied order}."""
    index = np.asarray(index).reshape(-1)
    occ = np.flatnonzero(index >= 0)
    c = index[occ].astype(np.int64)
    out = {"occ": occ.astype(np.int64), "free": np.where(index >= 0, 0, index).astype(np.int32)}
    for k, v in per_voxel.items():
        if v is None:
            continue
        v = np.asarray(v)
        out[k] = v[c] if len(c) else v[:0]
    return out


def canonical_state(st: dict) -> dict:
    """Canonical form of a state dict with keys index, hit, total, min_h[, metrics, eigen]."""
    return canonical_map(st["index"], hit=st.get("hit"), total=st.get("total"),
                         min_h=st.get("min_h"), metrics=st.get("metrics"), eigen=st.get("eigen"))


def sort_debug_voxels(rows):
    """Rows of make_debug_voxel_map sorted by (z, y, x) world position."""
    rows = np.asarray(rows)
    if rows.shape[0] == 0:
        return rows
    o = np.lexsort((rows[:, 0], rows[:, 1], rows[:, 2]))
    return rows[o]
