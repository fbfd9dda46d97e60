"""TEST INFRASTRUCTURE - CPU restatement of the reference ROS node's
OccupancyGrid payloads (scripts/gvom_ros.py:141-164), the checker for
gvom_ros_grids / Gvom.ros_grids.  Inputs are combine_maps' outputs
(pos, neg, roughness, visibility as [x, y] arrays); each payload is flattened
column-major (x fastest) as the node's np.reshape(..., -1, order='F') does and
cast to int8 the way numpy does on the node's x86 host: truncation toward
zero through a 32-bit integer (0 outside its range, and for NaN), then the
low 8 bits (the roughness payload of the node's defaults lies in
[-200, -100], outside int8, so the cast rule is part of the result)."""
from __future__ import annotations

import numpy as np


def int8_wrap(v: np.ndarray) -> np.ndarray:
    v = np.asarray(v, np.float64)
    out = np.zeros(v.shape, np.int64)
    # x86 truncates through a 32-bit integer: outside int32, or NaN, gives the
    # integer indefinite 0x80000000, low byte 0
    ok = (v > -2147483649.0) & (v < 2147483648.0)
    out[ok] = np.trunc(v[ok]).astype(np.int64)
    b = out & 0xFF
    return np.where(b >= 128, b - 256, b).astype(np.int8)


def ros_grids(pos, neg, rough, vis, density_threshold=50, min_roughness=-10, max_roughness=0) -> dict:
    """The five payloads, each int8[X * X] (x fastest)."""
    obs = np.asarray(pos, np.float64)
    negf = np.asarray(neg, np.int64)
    flat = lambda a: np.reshape(a, -1, order="F")  # noqa: E731  [x, y] -> x fastest
    hard = np.maximum(np.where(obs > density_threshold, 100, 0), negf)                    # :142
    soft = np.where((obs <= density_threshold) & (obs > 0), 100, 0)                       # :147
    cert = np.asarray(vis, np.int64) * 100                                                # :152
    r = np.asarray(rough, np.float64)
    r = np.maximum(np.minimum(r, max_roughness), min_roughness)                           # :162
    r = ((r + min_roughness) / (max_roughness - min_roughness)) * 100.0
    return {"hard": int8_wrap(flat(hard)), "soft": int8_wrap(flat(soft)), "certainty": int8_wrap(flat(cert)),
            "negative": int8_wrap(flat(negf)), "roughness": int8_wrap(flat(r))}
