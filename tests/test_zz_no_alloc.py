"""The allocation-free debug voxel export (gvom_debug_voxel_map_noalloc)
against the regular export (gvom_debug_voxel_map), through the C ABI.

Both run the same row kernel, so the rows must be equal bit for bit; the
allocation-free form is called twice in a row on each map state (its scratch
array is reused, never cleared) and on two map states with different voxel
counts.  A grid above the scratch's limit is refused with GVOM_ERR_ARG.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc_rows(lib, g, torch):
    rows = C.c_int64()
    assert lib.gvom_debug_voxel_map_noalloc(g._h, None, 0, C.byref(rows)) == 0, lib.gvom_last_error()
    n = rows.value
    out = torch.full((max(n, 1), 8), float("nan"), dtype=torch.float32, device="cuda")
    rows2 = C.c_int64()
    rc = lib.gvom_debug_voxel_map_noalloc(g._h, C.c_void_p(out.data_ptr()), n, C.byref(rows2))
    assert rc == 0, lib.gvom_last_error()
    assert rows2.value == n
    return out[:n].cpu().numpy()


def test_noalloc_debug_export_matches_regular(gpu_lib):
    import torch
    from gvom_gb300 import Gvom
    from gvom_gb300.synthetic import WORKLOADS, make_workload_scans
    lib = gpu_lib
    w = WORKLOADS["small_32x512"]
    scans = make_workload_scans(w, 3)
    g = Gvom(*w.gvom_args())
    rows = C.c_int64()
    assert lib.gvom_debug_voxel_map_noalloc(g._h, None, 0, C.byref(rows)) == 1  # GVOM_NO_DATA before a combine
    counts = []
    for batch in (scans[:1], scans[1:]):
        for s in batch:
            g.Process_pointcloud(s.points, s.ego, s.transform)
        g.combine_maps()
        ref = g.make_debug_voxel_map()
        assert ref.shape[0] > 0
        for _ in range(2):  # two calls in a row on the same state
            got = _noalloc_rows(lib, g, torch)
            np.testing.assert_array_equal(got, ref)
        counts.append(ref.shape[0])
    assert counts[0] != counts[1]


def test_noalloc_debug_export_capacity_and_limit(gpu_lib):
    import torch
    from gvom_gb300 import Gvom
    from gvom_gb300.synthetic import WORKLOADS, make_workload_scans
    lib = gpu_lib
    w = WORKLOADS["small_32x512"]
    s = make_workload_scans(w, 1)[0]
    g = Gvom(*w.gvom_args())
    g.Process_pointcloud(s.points, s.ego, s.transform)
    g.combine_maps()
    ref = g.make_debug_voxel_map()
    # a short buffer receives the first rows and nothing beyond them
    cap = ref.shape[0] // 2
    out = torch.full((cap + 4, 8), -7.0, dtype=torch.float32, device="cuda")
    rows = C.c_int64()
    assert lib.gvom_debug_voxel_map_noalloc(g._h, C.c_void_p(out.data_ptr()), cap, C.byref(rows)) == 0
    assert rows.value == ref.shape[0]
    got = out.cpu().numpy()
    np.testing.assert_array_equal(got[:cap], ref[:cap])
    assert np.all(got[cap:] == -7.0)
    # 33,554,432 voxels is the limit: a larger grid is refused before any device work
    big = Gvom(0.2, 0.2, 1449, 16, 1, 1.0, 0.5, 0.5, 0.3, 2.0, 4.0, 1.0, 0, 0)
    rc = lib.gvom_debug_voxel_map_noalloc(big._h, None, 0, C.byref(rows))
    assert rc == 2, rc  # GVOM_ERR_ARG
    assert b"allocation-free" in lib.gvom_last_error()
