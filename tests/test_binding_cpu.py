"""The Python binding's argument marshalling, on CPU: gvom_gb300.Gvom driven
against a recording stand-in of the C ABI (tests/cpp/recording_stub.c,
compiled from include/gvom_gb300.h), which stores what each call received.
Pointers, dtype codes, counts, row strides, ego positions, transforms and
output buffers must reach the library as the header specifies."""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)


@pytest.fixture(scope="module")
def stub(tmp_path_factory):
    if shutil.which("gcc") is None:
        pytest.skip("gcc not available")
    out = str(tmp_path_factory.mktemp("stub") / "librecording_stub.so")
    subprocess.run(["gcc", "-O1", "-Wall", "-Werror", "-shared", "-fPIC", "-I", os.path.join(REPO, "include"),
                    "-o", out, os.path.join(HERE, "cpp", "recording_stub.c")], check=True)
    from gvom_gb300 import _lib
    saved = _lib._lib
    lib = _lib.load(out)
    _lib._lib = lib
    try:
        yield lib
    finally:
        _lib._lib = saved


def _g(stub):
    from gvom_gb300 import Gvom
    return Gvom(0.2, 0.25, 16, 8, 2, 1.0, 0.5, 0.5, 0.3, 2.0, 4.0, 1.0, 1, 1)


def _rec(lib, ctype, name):
    return ctype.in_dll(lib, name)


def _process_args(lib):
    return dict(points=_rec(lib, C.c_void_p, "rec_points").value, dtype=_rec(lib, C.c_int32, "rec_dtype").value,
                n=_rec(lib, C.c_int64, "rec_n").value, stride=_rec(lib, C.c_int64, "rec_stride").value,
                ego=list(_rec(lib, C.c_double * 3, "rec_ego")),
                transform=_rec(lib, C.c_void_p, "rec_transform").value,
                tdtype=_rec(lib, C.c_int32, "rec_tdtype").value, device=_rec(lib, C.c_int32, "rec_device").value)


def test_process_pointcloud_arguments(stub):
    from gvom_gb300._lib import GVOM_F32, GVOM_F64, GVOM_NONE
    g = _g(stub)
    pts = np.arange(30, dtype=np.float32).reshape(10, 3)
    T = np.eye(4, dtype=np.float32)
    g.Process_pointcloud(pts, (1.0, -2.0, 0.5), T)
    a = _process_args(stub)
    assert a == dict(points=pts.ctypes.data, dtype=GVOM_F32, n=10, stride=3, ego=[1.0, -2.0, 0.5],
                     transform=T.ctypes.data, tdtype=GVOM_F32, device=0)
    # float64 rows of 4 (x, y, z, intensity), float64 transform, ego as a numpy array
    xyzi = np.ones((7, 4), np.float64)
    T64 = np.eye(4)
    g.process_pointcloud(xyzi, np.array([0.5, 0.25, 2.0]), T64)
    a = _process_args(stub)
    assert (a["points"], a["dtype"], a["n"], a["stride"]) == (xyzi.ctypes.data, GVOM_F64, 7, 4)
    assert (a["transform"], a["tdtype"], a["ego"]) == (T64.ctypes.data, GVOM_F64, [0.5, 0.25, 2.0])
    # no transform
    g.Process_pointcloud(pts, [0, 0, 0])
    a = _process_args(stub)
    assert a["transform"] is None and a["tdtype"] == GVOM_NONE
    # an ego position of shape (1, 3), float32 or integer, becomes three float64
    for ego in (np.array([[3.0, 4.0, 5.0]]), np.float32([3.0, 4.0, 5.0]), (3, 4, 5)):
        g.Process_pointcloud(pts, ego)
        assert _process_args(stub)["ego"] == [3.0, 4.0, 5.0]
    with pytest.raises(ValueError):
        g.Process_pointcloud(pts, (1.0, 2.0))
    # a strided view and integer points are copied to contiguous float rows
    g.Process_pointcloud(pts[::2], (0, 0, 0), T)
    a = _process_args(stub)
    assert (a["dtype"], a["n"], a["stride"]) == (GVOM_F32, 5, 3) and a["points"] != pts.ctypes.data
    g.Process_pointcloud(np.ones((4, 3), np.int32), (0, 0, 0), None)
    a = _process_args(stub)
    assert (a["dtype"], a["n"], a["stride"]) == (GVOM_F64, 4, 3)
    # an empty scan
    g.Process_pointcloud(np.zeros((0, 3), np.float32), (0, 0, 0), None)
    assert _process_args(stub)["n"] == 0
    with pytest.raises(ValueError):
        g.Process_pointcloud(np.zeros((5, 2), np.float32), (0, 0, 0))


def test_process_pointcloud_torch_cpu_tensor(stub):
    torch = pytest.importorskip("torch")
    from gvom_gb300._lib import GVOM_F32
    g = _g(stub)
    t = torch.arange(12, dtype=torch.float32).reshape(4, 3)
    g.Process_pointcloud(t, (0, 0, 0), torch.eye(4))
    a = _process_args(stub)
    assert (a["points"], a["dtype"], a["n"], a["stride"], a["device"]) == (t.data_ptr(), GVOM_F32, 4, 3, 0)


def test_combine_maps_outputs(stub):
    g = _g(stub)
    origin, pos, neg, rough, vis = g.combine_maps()
    assert origin.tolist() == [1.5, -2.5, 0.25]  # written by the stand-in
    out = list(_rec(stub, C.c_void_p * 5, "rec_out"))
    assert out == [origin.ctypes.data, pos.ctypes.data, neg.ctypes.data, rough.ctypes.data, vis.ctypes.data]
    for a, dt in ((pos, np.int32), (neg, np.int32), (rough, np.float64), (vis, np.int32)):
        assert a.shape == (16, 16) and a.dtype == dt and a.flags.c_contiguous and a.flags.writeable
    # one host block in the library's device order, so the four maps come down in one copy
    X2 = 16 * 16
    r = rough.ctypes.data
    assert [pos.ctypes.data, neg.ctypes.data, vis.ctypes.data] == [r + 8 * X2, r + 12 * X2, r + 16 * X2]


def _scans(lib):
    from gvom_gb300._lib import GvomScan
    n = _rec(lib, C.c_int32, "rec_nscans").value
    arr = (GvomScan * 16).in_dll(lib, "rec_scans")
    return [dict(points=arr[i].points, dtype=arr[i].dtype, tdtype=arr[i].transform_dtype, n=arr[i].n,
                 stride=arr[i].row_stride, ego=list(arr[i].ego), transform=arr[i].transform) for i in range(n)]


def test_process_batch_and_step_scan_tables(stub):
    from gvom_gb300._lib import GVOM_F32, GVOM_F64, GVOM_NONE
    g = _g(stub)
    a = np.zeros((5, 3), np.float32)
    b = np.zeros((3, 4), np.float64)
    Ta = np.eye(4, dtype=np.float32)
    g.process_batch([(a, (1, 2, 3), Ta), (b, (4, 5, 6), None)])
    s = _scans(stub)
    assert s == [dict(points=a.ctypes.data, dtype=GVOM_F32, tdtype=GVOM_F32, n=5, stride=3, ego=[1.0, 2.0, 3.0],
                      transform=Ta.ctypes.data),
                 dict(points=b.ctypes.data, dtype=GVOM_F64, tdtype=GVOM_NONE, n=3, stride=4, ego=[4.0, 5.0, 6.0],
                      transform=None)]
    assert _rec(stub, C.c_int32, "rec_points_on_device").value == 0
    origin, pos, neg, rough, vis = g.step([(b, (7, 8, 9), np.eye(4))])
    s = _scans(stub)
    assert len(s) == 1 and (s[0]["points"], s[0]["dtype"], s[0]["tdtype"], s[0]["ego"]) == \
        (b.ctypes.data, GVOM_F64, GVOM_F64, [7.0, 8.0, 9.0])
    out = list(_rec(stub, C.c_void_p * 5, "rec_out"))
    assert out == [origin.ctypes.data, pos.ctypes.data, neg.ctypes.data, rough.ctypes.data, vis.ctypes.data]
    assert _rec(stub, C.c_int32, "rec_outputs_on_device").value == 0
    assert origin.tolist() == [1.5, -2.5, 0.25]
