"""k_debug_maps (gvom_gb300/csrc/k_combine.cu: the height and inferred-height
debug clouds, scripts/gvom.py:412-479), compiled for the host from the
kernel source and run cell by cell on the oracle's maps, against the
reference's own debug clouds stored in every golden fixture: bit for bit."""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, golden_files
from oracle.oracle import OracleGvom
from replay import load, ops_of, params_of

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "gvom_gb300", "csrc")


class _Params(C.Structure):
    _fields_ = [("X", C.c_int), ("co", C.c_double * 3), ("xy_res", C.c_double), ("z_res", C.c_double),
                ("height", C.c_void_p), ("rough", C.c_void_p), ("slope_x", C.c_void_p), ("slope_y", C.c_void_p),
                ("guess", C.c_void_p), ("out_h", C.c_void_p), ("out_i", C.c_void_p)]


@pytest.fixture(scope="module")
def dbg_lib(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    src = open(os.path.join(CSRC, "k_combine.cu")).read()
    k = src.index("__global__ void k_debug_maps(DebugMapParams p) {")
    b = src.index("\n}\n", k) + 3
    d = tmp_path_factory.mktemp("dbg")
    cpp = d / "dbg_host.cpp"
    cpp.write_text('#include <cmath>\nusing std::sqrt;\n#include "gvom_internal.cuh"\nnamespace gvom {\n' + src[k:b] +
                   "}\nusing namespace gvom;\n"
                   'extern "C" void maps(const DebugMapParams *p) {\n'
                   "    for (long long c = 0; c < (long long)p->X * p->X; c++) "
                   "{ blockIdx.x = (unsigned)c; threadIdx.x = 0; blockDim.x = 1; k_debug_maps(*p); }\n}\n")
    so = d / "libdbg.so"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-I",
                    os.path.join(HERE, "cpp", "host_cuda"), "-I", CSRC, "-o", str(so), str(cpp)], check=True)
    lib = C.CDLL(str(so))
    lib.maps.argtypes = [C.POINTER(_Params)]
    return lib


@pytest.mark.parametrize("name", golden_files())
def test_kernel_debug_clouds_equal_reference(dbg_lib, name):
    fx = load(os.path.join(GOLDEN, name))
    p = params_of(fx)
    xy, zr, X = p[0], p[1], p[2]
    o = OracleGvom(*p)
    ci = 0
    for op in ops_of(fx):
        if op[0] == "P":
            o.Process_pointcloud(*op[2:])
            continue
        out = o.combine_maps()
        m = o.maps_state()
        arrs = [np.ascontiguousarray(a, np.float64) for a in (m["height"], out[3], m["slope_x"], m["slope_y"],
                                                               m["guess"])]
        oh = np.zeros((X * X, 7), np.float32)
        oi = np.zeros((X * X, 3), np.float32)
        co = (C.c_double * 3)(*np.round(np.asarray(out[0]) / np.array([xy, xy, zr])).tolist())
        prm = _Params(X, co, xy, zr, *[a.ctypes.data for a in arrs], oh.ctypes.data, oi.ctypes.data)
        dbg_lib.maps(C.byref(prm))
        np.testing.assert_array_equal(oh, fx[f"c{ci}_debug_height"], f"{name} combine {ci} height cloud")
        np.testing.assert_array_equal(oi, fx[f"c{ci}_debug_inferred"], f"{name} combine {ci} inferred cloud")
        ci += 1
