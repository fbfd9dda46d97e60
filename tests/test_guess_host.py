"""k_maps2d's guess-height search (gvom_gb300/csrc/k_combine.cu, the block
after "__guess_height"), compiled for the host from the kernel source with
next-known tables built the way the kernel defines them, against the
oracle's __guess_height (scripts/gvom.py:592-714, its loop-condition and
y_nh quirks included) on every golden fixture: bit for bit."""
import ctypes as C
import os
import re
import shutil
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, golden_files
from oracle.oracle import OracleGvom
from replay import load, ops_of, params_of

HERE = os.path.dirname(os.path.abspath(__file__))
KERNEL = os.path.join(os.path.dirname(HERE), "gvom_gb300", "csrc", "k_combine.cu")

PRELUDE = r"""
#include <algorithm>
#include <cstring>
using std::max; using std::min;
#define __dsub_rn(a, b) ((double)(a) - (double)(b))
#define __device__
#define __forceinline__ inline
static inline long long __double_as_longlong(double d) { long long b; std::memcpy(&b, &d, 8); return b; }
%(helpers)s
constexpr int kHalo = %(halo)d;
constexpr int kS = 250;  // one tile over the whole map: X + 2 kHalo <= kS (next-known indices are bytes)
static double sh[kS][kS];
static unsigned char kn[kS][kS];
static unsigned char nky[kS][kS + 2], nkx[kS][kS + 2];
struct { const double *inferred; } mp;
extern "C" int guess_all(const double *H, const double *inferred, int X, double *out) {
    if (X + 2 * kHalo > kS) return 1;
    const int len = X + 2 * kHalo;
    for (int i = 0; i < kS; i++)
        for (int j = 0; j < kS; j++) { sh[i][j] = -1000.0; kn[i][j] = 0; }
    for (int x = 0; x < X; x++)
        for (int y = 0; y < X; y++) {
            sh[x + kHalo][y + kHalo] = H[x * X + y];
            kn[x + kHalo][y + kHalo] = H[x * X + y] > -1000.0;
        }
    // nky[sx][sy]: the first known sy' >= sy in row sx, len if none; nkx[sy][sx] likewise along x
    for (int a = 0; a < len; a++) {
        int ny = len, nx = len;
        for (int b = len - 1; b >= 0; b--) {
            if (kn[a][b]) ny = b;
            nky[a][b] = (unsigned char)ny;
            if (kn[b][a]) nx = b;
            nkx[a][b] = (unsigned char)nx;
        }
    }
    mp.inferred = inferred;
    const int x0t = 0, y0t = 0;
    for (int x0 = 0; x0 < X; x0++)
        for (int y0 = 0; y0 < X; y0++) {
            const bool valid = true;
            const bool known = kn[x0 + kHalo][y0 + kHalo];
            const int cell = x0 * X + y0;
"""

POSTLUDE = r"""
            out[cell] = guess;
        }
    return 0;
}
"""


def _kernel_helpers():
    """The kernel's own -1000.0 constant and ordered-key helper."""
    src = open(KERNEL).read()
    const = re.search(r"^constexpr long long kMinus1000Bits = .*$", src, re.M).group(0)
    a = src.index("__device__ __forceinline__ long long double_order(double a) {")
    b = src.index("\n}\n", a) + 3
    return const + "\n" + src[a:b]


def _kernel_guess_block():
    src = open(KERNEL).read()
    a = src.index("    // __guess_height (scripts/gvom.py:592-714)")
    b = src.index("    // cell warps that finish their search", a)
    return src[a:b]


@pytest.fixture(scope="module")
def guess_lib(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    halo = int(re.search(r"constexpr int kHalo = (\d+);", open(KERNEL).read()).group(1))
    d = tmp_path_factory.mktemp("guess")
    cpp = d / "guess_host.cpp"
    cpp.write_text(PRELUDE % {"halo": halo, "helpers": _kernel_helpers()} + _kernel_guess_block() + POSTLUDE)
    so = d / "libguess.so"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-o", str(so), str(cpp)],
                   check=True)
    lib = C.CDLL(str(so))
    lib.guess_all.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]
    return lib


@pytest.mark.parametrize("name", golden_files())
def test_kernel_guess_search_equals_oracle(guess_lib, name):
    fx = load(os.path.join(GOLDEN, name))
    p = params_of(fx)
    X = p[2]
    o = OracleGvom(*p)
    for op in ops_of(fx):
        if op[0] == "P":
            o.Process_pointcloud(*op[2:])
            continue
        o.combine_maps()
        m = o.maps_state()
        H = np.ascontiguousarray(m["height"], np.float64)
        inf = np.ascontiguousarray(m["inferred"], np.float64)
        got = np.empty((X, X))
        assert guess_lib.guess_all(H.ctypes.data, inf.ctypes.data, X, got.ctypes.data) == 0
        np.testing.assert_array_equal(got, m["guess"], f"{name}")
