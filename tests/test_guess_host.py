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


def _reference_guess(H, inf, X, x0, y0):
    """__guess_height (scripts/gvom.py:592-714) for one cell, restated in
    Python with its quirks: the loop condition tests x_n_done twice and not
    x_p_done, the x ranges of the two y directions differ from the y ranges
    of the two x directions, and x_nh's test guards y_nh.  0.0 where the
    reference writes nothing."""
    if H[x0][y0] > -1000 or inf[x0][y0] == -1000.0:
        return 0.0
    xpd = xnd = ypd = ynd = False
    xp = xn = x0
    yp = yn = y0
    xph = xnh = yph = ynh = -1000
    i = 0
    while i < 15 and not (xnd and xnd and ypd and ynd):
        xp += 1
        xn -= 1
        yp += 1
        yn -= 1
        i += 1
        if not xpd:
            if xp < X:
                for dy in range(-i, i):
                    if 0 <= y0 + dy < X and H[xp][y0 + dy] > -1000:
                        xph, xpd = H[xp][y0 + dy], True
                        break
            else:
                xpd = True
        if not xnd:
            if xn >= 0:
                for dy in range(-i + 1, i + 1):
                    if 0 <= y0 + dy < X and H[xn][y0 + dy] > -1000:
                        xnh, xnd = H[xn][y0 + dy], True
                        break
            else:
                xnd = True
        if not ypd:
            if yp < X:
                for dx in range(-i + 1, i + 1):
                    if 0 <= x0 + dx < X and H[x0 + dx][yp] > -1000:
                        yph, ypd = H[x0 + dx][yp], True
                        break
            else:
                ypd = True
        if not ynd:
            if yn >= 0:
                for dx in range(-i, i):
                    if 0 <= x0 + dx < X and H[x0 + dx][yn] > -1000:
                        ynh, ynd = H[x0 + dx][yn], True
                        break
            else:
                ynd = True
    mn, mx = 1000.0, inf[x0][y0]
    if xph > -1000:
        mn, mx = min(xph, mn), max(xph, mx)
    if xnh > -1000:
        mn, mx = min(xnh, mn), max(xnh, mx)
    if yph > -1000:
        mn, mx = min(yph, mn), max(yph, mx)
    if xnh > -1000:
        mn, mx = min(ynh, mn), max(ynh, mx)
    dh = mx - mn
    return dh if dh > 0 else 0.0


@pytest.mark.parametrize("density", [0.02, 0.08, 0.3, 0.7])
def test_kernel_guess_search_on_random_maps(guess_lib, density):
    """Random sparse height and inferred-height maps (known cells at several
    densities, so rings reach from one cell to the 15-cell limit and the map
    edges): the kernel's search through its next-known tables against the
    Python restatement, bit for bit on every cell."""
    rng = np.random.default_rng(int(density * 1000))
    X = 48
    for _ in range(3):
        H = np.where(rng.random((X, X)) < density, rng.normal(1.0, 2.0, (X, X)), -1000.0)
        inf = np.where(rng.random((X, X)) < 0.8, rng.normal(0.0, 2.0, (X, X)), -1000.0)
        H = np.ascontiguousarray(H, np.float64)
        inf = np.ascontiguousarray(inf, np.float64)
        got = np.empty((X, X))
        assert guess_lib.guess_all(H.ctypes.data, inf.ctypes.data, X, got.ctypes.data) == 0
        Hl, il = H.tolist(), inf.tolist()
        ref = np.array([[_reference_guess(Hl, il, X, x, y) for y in range(X)] for x in range(X)])
        np.testing.assert_array_equal(got.view(np.uint64), ref.view(np.uint64))
        assert (ref > 0).any()
