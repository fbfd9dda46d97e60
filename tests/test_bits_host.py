"""k_maps2d's bit-pattern helpers (gvom_gb300/csrc/k_combine.cu: same_double,
double_order, widen), compiled for the host from the kernel source, against
the float64 compare and the float -> double conversion they replace, on
random bit patterns and the special values (zeros, subnormals, infinities,
NaN where the helper accepts it)."""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
KERNEL = os.path.join(os.path.dirname(HERE), "gvom_gb300", "csrc", "k_combine.cu")

PRELUDE = r"""
#include <cstring>
#define __device__
#define __forceinline__ inline
static inline long long __double_as_longlong(double d) { long long b; std::memcpy(&b, &d, 8); return b; }
static inline double __longlong_as_double(long long b) { double d; std::memcpy(&d, &b, 8); return d; }
static inline unsigned __float_as_uint(float f) { unsigned u; std::memcpy(&u, &f, 4); return u; }
"""

POSTLUDE = r"""
extern "C" void run(const double *a, const double *b, int n, int *eq, int *lt) {
    for (int i = 0; i < n; i++) {
        eq[i] = same_double(a[i], b[i]);
        lt[i] = double_order(a[i]) < double_order(b[i]);
    }
}
extern "C" void run_widen(const float *f, int n, double *out) {
    for (int i = 0; i < n; i++) out[i] = widen(f[i]);
}
"""


def _fn(src, head):
    a = src.index(head)
    return src[a:src.index("\n}\n", a) + 3]


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    src = open(KERNEL).read()
    body = "".join(_fn(src, h) for h in ("__device__ __forceinline__ bool same_double(",
                                         "__device__ __forceinline__ long long double_order(",
                                         "__device__ __forceinline__ double widen("))
    d = tmp_path_factory.mktemp("bits")
    cpp = d / "bits.cpp"
    cpp.write_text(PRELUDE + body + POSTLUDE)
    so = d / "libbits.so"
    subprocess.run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-o", str(so), str(cpp)], check=True)
    lib = C.CDLL(str(so))
    lib.run.argtypes = [C.c_void_p] * 2 + [C.c_int] + [C.c_void_p] * 2
    lib.run_widen.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
    return lib


def _doubles(rng, n):
    bits = rng.integers(0, 2**64, n, dtype=np.uint64)
    v = bits.view(np.float64)
    special = np.array([0.0, -0.0, 1.0, -1.0, -1000.0, 1000.0, 5e-324, -5e-324, np.inf, -np.inf,
                        2.2250738585072014e-308, 0.15, -0.15, 1e300, -1e300])
    v = np.concatenate([v, special, rng.choice(special, n), np.round(rng.normal(0, 3, n), 2)])
    return v[~np.isnan(v)]


def test_same_double_and_order_match_float64_compare(lib):
    rng = np.random.default_rng(11)
    a = _doubles(rng, 200_000)
    b = np.concatenate([rng.permutation(a[: a.size // 2]), a[a.size // 2:]])  # half of the pairs equal
    a = np.ascontiguousarray(a)
    b = np.ascontiguousarray(b)
    eq = np.empty(a.size, np.int32)
    lt = np.empty(a.size, np.int32)
    lib.run(a.ctypes.data, b.ctypes.data, a.size, eq.ctypes.data, lt.ctypes.data)
    np.testing.assert_array_equal(eq.astype(bool), a == b)
    # < on keys equals < on values except that -0 sorts below +0
    neg0 = np.signbit(a) & (a == 0) & ~np.signbit(b) & (b == 0)
    np.testing.assert_array_equal(lt.astype(bool), (a < b) | neg0)


def test_widen_equals_conversion(lib):
    rng = np.random.default_rng(12)
    f = rng.integers(0, 2**32, 1_000_000, dtype=np.uint64).astype(np.uint32).view(np.float32)
    f = np.ascontiguousarray(np.concatenate([f, np.array([0.0, -0.0, 1e-45, -1e-45, 1.1754944e-38, np.inf, -np.inf,
                                                          np.nan, 3.4028235e38], np.float32)]))
    out = np.empty(f.size, np.float64)
    lib.run_widen(f.ctypes.data, f.size, out.ctypes.data)
    with np.errstate(invalid="ignore"):
        ref = f.astype(np.float64)
    nan = np.isnan(ref)
    np.testing.assert_array_equal(np.isnan(out), nan)
    np.testing.assert_array_equal(out[~nan].view(np.uint64), ref[~nan].view(np.uint64))
