"""k_columns' positive-obstacle band density (`band_density` in
gvom_gb300/csrc/k_combine.cu: an integer quotient where it provably equals
the float64 sequence, the float64 sequence itself otherwise), compiled for
the host from the kernel source, against the reference's
int(float(dens) / float(nn) * 100) (scripts/gvom.py:548-555) on random
counts, ratios whose value is an integer, values one unit off an integer,
and counts on both sides of the 2^32 and 2^44 boundaries of the integer
paths: equal everywhere."""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
KERNEL = os.path.join(os.path.dirname(HERE), "gvom_gb300", "csrc", "k_combine.cu")

PRELUDE = r"""
#define __device__
#define __forceinline__ inline
#define __ddiv_rn(a, b) ((double)(a) / (double)(b))
#define __dmul_rn(a, b) ((double)(a) * (double)(b))
"""

DRIVER = r"""
extern "C" void run(const long long *dens, const long long *nn, int n, int *out) {
    for (int i = 0; i < n; i++) out[i] = band_density(dens[i], nn[i]);
}
"""


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    src = open(KERNEL).read()
    a = src.index("__device__ __forceinline__ int band_density(")
    body = src[a:src.index("\n}\n", a) + 3]
    d = tmp_path_factory.mktemp("density")
    cpp = d / "density.cpp"
    cpp.write_text(PRELUDE + body + DRIVER)
    so = d / "libdensity.so"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-o", str(so), str(cpp)],
                   check=True)
    lib = C.CDLL(str(so))
    lib.run.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]
    return lib


def _reference(dens, nn):
    return [int(float(d) / float(m) * 100) for d, m in zip(dens, nn)]


def _cases():
    rng = np.random.default_rng(21)
    dens, nn = [], []
    # random counts of the sizes a band holds (a few voxels of up to thousands of rays)
    m = rng.integers(1, 200_000, 20_000)
    dens += list(rng.integers(0, 200_000, 20_000))
    nn += list(m)
    # ratios whose value 100 dens / nn is an integer, and one unit off either way
    for _ in range(20_000):
        q = int(rng.integers(1, 20_000))
        k = int(rng.integers(0, 150))
        if (k * q) % 100:
            continue
        d = k * q // 100  # 100 d / q = k exactly
        for dd in (d, d + 1, max(d - 1, 0)):
            dens.append(dd)
            nn.append(q)
    # both sides of the 32-bit and 2^44 limits of the integer paths
    for P in (2 ** 32 - 100, 2 ** 32, 2 ** 32 + 100, 2 ** 44 - 100, 2 ** 44, 2 ** 44 + 100):
        for q in (3, 7, 97, 2 ** 31 - 1, 2 ** 32 + 15):
            d = P // 100
            for dd in (d - 1, d, d + 1):
                dens.append(dd)
                nn.append(q)
    # large counts near an integer ratio
    for q in (2 ** 20 + 7, 2 ** 33 + 5, 10 ** 11 + 3):
        for k in (1, 37, 99, 100):
            d = k * q // 100
            for dd in (d - 1, d, d + 1):
                if dd >= 0:
                    dens.append(dd)
                    nn.append(q)
    return np.array(dens, np.int64), np.array(nn, np.int64)


def test_band_density_equals_float64_formula(lib):
    dens, nn = _cases()
    out = np.empty(dens.size, np.int32)
    lib.run(dens.ctypes.data, nn.ctypes.data, dens.size, out.ctypes.data)
    ref = np.array(_reference(dens.tolist(), nn.tolist()), np.int64)
    ok = ref.astype(np.int32).astype(np.int64) == ref  # results that fit the kernel's int
    bad = np.flatnonzero(ok & (out.astype(np.int64) != ref))
    assert bad.size == 0, [(int(dens[i]), int(nn[i]), int(out[i]), int(ref[i])) for i in bad[:5]]
    assert ok.sum() > 20_000
