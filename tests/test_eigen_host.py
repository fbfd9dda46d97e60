"""The eigen-solve of the statistics merge (`jacobi_rot` / `eigen3` in
gvom_gb300/csrc/k_combine.cu: float32 cyclic Jacobi, float64 determinant
for a near-degenerate smallest eigenvalue), compiled for the host from the
kernel source, against the reference's closed form (the oracle, pinned to
scripts/gvom.py:1423-1487) on the combined covariances of every golden
fixture, at the parity tolerance.  The device's approximate division and
reciprocal square root are taken as correctly rounded ones here, which
moves results by a few float32 ulps, far inside the tolerance."""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, golden_files
from oracle.canonical import canonical_state
from oracle.oracle import OracleGvom
from replay import assert_eigen, load, ops_of, params_of

HERE = os.path.dirname(os.path.abspath(__file__))
KERNEL = os.path.join(os.path.dirname(HERE), "gvom_gb300", "csrc", "k_combine.cu")

PRELUDE = r"""
#include <cmath>
using std::fabs; using std::sqrt;
#define __device__
#define __forceinline__ inline
static inline float __fdividef(float a, float b) { return a / b; }
static inline float rsqrtf(float x) { return 1.0f / std::sqrt(x); }
"""

DRIVER = r"""
extern "C" void eigen_all(const float *cov, long long n, float *out) {
    for (long long i = 0; i < n; i++) eigen3(cov + 6 * i, out + 3 * i);
}
"""


def _kernel_eigen_source():
    src = open(KERNEL).read()
    a = src.index("__device__ __forceinline__ void jacobi_rot(")
    b = src.index("\n}\n", src.index("__device__ __forceinline__ void eigen3(")) + 3
    return src[a:b]


@pytest.fixture(scope="module")
def eigen_lib(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    d = tmp_path_factory.mktemp("eigen")
    cpp = d / "eigen_host.cpp"
    cpp.write_text(PRELUDE + _kernel_eigen_source() + DRIVER)
    so = d / "libeigen.so"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-o", str(so), str(cpp)],
                   check=True)
    lib = C.CDLL(str(so))
    lib.eigen_all.argtypes = [C.c_void_p, C.c_longlong, C.c_void_p]
    return lib


@pytest.mark.parametrize("name", golden_files())
def test_kernel_eigen_solve_within_tolerance_of_reference(eigen_lib, name):
    fx = load(os.path.join(GOLDEN, name))
    o = OracleGvom(*params_of(fx))
    n_checked = 0
    for op in ops_of(fx):
        if op[0] == "P":
            o.Process_pointcloud(*op[2:])
            continue
        o.combine_maps()
        st = canonical_state(o.combined_state())
        cov = np.ascontiguousarray(np.asarray(st["metrics"], np.float32)[:, 3:9])
        got = np.empty((len(cov), 3), np.float32)
        if len(cov):
            eigen_lib.eigen_all(cov.ctypes.data, len(cov), got.ctypes.data)
        assert_eigen(got, st["eigen"], f"{name} eigenvalues")
        n_checked += len(cov)
    assert n_checked > 0


def test_kernel_eigen_solve_on_random_covariances(eigen_lib):
    """Random symmetric covariances in float32 -- generic, isotropic, two equal
    eigenvalues, planar and linear (the smallest one or two eigenvalues 1e-9
    to 1e-4 of the largest), scales from 1e-6 to 1e2 -- against float64
    eigenvalues of the same float32 matrices (numpy), at the parity
    tolerance."""
    rng = np.random.default_rng(8)
    covs, ref = [], []
    for i in range(6000):
        Q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
        s = 10.0 ** rng.uniform(-6, 2)
        kind = i % 6
        if kind == 0:
            lam = rng.random(3)
        elif kind == 1:
            lam = np.ones(3)
        elif kind == 2:
            lam = np.array([1.0, 1.0, rng.random()])
        elif kind == 3:
            lam = np.array([1.0, rng.random(), rng.random()])
            lam[2] = lam[0] * 10.0 ** rng.uniform(-9, -4)
        elif kind == 4:
            lam = np.array([1.0, 10.0 ** rng.uniform(-9, -4), 10.0 ** rng.uniform(-9, -4)])
        else:
            lam = np.array([1.0, 1.0 - 10.0 ** rng.uniform(-7, -2), rng.random()])
        A = (Q * (lam * s)) @ Q.T
        c = np.array([A[0, 0], A[0, 1], A[0, 2], A[1, 1], A[1, 2], A[2, 2]], np.float32)
        B = np.array([[c[0], c[1], c[2]], [c[1], c[3], c[4]], [c[2], c[4], c[5]]], np.float64)
        covs.append(c)
        ref.append(np.sort(np.linalg.eigvalsh(B))[::-1])
    cov = np.ascontiguousarray(np.array(covs, np.float32))
    got = np.empty((len(cov), 3), np.float32)
    eigen_lib.eigen_all(cov.ctypes.data, len(cov), got.ctypes.data)
    assert_eigen(np.sort(got, axis=1)[:, ::-1], np.array(ref), "random covariances")
