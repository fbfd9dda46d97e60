"""The reference's 2-D image kernels that no caller launches
(scripts/gvom.py:807-885).

CPU: the oracle's restatement reproduces the reference's own outputs for
__expand_binary and __lowpass_binary, bit for bit (tests/golden/morph_binary.npz,
made by running the unchanged kernels through the sequential stand-in), and
its __convolve equals the kernel's closed form as written (every term reads
input[x + r, y + r]; the reference's own kernel cannot run: its float radius
is rejected by range()).
GPU: gvom_expand_binary / gvom_lowpass_binary / gvom_convolve through the C
ABI equal the fixtures and the oracle bit for bit, on the shared-memory
staged path and on the direct path of radii too large to stage.
Host build: the same kernel file compiled for the host (tests/hostbuild.py)
gives the same outputs on the same cases.
"""
import ctypes as C
import os

import numpy as np
import pytest

from conftest import GOLDEN
from oracle.oracle import convolve, expand_binary, lowpass_binary

FIX = os.path.join(GOLDEN, "morph_binary.npz")


def _fixture():
    with np.load(FIX) as z:
        return {k: z[k] for k in z.files}


def _cases(fx, kind):
    n = 0
    while f"{kind}{n}_img" in fx:
        yield n
        n += 1


def test_oracle_expand_and_lowpass_equal_reference_fixture():
    fx = _fixture()
    ne = nl = 0
    for n in _cases(fx, "expand"):
        np.testing.assert_array_equal(expand_binary(fx[f"expand{n}_img"], fx[f"expand{n}_r"]), fx[f"expand{n}_out"])
        ne += 1
    for n in _cases(fx, "lowpass"):
        got = lowpass_binary(fx[f"lowpass{n}_img"], fx[f"lowpass{n}_fs"], fx[f"lowpass{n}_frac"])
        np.testing.assert_array_equal(got, fx[f"lowpass{n}_out"])
        nl += 1
    assert ne >= 6 and nl >= 6


def test_oracle_convolve_as_written():
    rng = np.random.default_rng(5)
    for X, ks in ((17, 3), (17, 4), (30, 5), (9, 1)):
        img = rng.normal(size=(X, X))
        k = rng.normal(size=(ks, ks))
        r = (ks - 1) // 2
        want = np.zeros((X, X))
        for x in range(X):
            for y in range(X):
                if x + r < X and y + r < X:
                    acc = 0.0
                    for v in k[:2 * r + 1, :2 * r + 1].reshape(-1):  # entries [0, 2r] x [0, 2r], row order
                        acc += img[x + r, y + r] * v
                    want[x, y] = acc
        np.testing.assert_array_equal(convolve(img, k), want)


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.mark.gpu
def test_device_image_kernels_equal_reference_and_oracle(gpu_lib):
    import torch
    lib = gpu_lib
    fx = _fixture()
    P = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731
    for n in _cases(fx, "expand"):
        img = _dev(torch, fx[f"expand{n}_img"])
        out = torch.full_like(img, -7)
        assert lib.gvom_expand_binary(P(img), P(out), img.shape[0], float(fx[f"expand{n}_r"]), None) == 0
        torch.cuda.synchronize()
        np.testing.assert_array_equal(out.cpu().numpy(), fx[f"expand{n}_out"], f"expand case {n}")
    for n in _cases(fx, "lowpass"):
        img = _dev(torch, fx[f"lowpass{n}_img"])
        out = torch.full_like(img, -7)
        assert lib.gvom_lowpass_binary(P(img), P(out), img.shape[0], int(fx[f"lowpass{n}_fs"]),
                                       float(fx[f"lowpass{n}_frac"]), None) == 0
        torch.cuda.synchronize()
        np.testing.assert_array_equal(out.cpu().numpy(), fx[f"lowpass{n}_out"], f"lowpass case {n}")
    rng = np.random.default_rng(9)
    # radii / windows beyond the shared-memory staging (direct loads), and a 256 x 256 map
    for X, r in ((100, 60.0), (256, 3.3), (70, 45.5)):
        a = (rng.uniform(size=(X, X)) < 0.003).astype(np.int32)
        img = _dev(torch, a)
        out = torch.full_like(img, -7)
        assert lib.gvom_expand_binary(P(img), P(out), X, r, None) == 0
        torch.cuda.synchronize()
        np.testing.assert_array_equal(out.cpu().numpy(), expand_binary(a, r), f"expand {X} {r}")
    for X, fs, frac in ((100, 45, 0.5), (256, 2, 0.6)):
        a = (rng.uniform(size=(X, X)) < 0.5).astype(np.int32)
        img = _dev(torch, a)
        out = torch.full_like(img, -7)
        assert lib.gvom_lowpass_binary(P(img), P(out), X, fs, frac, None) == 0
        torch.cuda.synchronize()
        np.testing.assert_array_equal(out.cpu().numpy(), lowpass_binary(a, fs, frac), f"lowpass {X} {fs}")
    for X, ks in ((256, 5), (33, 4), (40, 1)):
        a = rng.normal(size=(X, X))
        k = rng.normal(size=(ks, ks))
        img, kd = _dev(torch, a), _dev(torch, k)
        out = torch.full_like(img, float("nan"))
        assert lib.gvom_convolve(P(img), P(out), P(kd), X, ks, None) == 0
        torch.cuda.synchronize()
        np.testing.assert_array_equal(out.cpu().numpy(), convolve(a, k), f"convolve {X} {ks}")
    # arguments the kernels cannot take are refused before any launch
    assert lib.gvom_expand_binary(None, None, 8, 1.0, None) == 2
    assert lib.gvom_lowpass_binary(P(img), P(out), 8, -1, 0.5, None) == 2
    assert lib.gvom_convolve(P(img), P(out), P(kd), 8, 0, None) == 2


MORPH_DRIVER = r"""
extern "C" int run_expand(const int32_t *in, int32_t *out, int X, double r) {
    return gvom::launch_expand_binary(in, out, X, r, nullptr);
}
extern "C" int run_lowpass(const int32_t *in, int32_t *out, int X, int fs, double frac) {
    return gvom::launch_lowpass_binary(in, out, X, fs, frac, nullptr);
}
extern "C" int run_convolve(const double *in, double *out, const double *kern, int X, int ks) {
    return gvom::launch_convolve(in, out, kern, X, ks, nullptr);
}
"""


@pytest.fixture(scope="module")
def morph_host(tmp_path_factory):
    import shutil
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    from hostbuild import CSRC, PRELUDE, compile_units, host_source
    src = host_source(open(os.path.join(CSRC, "k_morph.cu")).read())
    so = compile_units({"morph.cpp": PRELUDE + src + MORPH_DRIVER}, tmp_path_factory.mktemp("morph"), "libmorph.so")
    lib = C.CDLL(str(so))
    P = C.c_void_p
    lib.run_expand.argtypes = [P, P, C.c_int, C.c_double]
    lib.run_lowpass.argtypes = [P, P, C.c_int, C.c_int, C.c_double]
    lib.run_convolve.argtypes = [P, P, P, C.c_int, C.c_int]
    return lib


def test_host_build_image_kernels_equal_reference_and_oracle(morph_host):
    """k_morph.cu compiled unchanged for the host (its launches and dynamic
    shared staging rewritten for a host compiler, blocks run one fiber per
    CUDA thread): the reference's own outputs on every fixture case, and the
    oracle on the staged and direct paths of the GPU test's sizes."""
    lib = morph_host
    fx = _fixture()
    P = lambda a: a.ctypes.data  # noqa: E731
    for n in _cases(fx, "expand"):
        img = np.ascontiguousarray(fx[f"expand{n}_img"], np.int32)
        out = np.full_like(img, -7)
        assert lib.run_expand(P(img), P(out), img.shape[0], float(fx[f"expand{n}_r"])) == 0
        np.testing.assert_array_equal(out, fx[f"expand{n}_out"], f"expand case {n}")
    for n in _cases(fx, "lowpass"):
        img = np.ascontiguousarray(fx[f"lowpass{n}_img"], np.int32)
        out = np.full_like(img, -7)
        assert lib.run_lowpass(P(img), P(out), img.shape[0], int(fx[f"lowpass{n}_fs"]),
                               float(fx[f"lowpass{n}_frac"])) == 0
        np.testing.assert_array_equal(out, fx[f"lowpass{n}_out"], f"lowpass case {n}")
    rng = np.random.default_rng(9)
    for X, r in ((100, 60.0), (64, 3.3), (70, 45.5)):
        a = (rng.uniform(size=(X, X)) < 0.003).astype(np.int32)
        out = np.full_like(a, -7)
        assert lib.run_expand(P(a), P(out), X, r) == 0
        np.testing.assert_array_equal(out, expand_binary(a, r), f"expand {X} {r}")
    for X, fs, frac in ((100, 45, 0.5), (64, 2, 0.6)):
        a = (rng.uniform(size=(X, X)) < 0.5).astype(np.int32)
        out = np.full_like(a, -7)
        assert lib.run_lowpass(P(a), P(out), X, fs, frac) == 0
        np.testing.assert_array_equal(out, lowpass_binary(a, fs, frac), f"lowpass {X} {fs}")
    for X, ks in ((64, 5), (33, 4), (40, 1)):
        a = rng.normal(size=(X, X))
        k = rng.normal(size=(ks, ks))
        out = np.full_like(a, np.nan)
        assert lib.run_convolve(P(a), P(out), P(k), X, ks) == 0
        np.testing.assert_array_equal(out, convolve(a, k), f"convolve {X} {ks}")
