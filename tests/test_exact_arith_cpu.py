"""Host check of the integer implementation of the reference's float64 voxel
arithmetic (gvom_gb300/csrc/gvom_exact.cuh, the same source the scan kernel
compiles): end = RN32(RN64(p/r)), b = floor(RN64(RN64(p/r) - o)) and
frac = RN32(t - b) must match native IEEE float64 bit for bit on random and
adversarial inputs over 12 voxel sizes; and the integer ray step count
(gx_step_count) must equal the float64 loop it replaces, including rays whose
length sits at a step boundary and increments whose additions tie."""
import os
import shutil
import subprocess

import pytest

from conftest import REPO


def test_integer_voxel_arithmetic_matches_float64(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    exe = str(tmp_path / "exact_check")
    subprocess.run([gxx, "-std=c++17", "-O2", "-ffp-contract=off", "-o", exe,
                    os.path.join(REPO, "tests", "cpp", "exact_check.cpp")], check=True)
    r = subprocess.run([exe, "150000"], capture_output=True, text=True, timeout=300)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert " 0 mismatches" in r.stdout
    assert " 0 step-count mismatches" in r.stdout
