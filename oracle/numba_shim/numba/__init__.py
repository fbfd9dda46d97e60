"""TEST INFRASTRUCTURE - a sequential stand-in for the `numba` package.

`numba` (and llvmlite) are not installed in this build environment and there
is no network, so the reference mapper (scripts/gvom.py) cannot be imported
as shipped.  This package, put first on sys.path by tests/golden/make_golden.py
only, provides exactly the surface that file uses -- ``cuda.jit``,
``cuda.grid``, ``cuda.atomic.add/min``, ``cuda.local.array``,
``cuda.to_device``, ``cuda.device_array``, ``.copy_to_host()``,
``numba.float32/float64`` -- and executes every launched kernel thread by
thread, in block/thread order, on the host.  That is a valid schedule of the
reference's launches (its only cross-thread interactions are atomics).

Scalar typing follows compiled Numba, not NumPy 2: a float32 value read from
an array is an `NF32` whose arithmetic with another float32 stays float32 but
with a Python float / int literal (Numba: float64 / int64) or a float64 value
becomes float64; ``math.sqrt`` of a float32 is float32.  Float scalar kernel
arguments are float64, as Numba types Python floats.  The reference module's
``math`` global is replaced by `math_proxy` for that (see make_golden.py).
"""
from __future__ import annotations

import math as _math

import numpy as np

from . import cuda  # noqa: F401  (``from numba import cuda``)
from ._types import NF32, math_proxy  # noqa: F401

float32 = np.float32
float64 = np.float64
int32 = np.int32
int64 = np.int64

__version__ = "0.0-shim"


def jit(*args, **kwargs):  # host-side numba.jit: identity decorator (unused by the reference)
    if args and callable(args[0]) and len(args) == 1 and not kwargs:
        return args[0]
    return lambda f: f


def vectorize(*args, **kwargs):  # imported by the reference, never used
    return jit(*args, **kwargs)
