"""Compiled-Numba scalar typing on top of NumPy 2 (test infrastructure)."""
from __future__ import annotations

import math as _math
import operator as _op

import numpy as np


def _is_py_number(x):
    return isinstance(x, (bool, int, float)) and not isinstance(x, np.generic)


class NF32(np.float32):
    """A float32 scalar with compiled-Numba promotion rules.

    float32 (op) float32 -> float32; float32 (op) Python int/float literal ->
    float64 (Numba types literals as int64 / float64); float32 (op) any other
    NumPy scalar -> NumPy's own promotion (float64 for float64 / int32 / int64).
    Comparisons are exact (mixed operands compared as float64).
    """

    __slots__ = ()

    def _bin(self, other, fn, reflected):
        a = np.float32(self)
        if isinstance(other, np.float32):
            b = np.float32(other)
            return NF32(fn(b, a) if reflected else fn(a, b))
        if _is_py_number(other):
            a64 = np.float64(a)
            b64 = np.float64(other)
            return fn(b64, a64) if reflected else fn(a64, b64)
        r = fn(other, a) if reflected else fn(a, other)
        if type(r) is np.float32:
            return NF32(r)
        return r

    def __add__(self, o): return self._bin(o, _op.add, False)
    def __radd__(self, o): return self._bin(o, _op.add, True)
    def __sub__(self, o): return self._bin(o, _op.sub, False)
    def __rsub__(self, o): return self._bin(o, _op.sub, True)
    def __mul__(self, o): return self._bin(o, _op.mul, False)
    def __rmul__(self, o): return self._bin(o, _op.mul, True)
    def __truediv__(self, o): return self._bin(o, _op.truediv, False)
    def __rtruediv__(self, o): return self._bin(o, _op.truediv, True)

    def __neg__(self): return NF32(-np.float32(self))
    def __pos__(self): return self
    def __abs__(self): return NF32(abs(np.float32(self)))

    def _cmp(self, other, fn):
        if isinstance(other, np.float32):
            return bool(fn(np.float32(self), np.float32(other)))
        return bool(fn(np.float64(self), np.float64(other)))

    def __lt__(self, o): return self._cmp(o, _op.lt)
    def __le__(self, o): return self._cmp(o, _op.le)
    def __gt__(self, o): return self._cmp(o, _op.gt)
    def __ge__(self, o): return self._cmp(o, _op.ge)
    def __eq__(self, o): return self._cmp(o, _op.eq)
    def __ne__(self, o): return self._cmp(o, _op.ne)
    __hash__ = np.float32.__hash__


def wrap_scalar(v):
    if type(v) is np.float32:
        return NF32(v)
    return v


class _MathProxy:
    """`math` as compiled Numba types it: sqrt(float32) is a float32 sqrt."""

    def __getattr__(self, name):
        return getattr(_math, name)

    @staticmethod
    def sqrt(x):
        if isinstance(x, np.float32):
            return NF32(np.sqrt(np.float32(x)))
        return _math.sqrt(x)

    @staticmethod
    def floor(x):
        return int(np.floor(np.float64(x)))


math_proxy = _MathProxy()
