"""The shared-divisor division of the FP64 kernels (div_r, Markstein's method
with the correctly rounded reciprocal) against the IEEE division: the
bit-exact FD Jacobian depends on every quotient being the IEEE one.  The
parity tests check it on the real operands; this checks 2^30 random pairs,
including awkward divisor mantissas, bit for bit."""
import ctypes
import os

import numpy as np
import pytest

from ve_flow_around_cylinder_fortran_gb300 import build as B

pytestmark = pytest.mark.gpu


def test_div_r_equals_ieee_division():
    B.build()
    L = ctypes.CDLL(B.PROBE)
    L.vefem_probe_div.argtypes = [ctypes.c_int, ctypes.c_ulonglong, ctypes.c_ulonglong,
                                  ctypes.c_void_p, ctypes.c_void_p]
    mism = ctypes.c_ulonglong(0)
    ex = np.zeros(4)
    for seed in (1, 2):
        rc = L.vefem_probe_div(0, 1 << 30, seed, ctypes.byref(mism), ex.ctypes.data)
        assert rc == 0
        assert mism.value == 0, f"first mismatch x={ex[0]!r} y={ex[1]!r} got {ex[2]!r} want {ex[3]!r}"
