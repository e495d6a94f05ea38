"""The primary direction's sine and cosine on the device (UniformSampleSphere in the
reference-phase kernels): the fast certified evaluation gives the double-precision
evaluation's bits for every float in [-8, 8], which holds the angle 2 pi u of every
Halton point. The double-precision evaluation is the one the CPU restatement computes
(the per-sample record tests compare primary directions bit for bit)."""
import ctypes
import struct

import pytest

from hussar_gb300 import _lib

pytestmark = pytest.mark.gpu


def sweep(L, lo, hi):
    n, m, s = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
    _lib.check(L.hsr_debug_sincos_sweep(lo, hi, ctypes.byref(n), ctypes.byref(m), ctypes.byref(s)))
    return n.value, m.value, s.value


def bits(x):
    return struct.unpack("<I", struct.pack("<f", x))[0]


def test_device_sincos_every_float(product_lib):
    n, m, s = sweep(product_lib, 0.0, 8.0)
    assert n == 2 * (bits(8.0) + 1)
    assert m == 0
    # the sampler's angles 2 pi u, u in [0, 1): nearly all take the fast evaluation
    n, m, s = sweep(product_lib, 0.5, 6.2831855)
    print("fallback fraction %.2e" % (s / n))
    assert m == 0 and s < 1e-3 * n
