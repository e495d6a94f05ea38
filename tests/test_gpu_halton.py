"""The device Halton sampler (the one the trace kernels call) against the reference's own
radicalInverse outputs (tests/golden/halton_ref.npz, made by tests/golden/make_golden.py
from halton.h): bit-exact in every dimension, over indices from 0 to 2^62 (the 32-bit
and 64-bit digit loops, and the bit-reversal form of base 2)."""
import ctypes
import os

import numpy as np
import pytest

from hussar_gb300 import _lib

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def device_halton(L, index, dim):
    index = np.ascontiguousarray(index, np.uint64)
    out = np.zeros(len(index), np.float32)
    _lib.check(L.hsr_debug_halton(index.ctypes.data_as(ctypes.c_void_p), len(index), int(dim),
                                  out.ctypes.data_as(ctypes.c_void_p)))
    return out


def test_device_halton_matches_reference(product_lib):
    g = np.load(os.path.join(GOLD, "halton_ref.npz"))
    idx, dims, val = g["index"], g["dims"], g["value"]
    for j, d in enumerate(dims):
        got = device_halton(product_lib, idx, d)
        assert np.array_equal(got.view(np.uint32), val[:, j].view(np.uint32)), int(d)


def u64_to_f32(x):
    """Round-to-nearest-even of an unsigned integer to float32 in one step (the C
    conversion the reference applies; numpy would round through float64 first)."""
    n = x.bit_length()
    if n <= 24:
        return np.float32(x)
    shift = n - 24
    m, rem, half = x >> shift, x & ((1 << shift) - 1), 1 << (shift - 1)
    if rem > half or (rem == half and m & 1):
        m += 1
    return np.float32(np.ldexp(np.float64(m), shift))


def test_device_halton_base2_is_bit_reversal(product_lib):
    rng = np.random.default_rng(11)
    idx = np.concatenate([np.arange(4096, dtype=np.uint64),
                          rng.integers(0, 2 ** 63, 4096, dtype=np.uint64) >> rng.integers(0, 63, 4096).astype(np.uint64)])
    got = device_halton(product_lib, idx, 0)
    # the reference's loop: reversed binary digits times 2^-digits, in float
    want = []
    for v in idx.tolist():
        rev, n = 0, 0
        while v:
            rev = rev * 2 + (v & 1)
            v >>= 1
            n += 1
        want.append(min(u64_to_f32(rev) * np.float32(2.0 ** -n), np.float32(0.99999994)))
    assert np.array_equal(got.view(np.uint32), np.array(want, np.float32).view(np.uint32))


def test_device_halton_arguments(product_lib):
    assert product_lib.hsr_debug_halton(None, 4, 0, None) == _lib.HSR_ERR_INVALID_ARGUMENT
    assert product_lib.hsr_debug_halton(None, 0, 0, None) == _lib.HSR_OK
