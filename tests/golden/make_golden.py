"""Generates the golden fixtures in this directory from the reference's own code.

Runs only where the reference tree is mounted: it builds oracle/_ref/libhsr_ref.so
with oracle/Makefile.ref (which compiles the reference's halton.h and radar.h in
place) and records their outputs for seeded inputs:

  halton_ref.npz   radicalInverse(index, dim) for dims 0..11      (halton.h:38-67)
  splat_ref.npz    Frame::splat<16> on random fractional indices  (radar.h:564-626)
  settime_ref.npz  PIndex::setTime                               (radar.h:232-241)
  cexp_ref.npz     std::exp(Complex(0, angle)) via radar::polar   (complex.h:184-187,249-251)

Usage: python tests/golden/make_golden.py
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))


def main():
    subprocess.check_call(["make", "-s", "-f", os.path.join(ROOT, "oracle", "Makefile.ref")])
    ref = ctypes.CDLL(os.path.join(ROOT, "oracle", "_ref", "libhsr_ref.so"))
    fp = ctypes.POINTER(ctypes.c_float)
    ref.ref_radical_inverse.restype = ctypes.c_float
    ref.ref_radical_inverse.argtypes = [ctypes.c_uint64, ctypes.c_int]
    ref.ref_frame_splat.argtypes = [ctypes.c_int] * 3 + [ctypes.c_float] * 5 + [fp]
    ref.ref_set_time.restype = ctypes.c_float
    ref.ref_set_time.argtypes = [ctypes.c_float] * 4 + [ctypes.c_int]
    ref.ref_cexp.argtypes = [ctypes.c_float, fp]

    rng = np.random.default_rng(0x600D)
    # --- Halton: small indices densely, large ones sparsely, dims past the table
    idx = np.concatenate([np.arange(0, 4096), rng.integers(0, 2**24, 2048),
                          rng.integers(0, 2**62, 512)]).astype(np.uint64)
    dims = np.arange(12)
    vals = np.zeros((len(idx), len(dims)), np.float32)
    for i, v in enumerate(idx):
        for d in dims:
            vals[i, d] = ref.ref_radical_inverse(int(v), int(d))
    np.savez_compressed(os.path.join(HERE, "halton_ref.npz"), index=idx, dims=dims, value=vals)

    # --- Frame::splat<16>
    cases = []
    frames = []
    for k in range(400):
        n = int(rng.choice([1, 7, 16, 64, 256, 512]))
        ch = int(rng.choice([1, 4]))
        cc = int(rng.choice([1, 3]))
        mode = k % 4
        if mode == 0:
            s = rng.uniform(-2.0, n + 2.0)
        elif mode == 1:
            s = np.floor(rng.uniform(0, n - 1)) + rng.choice([0.0, 4e-5, -4e-5, 0.5, -0.5, 2e-4])
        elif mode == 2:
            s = rng.uniform(0, n - 1)
        else:
            s = np.floor(rng.uniform(0, n - 1)) + 0.5
        c = float(rng.choice([0.0, 1.0, 0.25])) if cc > 1 else 0.0
        chn = float(rng.choice([0.0, 2.0])) if ch > 1 else 0.0
        s = float(np.float32(s))
        # the reference writes out of bounds for a delta index rounded up to n; skip those
        if abs(s - np.round(s)) < 1e-4 and (np.round(s) >= n or np.round(s) < 0):
            continue
        re, im = (float(x) for x in rng.normal(size=2).astype(np.float32))
        out = np.zeros(2 * cc * n * ch, np.float32)
        ref.ref_frame_splat(cc, n, ch, c, s, chn, re, im, out.ctypes.data_as(fp))
        cases.append((cc, n, ch, c, s, chn, re, im))
        frames.append(out)
    offsets = np.cumsum([0] + [len(f) for f in frames]).astype(np.int64)
    np.savez_compressed(os.path.join(HERE, "splat_ref.npz"),
                        cases=np.array(cases, np.float64), offsets=offsets,
                        frames=np.concatenate(frames))

    # --- setTime and cexp
    dts = rng.uniform(0, 2.5e-7, 4000).astype(np.float32)
    cfg = [(77e9, 78.125e12, 5e6, 256), (77e9, 78.125e12, 10e6, 512), (78e9, 60e12, 5e6, 256)]
    st = np.zeros((len(cfg), len(dts)), np.float32)
    for j, (f0, sl, ad, n) in enumerate(cfg):
        for i, dt in enumerate(dts):
            st[j, i] = ref.ref_set_time(float(dt), f0, sl, ad, n)
    np.savez_compressed(os.path.join(HERE, "settime_ref.npz"), dt=dts,
                        cfg=np.array(cfg, np.float64), sample=st)
    ang = np.concatenate([rng.uniform(-10, 10, 2000), rng.uniform(0, 7e4, 2000)]).astype(np.float32)
    ce = np.zeros((len(ang), 2), np.float32)
    tmp = np.zeros(2, np.float32)
    for i, a in enumerate(ang):
        ref.ref_cexp(float(a), tmp.ctypes.data_as(fp))
        ce[i] = tmp
    np.savez_compressed(os.path.join(HERE, "cexp_ref.npz"), angle=ang, value=ce)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
