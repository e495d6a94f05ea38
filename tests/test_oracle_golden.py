"""The oracle against the reference's own outputs (tests/golden/*, made by
tests/golden/make_golden.py from the reference's halton.h and radar.h): bit-exact."""
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")


def test_halton_matches_reference(oracle_lib):
    g = np.load(os.path.join(GOLD, "halton_ref.npz"))
    idx, dims, val = g["index"], g["dims"], g["value"]
    got = np.array([[oracle_lib.radical_inverse(int(i), int(d)) for d in dims] for i in idx], np.float32)
    assert np.array_equal(got.view(np.uint32), val.view(np.uint32))


def test_halton_known_answer(oracle_lib):
    # the reference probe's values for index 12345, dims 0..2
    got = [oracle_lib.radical_inverse(12345, d) for d in range(3)]
    assert np.float32(got[0]) == np.float32(0.609558105)
    assert abs(got[1] - 0.246354789) < 1e-7 and abs(got[2] - 0.190272018) < 1e-7
    # dimensions past the reference's table return 0 (halton.h:1082-1084)
    assert oracle_lib.radical_inverse(12345, 10) == 0.0


def test_frame_splat_matches_reference(oracle_lib):
    g = np.load(os.path.join(GOLD, "splat_ref.npz"))
    cases, offs, frames = g["cases"], g["offsets"], g["frames"]
    for k, (cc, n, ch, c, s, chn, re, im) in enumerate(cases):
        want = frames[offs[k]:offs[k + 1]]
        got = oracle_lib.frame_splat(int(cc), int(n), int(ch), float(c), float(s), float(chn), float(re), float(im))
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), (k, cases[k])


def test_settime_matches_reference_bit_exact(oracle_lib):
    """The oracle's PIndex::setTime (the function its splat uses) against the reference's
    own setTime on 4000 delays x 3 RF configurations: identical bits."""
    import ctypes
    g = np.load(os.path.join(GOLD, "settime_ref.npz"))
    L = oracle_lib.lib()
    L.oracle_set_time.restype = ctypes.c_float
    L.oracle_set_time.argtypes = [ctypes.c_float] * 3 + [ctypes.c_int]
    for j, (f0, sl, ad, n) in enumerate(g["cfg"]):
        got = np.array([L.oracle_set_time(float(dt), float(sl), float(ad), int(n)) for dt in g["dt"]], np.float32)
        assert np.array_equal(got.view(np.uint32), g["sample"][j].view(np.uint32)), j


def test_cexp_matches_reference_bit_exact(oracle_lib):
    """The oracle's exp(j angle) (radar::polar, the function its measureRay uses) against the
    reference's std::exp(Complex(0, angle)) on 4000 angles up to 7e4 rad: identical bits."""
    import ctypes
    c = np.load(os.path.join(GOLD, "cexp_ref.npz"))
    L = oracle_lib.lib()
    fp = ctypes.POINTER(ctypes.c_float)
    L.oracle_cexp.argtypes = [ctypes.c_float, fp]
    out = np.zeros(2, np.float32)
    got = np.zeros((len(c["angle"]), 2), np.float32)
    for i, a in enumerate(c["angle"]):
        L.oracle_cexp(float(a), out.ctypes.data_as(fp))
        got[i] = out
    assert np.array_equal(got.view(np.uint32), c["value"].view(np.uint32))


def test_measure_ray_is_cexp_of_the_float_angle(oracle_lib):
    """measureRay forms its angle in float in the reference's order, then exp(j angle)."""
    import ctypes
    L = oracle_lib.lib()
    fp = ctypes.POINTER(ctypes.c_float)
    L.oracle_measure_ray.argtypes = [ctypes.c_float] * 3 + [fp]
    L.oracle_cexp.argtypes = [ctypes.c_float, fp]
    rng = np.random.default_rng(3)
    a, b = np.zeros(2, np.float32), np.zeros(2, np.float32)
    f32 = np.float32
    for dt in rng.uniform(0, 2.5e-7, 500).astype(np.float32):
        L.oracle_measure_ray(float(dt), 77e9, 78.125e12, a.ctypes.data_as(fp))
        ang = f32(2) * f32(np.pi) * (f32(77e9) - dt * f32(78.125e12) / f32(2)) * dt
        L.oracle_cexp(float(ang), b.ctypes.data_as(fp))
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_rounded_sincos_is_correctly_rounded(oracle_lib):
    """The primary direction's sin/cos (what the GPU computes): the correctly rounded float
    values, checked against sin/cos in double rounded to float, on every angle 2 pi u of a
    2^20-point grid of u and on random angles in [0, 2 pi)."""
    import ctypes
    L = oracle_lib.lib()
    fp = ctypes.POINTER(ctypes.c_float)
    L.oracle_sincos_rounded.argtypes = [ctypes.c_float, fp, fp]
    f32 = np.float32
    u = np.arange(0, 1 << 20, 7, dtype=np.float64) / (1 << 20)
    x = np.concatenate([f32(2) * f32(np.pi) * u.astype(np.float32),
                        np.random.default_rng(1).uniform(0, 2 * np.pi, 20000).astype(np.float32)])
    s, c = np.zeros(1, np.float32), np.zeros(1, np.float32)
    got = np.zeros((len(x), 2), np.float32)
    for i, v in enumerate(x):
        L.oracle_sincos_rounded(float(v), s.ctypes.data_as(fp), c.ctypes.data_as(fp))
        got[i] = s[0], c[0]
    want = np.stack([np.sin(x.astype(np.float64)), np.cos(x.astype(np.float64))], 1).astype(np.float32)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def test_path_frames_match_reference_bit_exact(oracle_lib):
    """The restatement's PathTracer::run (FP32, one thread, the platform's sinf/cosf in the
    primary direction as a GCC build of the reference uses) against the reference's own
    PathTracer::run compiled from its sources (oracle/ref_path.cpp over stand-ins for
    Eigen, libguiding and Embree; tests/golden/make_golden.py): identical raw frame sums,
    bit for bit, and identical total weights, on the dihedral, a sphere above ground and a
    boxes scene, over the tracer flags and edge cases (direct path, non-GO sampling,
    non-power-of-two N, debug-image early-out, CW chirp)."""
    import ctypes
    g = np.load(os.path.join(GOLD, "path_ref.npz"))
    L = oracle_lib.lib()
    scenes_ = {}
    L.oracle_set_libm_trig(1)
    try:
        for k, row in enumerate(g["cases"]):
            mi, N, budget = int(row[0]), int(row[1]), int(row[2])
            rf = row[3:9].astype(np.float32)
            tx = row[9:21].astype(np.float32)
            rx = row[21:33].astype(np.float32)
            fl = row[33:47].astype(np.int64).astype(np.int32)
            if mi not in scenes_:
                v, f = g["mesh%d_v" % mi], g["mesh%d_f" % mi]
                scenes_[mi] = L.oracle_scene_create(v.ctypes.data_as(ctypes.c_void_p), len(v),
                                                    f.ctypes.data_as(ctypes.c_void_p), len(f))
                assert scenes_[mi]
            fc = np.array([1, N, 1], np.int32)
            out = np.zeros(2 * N, np.float64)
            w = ctypes.c_double(0.0)
            P = oracle_lib
            rc = L.oracle_simulate(ctypes.c_void_p(scenes_[mi]), ctypes.byref(P.RF.from_buffer_copy(rf.tobytes())),
                                   ctypes.byref(P.FC.from_buffer_copy(fc.tobytes())),
                                   ctypes.byref(P.ANT.from_buffer_copy(tx.tobytes())),
                                   ctypes.byref(P.ANT.from_buffer_copy(rx.tobytes())),
                                   ctypes.byref(P.FLAGS.from_buffer_copy(fl.tobytes())), budget, 0, 1.0, 32, 1,
                                   out.ctypes.data_as(ctypes.c_void_p), ctypes.byref(w))
            assert rc == 0, k
            want = g["frames"][g["offsets"][k]:g["offsets"][k + 1]]
            got = out.astype(np.float32)
            assert np.array_equal(out, got.astype(np.float64)), k  # float sums, carried exactly
            assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), (k, np.abs(got - want).max())
            assert w.value == g["weights"][k], k
    finally:
        L.oracle_set_libm_trig(0)
        for h in scenes_.values():
            L.oracle_scene_destroy(ctypes.c_void_p(h))


def test_sampling_and_phase_match_reference_bit_exact(oracle_lib):
    """UniformSampleSphere (with the platform's sinf/cosf), Integrator::measureRay and the
    order of HaltonSampler::get2D's pair against the reference's own compiled code."""
    import ctypes
    g = np.load(os.path.join(GOLD, "sample_ref.npz"))
    L = oracle_lib.lib()
    fp = ctypes.POINTER(ctypes.c_float)
    L.oracle_uniform_sample_sphere.argtypes = [ctypes.c_float, ctypes.c_float, fp]
    L.oracle_measure_ray.argtypes = [ctypes.c_float] * 3 + [fp]
    tmp = np.zeros(3, np.float32)
    L.oracle_set_libm_trig(1)
    try:
        d = np.zeros_like(g["dir"])
        for i, (a, b) in enumerate(g["u"]):
            L.oracle_uniform_sample_sphere(float(a), float(b), tmp.ctypes.data_as(fp))
            d[i] = tmp
    finally:
        L.oracle_set_libm_trig(0)
    assert np.array_equal(d.view(np.uint32), g["dir"].view(np.uint32))
    m = np.zeros_like(g["measure"])
    for i, dt in enumerate(g["dt"]):
        L.oracle_measure_ray(float(dt), 77e9, 78.125e12, tmp.ctypes.data_as(fp))
        m[i] = tmp[:2]
    assert np.array_equal(m.view(np.uint32), g["measure"].view(np.uint32))
    # get2D after one get1D: (dimension 2, dimension 1) in a GCC build
    pair = np.array([[oracle_lib.radical_inverse(int(k), 2), oracle_lib.radical_inverse(int(k), 1)]
                     for k in g["get2d_index"]], np.float32)
    assert np.array_equal(pair.view(np.uint32), g["get2d"].view(np.uint32))
