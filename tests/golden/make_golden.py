"""Generates the golden fixtures in this directory from the reference's own code.

Runs only where the reference tree is mounted: it builds oracle/_ref/libhsr_ref.so
with oracle/Makefile.ref (which compiles the reference's halton.h and radar.h in
place) and records their outputs for seeded inputs:

  halton_ref.npz   radicalInverse(index, dim) for dims 0..11      (halton.h:38-67)
  splat_ref.npz    Frame::splat<16> on random fractional indices  (radar.h:564-626)
  settime_ref.npz  PIndex::setTime                               (radar.h:232-241)
  cexp_ref.npz     std::exp(Complex(0, angle)) via radar::polar   (complex.h:184-187,249-251)

and, from oracle/_ref/libhsr_refpath.so (the reference's PathTracer::run and
PathTracer::sample with its emitters, geometry, integrator and frame, over stand-ins
for the absent Eigen, libguiding and Embree; oracle/ref_path.cpp):

  path_ref.npz     raw frame sums and total weight of PathTracer::run (doGuiding =
                   false) on the dihedral, a small sphere above ground and a small boxes
                   scene, across the tracer flags (path.h:153-169); the meshes are stored
  sample_ref.npz   UniformSampleSphere (sampling.h:38-43), Integrator::measureRay
                   (integrator.h:107-110) and HaltonSampler::get2D (halton.h:23-26)

Usage: HUSSAR_REFERENCE=<reference checkout> python tests/golden/make_golden.py
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
    path_fixtures(rng)
    print("golden fixtures written to", HERE)


def path_fixtures(rng):
    import sys
    sys.path.insert(0, ROOT)
    from hussar_gb300 import PathTracer, _lib, scenes
    from hussar_gb300.core import NFAntenna, TriangleMesh

    R = ctypes.CDLL(os.path.join(ROOT, "oracle", "_ref", "libhsr_refpath.so"))
    fp = ctypes.POINTER(ctypes.c_float)
    vp = ctypes.c_void_p
    R.ref_path_frame.argtypes = [vp, ctypes.c_int64, vp, ctypes.c_int64, vp, vp, vp, vp, vp, ctypes.c_int64, vp,
                                 ctypes.POINTER(ctypes.c_double)]
    R.ref_uniform_sample_sphere.argtypes = [ctypes.c_float, ctypes.c_float, fp]
    R.ref_measure_ray.argtypes = [ctypes.c_float] * 3 + [fp]
    R.ref_halton_get2d.argtypes = [ctypes.c_uint64, ctypes.c_int, fp]

    dih = scenes.dihedral_workload()
    sph = scenes.sphere_ground_workload(level=3)
    box_mesh = scenes.boxes_mesh(seed=5, count=400, extent=30.0)
    one = TriangleMesh()
    one.append(np.array([[0, -0.2, -0.2], [0, 0.3, -0.2], [0, 0.0, 0.4]], np.float32), [[0, 1, 2]])
    meshes = [dih.mesh, sph.mesh, box_mesh, one]
    rf_sph = sph.rf
    rf_dih = dih.rf
    box_pose = NFAntenna(np.array([2.0, 1.0, -3.0], np.float32), scenes.looking(0.7))
    a1 = NFAntenna([1.0, 0.05, 0.3], scenes.looking(0.3))
    a2 = NFAntenna([1.0, 0.05, 0.35], scenes.looking(0.3))
    cw = scenes.RFConfig(startFreq=78e9, freqSlope=0.0, adcRate=5e6, idleTime=1e-4, rampTime=5e-5)

    def tr(depth, **kw):
        t = PathTracer()
        t.doGuiding = False
        t.maxDepth = depth
        for k, v in kw.items():
            setattr(t, k, v)
        return t

    # (mesh, rf, N, tx, rx, tracer, budget)
    cases = [
        (0, rf_dih, 256, dih.tx[45], dih.rx[45], tr(2), 1 << 14),
        (0, rf_dih, 256, dih.tx[10], dih.rx[10], tr(2), 1 << 13),
        (0, rf_dih, 256, dih.tx[20], dih.rx[22], tr(2, onlyIndirect=False), 1 << 13),
        (0, rf_dih, 256, dih.tx[60], dih.rx[60], tr(2, useGeometricalOptics=False), 1 << 12),
        (0, rf_dih, 200, dih.tx[45], dih.rx[45], tr(2), 1 << 12),
        (0, rf_dih, 256, dih.tx[30], dih.rx[30], tr(2, produceDebugImage=True), 1 << 12),
        (1, rf_sph, 512, sph.tx[0], sph.rx[0], tr(3), 1 << 13),
        (1, rf_sph, 512, sph.tx[0], sph.rx[0], tr(3, doFiltering=False), 1 << 12),
        (1, rf_sph, 512, sph.tx[0], sph.rx[0], tr(3, filteringSphere=False), 1 << 12),
        (1, rf_sph, 512, sph.tx[0], sph.rx[0], tr(3, correctPhase=True), 1 << 12),
        (1, rf_sph, 512, sph.tx[0], sph.rx[0], tr(3, poDiffraction=True), 1 << 12),
        (1, rf_sph, 512, sph.tx[0], sph.rx[0], tr(3, useGeometricalOptics=False), 1 << 12),
        (2, rf_dih, 256, box_pose, box_pose, tr(4), 1 << 12),
        (3, rf_dih, 256, a1, a1, tr(3), 1 << 13),
        (3, rf_dih, 256, a1, a2, tr(3, onlyIndirect=False), 1 << 12),
        (3, cw, 1, a1, a1, tr(3), 1 << 12),
    ]
    rows, out_frames, weights, offs = [], [], [], [0]
    for mi, rf, N, tx, rx, t, budget in cases:
        m = meshes[mi]
        v = np.ascontiguousarray(m.vertexBuffer, np.float32)
        f = np.ascontiguousarray(m.indexBuffer, np.int32)
        rfc, fcc = rf.to_c(), _lib.FrameConfigC(1, N, 1)
        txc, rxc, flc = tx.to_c(), rx.to_c(), t.flags_c()
        fr = np.zeros(2 * N, np.float32)
        w = ctypes.c_double()
        rc = R.ref_path_frame(v.ctypes.data, len(v), f.ctypes.data, len(f), ctypes.addressof(rfc),
                              ctypes.addressof(fcc), ctypes.addressof(txc), ctypes.addressof(rxc),
                              ctypes.addressof(flc), int(budget), fr.ctypes.data, ctypes.byref(w))
        assert rc == 0
        rows.append(np.concatenate([[mi, N, budget], np.frombuffer(bytes(rfc), np.float32),
                                    np.frombuffer(bytes(txc), np.float32), np.frombuffer(bytes(rxc), np.float32),
                                    np.frombuffer(bytes(flc), np.uint8).view(np.int32).astype(np.float64)]))
        out_frames.append(fr)
        weights.append(w.value)
        offs.append(offs[-1] + len(fr))
    mesh_arrays = {}
    for i, m in enumerate(meshes):
        mesh_arrays["mesh%d_v" % i] = np.ascontiguousarray(m.vertexBuffer, np.float32)
        mesh_arrays["mesh%d_f" % i] = np.ascontiguousarray(m.indexBuffer, np.int32)
    np.savez_compressed(os.path.join(HERE, "path_ref.npz"), cases=np.array(rows, np.float64),
                        frames=np.concatenate(out_frames), offsets=np.array(offs, np.int64),
                        weights=np.array(weights, np.float64), **mesh_arrays)

    # primary direction, de-chirp phase and the get2D pair order
    u = rng.random((4000, 2)).astype(np.float32)
    d = np.zeros((len(u), 3), np.float32)
    tmp = np.zeros(3, np.float32)
    for i, (a, b) in enumerate(u):
        R.ref_uniform_sample_sphere(float(a), float(b), tmp.ctypes.data_as(fp))
        d[i] = tmp
    dts = rng.uniform(0, 2.5e-7, 2000).astype(np.float32)
    mr = np.zeros((len(dts), 2), np.float32)
    for i, dt in enumerate(dts):
        R.ref_measure_ray(float(dt), 77e9, 78.125e12, tmp.ctypes.data_as(fp))
        mr[i] = tmp[:2]
    idx = rng.integers(0, 2**40, 500).astype(np.uint64)
    g2 = np.zeros((len(idx), 2), np.float32)
    for i, k in enumerate(idx):
        R.ref_halton_get2d(int(k), 1, tmp.ctypes.data_as(fp))
        g2[i] = tmp[:2]
    np.savez_compressed(os.path.join(HERE, "sample_ref.npz"), u=u, dir=d, dt=dts, measure=mr, get2d_index=idx,
                        get2d=g2)


if __name__ == "__main__":
    main()
