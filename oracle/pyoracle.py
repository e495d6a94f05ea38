"""ORACLE — TEST INFRASTRUCTURE ONLY.

ctypes binding of liboracle.so (the CPU restatement in hsr_oracle.cpp). Imported only
by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")


class RF(ctypes.Structure):
    _fields_ = [(n, ctypes.c_float) for n in
                ("startFreq", "freqSlope", "adcRate", "idleTime", "rampTime", "antennaDelay")]


class FC(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int32) for n in ("chirpCount", "samplesPerChirp", "channelCount")]


class ANT(ctypes.Structure):
    _fields_ = [("position", ctypes.c_float * 3), ("rotation", ctypes.c_float * 9)]


class FFANT(ctypes.Structure):
    _fields_ = [("direction", ctypes.c_float * 3), ("polarization", ctypes.c_float * 6),
                ("scene_center", ctypes.c_float * 3), ("radius", ctypes.c_float)]


class FLAGS(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int32) for n in
                ("onlyIndirect", "maxDepth", "useGeometricalOptics", "poDiffraction", "doGuiding",
                 "clearBeforeIteration", "correctPhase", "filterGuiding", "doFiltering", "filteringSphere",
                 "produceDebugImage")] + \
              [(n, ctypes.c_float) for n in ("filteringMin", "filteringMax", "filteringRadius")]


RECORD_DTYPE = np.dtype([("depth", "<i4"), ("splatted", "<i4"), ("time", "<f8"), ("v_re", "<f8"),
                         ("v_im", "<f8"), ("dphase", "<f8"), ("bin", "<f8"), ("value_re", "<f8"),
                         ("value_im", "<f8")])

_lib = None


def build():
    subprocess.check_call(["make", "-s", "-C", HERE])


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = ctypes.CDLL(LIB)
        vp = ctypes.c_void_p
        P = ctypes.POINTER
        L.oracle_radical_inverse_f.restype = ctypes.c_float
        L.oracle_radical_inverse_f.argtypes = [ctypes.c_uint64, ctypes.c_int]
        L.oracle_radical_inverse_d.restype = ctypes.c_double
        L.oracle_radical_inverse_d.argtypes = [ctypes.c_uint64, ctypes.c_int]
        L.oracle_scene_create.restype = vp
        L.oracle_scene_create.argtypes = [vp, ctypes.c_int64, vp, ctypes.c_int64]
        L.oracle_scene_destroy.argtypes = [vp]
        L.oracle_bvh_nodes.restype = ctypes.c_int64
        L.oracle_bvh_nodes.argtypes = [vp]
        L.oracle_intersect.argtypes = [vp, ctypes.c_int64, vp, vp, vp, vp, vp, vp, vp]
        L.oracle_visible.argtypes = [vp, ctypes.c_int64, vp, vp, vp, vp]
        L.oracle_simulate.argtypes = [vp, P(RF), P(FC), P(ANT), P(ANT), P(FLAGS), ctypes.c_int64, ctypes.c_int64,
                                      ctypes.c_float, ctypes.c_int, ctypes.c_int, vp, P(ctypes.c_double)]
        L.oracle_simulate_ff.argtypes = [vp, P(RF), P(FC), P(FFANT), P(FFANT), P(FLAGS), ctypes.c_int64,
                                         ctypes.c_int64, ctypes.c_float, ctypes.c_int, ctypes.c_int, vp,
                                         P(ctypes.c_double)]
        L.oracle_records.argtypes = [vp, P(RF), P(FC), P(ANT), P(ANT), P(FLAGS), ctypes.c_int64, ctypes.c_int64,
                                     ctypes.c_int64, ctypes.c_int, vp]
        fp = P(ctypes.c_float)
        L.oracle_frame_splat.argtypes = [ctypes.c_int] * 3 + [ctypes.c_float] * 5 + [fp]
        L.oracle_awr_evaluate.argtypes = [fp, fp]
        L.oracle_uniform_sample_sphere.argtypes = [ctypes.c_float, ctypes.c_float, fp]
        L.oracle_measure_ray.argtypes = [ctypes.c_float] * 3 + [fp]
        L.oracle_guide_create.restype = vp
        L.oracle_guide_destroy.argtypes = [vp]
        L.oracle_guide_reset.argtypes = [vp]
        L.oracle_guide_step.argtypes = [vp]
        L.oracle_guide_get.restype = ctypes.c_int32
        L.oracle_guide_get.argtypes = [vp, vp, vp, vp, vp]
        L.oracle_guide_set.argtypes = [vp, ctypes.c_int32, vp, vp, vp, vp]
        L.oracle_guide_sample.restype = ctypes.c_float
        L.oracle_guide_sample.argtypes = [vp, ctypes.c_float, ctypes.c_float, fp]
        L.oracle_guided_pass.argtypes = [vp, P(RF), P(FC), P(ANT), P(ANT), P(FLAGS), ctypes.c_int64, ctypes.c_int64,
                                         ctypes.c_float, ctypes.c_int, vp, vp, P(ctypes.c_double)]
        L.oracle_path_tracer_run.argtypes = [vp, P(RF), P(FC), P(ANT), P(ANT), P(FLAGS), ctypes.c_int64, vp, vp,
                                             P(ctypes.c_double)]
        _lib = L
    return _lib


def _p(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None else None


def rf_c(rf):
    return RF(*(np.float32(getattr(rf, n)) for n, _ in RF._fields_))


def fc_c(fc):
    return FC(fc.chirpCount, fc.samplesPerChirp, fc.channelCount)


def ant_c(a):
    c = ANT()
    c.position[:] = [float(x) for x in a.position()]
    c.rotation[:] = [float(x) for x in np.asarray(a.rotation()).reshape(-1)]
    return c


def ffant_c(a):
    """A far-field antenna (direction, complex polarization, scene centre, radius)."""
    c = FFANT()
    c.direction[:] = [float(x) for x in np.asarray(a.direction, np.float32)]
    pol = np.asarray(a.polarization, np.complex64)
    c.polarization[:] = [float(x) for x in np.stack([pol.real, pol.imag], 1).reshape(-1)]
    c.scene_center[:] = [float(x) for x in np.asarray(a.scene_center, np.float32)]
    c.radius = float(np.float32(a.radius))
    return c


def flags_c(tracer):
    f = FLAGS()
    for n, _ in FLAGS._fields_:
        setattr(f, n, getattr(tracer, n))
    return f


class Scene:
    """CPU scene with its own BVH (binned SAH)."""

    def __init__(self, mesh):
        v = np.ascontiguousarray(mesh.vertexBuffer, np.float32)
        i = np.ascontiguousarray(mesh.indexBuffer, np.int32)
        self.h = lib().oracle_scene_create(_p(v), len(v), _p(i), len(i))
        if not self.h:
            raise ValueError("oracle rejected the mesh")

    def __del__(self):
        if getattr(self, "h", None):
            lib().oracle_scene_destroy(self.h)
            self.h = None

    def intersect(self, o, d, tfar=None):
        o = np.ascontiguousarray(o, np.float32).reshape(-1, 3)
        d = np.ascontiguousarray(d, np.float32).reshape(-1, 3)
        n = len(o)
        tf = np.full(n, np.inf, np.float32) if tfar is None else np.ascontiguousarray(tfar, np.float32)
        t = np.zeros(n, np.float32)
        p = np.zeros((n, 3), np.float32)
        nn = np.zeros((n, 3), np.float32)
        prim = np.zeros(n, np.int32)
        lib().oracle_intersect(self.h, n, _p(o), _p(d), _p(tf), _p(t), _p(p), _p(nn), _p(prim))
        return t, p, nn, prim

    def visible(self, o, d, tfar):
        o = np.ascontiguousarray(o, np.float32).reshape(-1, 3)
        d = np.ascontiguousarray(d, np.float32).reshape(-1, 3)
        tf = np.ascontiguousarray(tfar, np.float32).reshape(-1)
        vis = np.zeros(len(o), np.int32)
        lib().oracle_visible(self.h, len(o), _p(o), _p(d), _p(tf), _p(vis))
        return vis

    def simulate(self, rf, fc, tx, rx, tracer, budget, offset=0, sample_weight=1.0, precision=32, threads=0):
        """One plain backend run: returns (raw frame sums [chirp][sample][channel] complex128, total weight)."""
        n = fc.chirpCount * fc.samplesPerChirp * fc.channelCount
        out = np.zeros(2 * n, np.float64)
        w = ctypes.c_double(0.0)
        rc = lib().oracle_simulate(self.h, ctypes.byref(rf_c(rf)), ctypes.byref(fc_c(fc)), ctypes.byref(ant_c(tx)),
                                   ctypes.byref(ant_c(rx)), ctypes.byref(flags_c(tracer)), int(budget), int(offset),
                                   float(sample_weight), int(precision), int(threads), _p(out), ctypes.byref(w))
        if rc != 0:
            raise RuntimeError("oracle_simulate failed (%d)" % rc)
        frame = out.view(np.complex128).reshape(fc.chirpCount, fc.samplesPerChirp, fc.channelCount)
        return frame, w.value

    def fetch_row(self, rf, samples, tx, rx, tracer, budget, precision=32, threads=0, offset=0, exact=False):
        """fetchFrame() row (chirp 0, channel 0) of a plain run: frame / totalWeight.
        exact: the untruncated finite-N Dirichlet synthesis instead of Frame::splat<16>."""
        from hussar_gb300.radar import FrameConfig
        fr, w = self.simulate(rf, FrameConfig(1, samples, 1), tx, rx, tracer, budget, offset=offset,
                              precision=precision | (0x100 if exact else 0), threads=threads)
        return fr[0, :, 0] / w

    def fetch_row_ff(self, rf, samples, tx, rx, tracer, budget, precision=32, threads=0, offset=0):
        """fetchFrame() row of a plain run with far-field TX and RX (FFAntenna)."""
        from hussar_gb300.radar import FrameConfig
        fc = FrameConfig(1, samples, 1)
        out = np.zeros(2 * samples, np.float64)
        w = ctypes.c_double(0.0)
        rc = lib().oracle_simulate_ff(self.h, ctypes.byref(rf_c(rf)), ctypes.byref(fc_c(fc)),
                                      ctypes.byref(ffant_c(tx)), ctypes.byref(ffant_c(rx)),
                                      ctypes.byref(flags_c(tracer)), int(budget), int(offset), 1.0, int(precision),
                                      int(threads), _p(out), ctypes.byref(w))
        if rc != 0:
            raise RuntimeError("oracle_simulate_ff failed (%d)" % rc)
        return out.view(np.complex128) / w.value

    def records(self, rf, fc, tx, rx, tracer, first, count, offset=0, max_records=None):
        mr = max_records or (tracer.maxDepth + 1)
        out = np.zeros((count, mr), RECORD_DTYPE)
        lib().oracle_records(self.h, ctypes.byref(rf_c(rf)), ctypes.byref(fc_c(fc)), ctypes.byref(ant_c(tx)),
                             ctypes.byref(ant_c(rx)), ctypes.byref(flags_c(tracer)), int(first), int(count),
                             int(offset), int(mr), _p(out))
        return out


GUIDE_NODES = 2048


class GuideState:
    """The arrays of a guiding tree (sampling links and first-child probabilities,
    training links and second-moment sums, training node count)."""

    def __init__(self, count=1, samp_child=None, samp_p=None, train_child=None, acc2=None):
        self.count = int(count)
        self.samp_child = np.full(GUIDE_NODES, -1, np.int32) if samp_child is None else \
            np.ascontiguousarray(samp_child, np.int32)
        self.samp_p = np.full(GUIDE_NODES, 0.5, np.float32) if samp_p is None else \
            np.ascontiguousarray(samp_p, np.float32)
        self.train_child = np.full(GUIDE_NODES, -1, np.int32) if train_child is None else \
            np.ascontiguousarray(train_child, np.int32)
        self.acc2 = np.zeros(GUIDE_NODES, np.float32) if acc2 is None else np.ascontiguousarray(acc2, np.float32)

    def reachable(self, which="samp"):
        """Node indices reachable from the root of the sampling or training tree."""
        child = self.samp_child if which == "samp" else self.train_child
        out, todo = [], [0]
        while todo:
            n = todo.pop()
            out.append(n)
            if child[n] >= 0:
                todo += [int(child[n]), int(child[n]) + 1]
        return np.array(sorted(out), np.int64)


class Guide:
    """The oracle's restatement of the guiding tree (GuidingWrapper over the product's
    2-D tree)."""

    def __init__(self):
        self.h = lib().oracle_guide_create()

    def __del__(self):
        if getattr(self, "h", None):
            lib().oracle_guide_destroy(self.h)
            self.h = None

    def reset(self):
        lib().oracle_guide_reset(self.h)

    def step(self):
        lib().oracle_guide_step(self.h)

    def get(self):
        s = GuideState()
        s.count = lib().oracle_guide_get(self.h, _p(s.samp_child), _p(s.samp_p), _p(s.train_child), _p(s.acc2))
        return s

    def set(self, s):
        rc = lib().oracle_guide_set(self.h, int(s.count), _p(s.samp_child), _p(s.samp_p), _p(s.train_child),
                                    _p(s.acc2))
        if rc:
            raise ValueError("oracle_guide_set rejected the state")

    def sample(self, x0, x1):
        y = np.zeros(2, np.float32)
        pdf = lib().oracle_guide_sample(self.h, float(x0), float(x1), y.ctypes.data_as(ctypes.POINTER(ctypes.c_float)))
        return float(y[0]), float(y[1]), float(pdf)

    def run_pass(self, scene, rf, fc, tx, rx, tracer, budget, offset=0, sample_weight=1.0, train=True):
        """One guided iteration (one thread, FP32): (raw frame sums, total weight)."""
        n = fc.chirpCount * fc.samplesPerChirp * fc.channelCount
        out = np.zeros(2 * n, np.float64)
        w = ctypes.c_double(0.0)
        rc = lib().oracle_guided_pass(scene.h, ctypes.byref(rf_c(rf)), ctypes.byref(fc_c(fc)),
                                      ctypes.byref(ant_c(tx)), ctypes.byref(ant_c(rx)), ctypes.byref(flags_c(tracer)),
                                      int(budget), int(offset), float(sample_weight), 1 if train else 0, self.h,
                                      _p(out), ctypes.byref(w))
        if rc:
            raise RuntimeError("oracle_guided_pass failed (%d)" % rc)
        return out.view(np.complex128).reshape(fc.chirpCount, fc.samplesPerChirp, fc.channelCount), w.value

    def path_tracer_run(self, scene, rf, fc, tx, rx, tracer, samples):
        """PathTracer::run's guided schedule: (raw frame sums, total weight); the tree
        ends in its state after the last step."""
        n = fc.chirpCount * fc.samplesPerChirp * fc.channelCount
        out = np.zeros(2 * n, np.float64)
        w = ctypes.c_double(0.0)
        rc = lib().oracle_path_tracer_run(scene.h, ctypes.byref(rf_c(rf)), ctypes.byref(fc_c(fc)),
                                          ctypes.byref(ant_c(tx)), ctypes.byref(ant_c(rx)),
                                          ctypes.byref(flags_c(tracer)), int(samples), self.h, _p(out),
                                          ctypes.byref(w))
        if rc:
            raise RuntimeError("oracle_path_tracer_run failed (%d)" % rc)
        return out.view(np.complex128).reshape(fc.chirpCount, fc.samplesPerChirp, fc.channelCount), w.value


def radical_inverse(index, dim, precision=32):
    L = lib()
    return L.oracle_radical_inverse_f(int(index), int(dim)) if precision == 32 else \
        L.oracle_radical_inverse_d(int(index), int(dim))


def frame_splat(chirps, samples, channels, ic, isample, ich, re, im):
    out = np.zeros(2 * chirps * samples * channels, np.float32)
    lib().oracle_frame_splat(chirps, samples, channels, ic, isample, ich, re, im,
                             out.ctypes.data_as(ctypes.POINTER(ctypes.c_float)))
    return out
