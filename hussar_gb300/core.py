"""libhussar's scene / sensor / integrator API, backed by the GB300 C ABI.

Names, arguments and defaults mirror the reference so that programs written against
libhussar read the same:

    TriangleMesh            libhussar/include/hussar/core/mesh.h:14-55
    AWRAngularDistribution  libhussar/include/hussar/core/emitter.h:109-137
    NFAntenna               libhussar/include/hussar/core/emitter.h:159-214
    Scene                   libhussar/include/hussar/core/scene.h:9-14
    PathTracer              libhussar/include/hussar/integrators/path.h:133-476
    gb300.Backend           replaces cpu::Backend (arch/cpu.h:17-63) / gpu::Backend (arch/gpu.h:17-47)
"""
import ctypes

import numpy as np

from . import _lib
from .radar import Frame, FrameConfig, RFConfig


class TriangleMesh:
    """hussar::TriangleMesh: float3 vertexBuffer and int3 indexBuffer (mesh.h:14-55)."""

    def __init__(self, vertices=None, indices=None):
        self._v = [] if vertices is None else [np.asarray(vertices, np.float32).reshape(-1, 3)]
        self._i = [] if indices is None else [np.asarray(indices, np.int32).reshape(-1, 3)]
        self._nv = 0 if vertices is None else len(self._v[0])

    @property
    def vertexBuffer(self):
        return np.concatenate(self._v, 0) if self._v else np.zeros((0, 3), np.float32)

    @property
    def indexBuffer(self):
        return np.concatenate(self._i, 0) if self._i else np.zeros((0, 3), np.int32)

    def addQuad(self, a, b, c):
        """mesh.h:30-40: vertices a, a+b, a+b+c, a+c; triangles (0,1,2), (0,2,3)."""
        a = np.asarray(a, np.float32)
        b = np.asarray(b, np.float32)
        c = np.asarray(c, np.float32)
        ab = a + b
        v = np.stack([a, ab, ab + c, a + c]).astype(np.float32)
        i = self._nv
        self._v.append(v)
        self._i.append(np.array([[i, i + 1, i + 2], [i, i + 2, i + 3]], np.int32))
        self._nv += 4

    def addBox(self, mn, mx):
        """mesh.h:42-54: six quads, 12 triangles."""
        mn = np.asarray(mn, np.float32)
        mx = np.asarray(mx, np.float32)
        d = mx - mn
        z = np.float32(0)
        self.addQuad(mn, [z, d[1], z], [z, z, d[2]])
        self.addQuad(mn, [z, z, d[2]], [d[0], z, z])
        self.addQuad(mn, [d[0], z, z], [z, d[1], z])
        d = mn - mx
        self.addQuad(mx, [z, d[1], z], [d[0], z, z])
        self.addQuad(mx, [z, z, d[2]], [z, d[1], z])
        self.addQuad(mx, [d[0], z, z], [z, z, d[2]])

    def append(self, vertices, indices):
        """Bulk append (indices relative to the appended vertices)."""
        v = np.asarray(vertices, np.float32).reshape(-1, 3)
        i = np.asarray(indices, np.int32).reshape(-1, 3) + self._nv
        self._v.append(v)
        self._i.append(i.astype(np.int32))
        self._nv += len(v)

    def triangleCount(self):
        return sum(len(x) for x in self._i)


class AWRAngularDistribution:
    """The AWR1243 antenna pattern (emitter.h:109-137); evaluated on the device."""


class NFAntenna:
    """hussar::NFAntenna (emitter.h:159-214): a point antenna at `position` whose local
    frame is `rotation` (3x3; third column = boresight)."""

    def __init__(self, position=(0, 0, 0), rotation=np.eye(3), radiation=None):
        self._position = np.asarray(position, np.float32).reshape(3)
        self._rotation = np.asarray(rotation, np.float32).reshape(3, 3)
        self.radiation = radiation if radiation is not None else AWRAngularDistribution()
        det = np.linalg.det(self._rotation.astype(np.float64))
        if abs(abs(det) - 1) >= 1e-2:  # emitter.h:166-169
            raise ValueError("supplied rotation matrix is - in fact - not a rotation matrix!")

    def position(self):
        return self._position

    def rotation(self):
        return self._rotation

    def to_c(self):
        a = _lib.AntennaC()
        a.position[:] = [float(x) for x in self._position]
        a.rotation[:] = [float(x) for x in self._rotation.reshape(-1)]
        return a


class FFAntenna:
    """hussar::FFAntenna (emitter.h:218-291): a far-field antenna (plane wave), a disk of
    `radius` at sceneCenter + dir * radius facing the scene. Rays leave it along -dir;
    it is reached along +dir. `polarization` is the complex H field (3 components),
    orthogonal to `dir`; `dir` is normalised (the reference asserts both)."""

    def __init__(self, dir, polarization, sceneCenter, radius):
        self.direction = np.asarray(dir, np.float32).reshape(3)
        self.polarization = np.asarray(polarization, np.complex64).reshape(3)
        self.scene_center = np.asarray(sceneCenter, np.float32).reshape(3)
        self.radius = np.float32(radius)
        if abs(float(np.linalg.norm(self.direction.astype(np.float64))) - 1.0) > 1e-3:
            raise ValueError("normal of plane wave must be normalized")
        if abs(complex(np.dot(self.direction.astype(np.complex128), self.polarization.astype(np.complex128)))) > 1e-3:
            raise ValueError("H-field must be orthogonal to direction of propagation")
        if not self.radius > 0:
            raise ValueError("radius must be positive")

    def to_c(self):
        a = _lib.FfAntennaC()
        a.direction[:] = [float(x) for x in self.direction]
        a.polarization[:] = [float(x) for x in np.stack([self.polarization.real, self.polarization.imag], 1).reshape(-1)]
        a.scene_center[:] = [float(x) for x in self.scene_center]
        a.radius = float(self.radius)
        return a


class Scene:
    """hussar::Scene (scene.h:9-14): RF configuration plus the RX and TX antennas."""

    def __init__(self, rfConfig=None, tx=None, rx=None):
        self.rfConfig = rfConfig if rfConfig is not None else RFConfig()
        self.tx = tx if tx is not None else NFAntenna()
        self.rx = rx if rx is not None else NFAntenna()


_FLAG_FIELDS = ("onlyIndirect", "maxDepth", "useGeometricalOptics", "poDiffraction", "doGuiding",
                "clearBeforeIteration", "correctPhase", "filterGuiding", "doFiltering", "filteringSphere",
                "produceDebugImage", "filteringMin", "filteringMax", "filteringRadius")


class PathTracer:
    """hussar::PathTracer (path.h:133-476): the plain radar path tracer's configuration,
    frame and run schedule. The per-sample work runs on the GB300 behind the backend."""

    def __init__(self):
        # path.h:153-169 defaults
        self.onlyIndirect = True
        self.maxDepth = 10
        self.useGeometricalOptics = True
        self.poDiffraction = False
        self.doGuiding = True
        self.clearBeforeIteration = True
        self.correctPhase = False
        self.filterGuiding = True
        self.doFiltering = True
        self.filteringSphere = True
        self.filteringMin = 600.0
        self.filteringMax = 900.0
        self.filteringRadius = 160.0
        self.produceDebugImage = False  # core/integrator.h:58
        self.phaseMode = _lib.HSR_PHASE_REFERENCE_FP32
        self.frame = Frame()
        self.totalWeight = 0.0
        self.sampleIndexOffset = 0
        self.currentSampleWeight = 1.0

    def flags_c(self):
        f = _lib.FlagsC()
        for name in _FLAG_FIELDS:
            setattr(f, name, getattr(self, name))
        return f

    def configureFrame(self, config):
        """Integrator::configureFrame (integrator.h:60-62)."""
        self.frame.configure(config)

    def clearFrame(self):
        """path.h:147-150."""
        self.frame.clear()
        self.totalWeight = 0.0

    def run(self, backend, scene, samples, interruptFlag=None):
        """PathTracer::run (path.h:171-224). The plain schedule traces Halton indices
        [0, samples) in one backend.run call; the guided schedule (doGuiding) runs the
        doubling iterations with device path guiding inside the backend."""
        self.clearFrame()
        self.sampleIndexOffset = 0
        self.currentSampleWeight = 1.0
        if not self.doGuiding:
            backend.run(scene, samples, interruptFlag)
            return
        backend.run_path_tracer(scene, samples, interruptFlag)

    def fetchFrame(self):
        """path.h:453-455: frame / totalWeight."""
        return self.frame / np.float32(self.totalWeight)


# struct DNode (hussar_gb300/csrc/hsr_common.cuh): both child boxes of a binary node
DNODE_DTYPE = np.dtype([("a", "<f4", 4), ("b", "<f4", 4), ("c", "<f4", 4), ("child", "<i4", 2), ("unused", "<i4", 2)])


def child_boxes(nodes):
    """(lo, hi) of both children of every node, shape [nodes, 2, 3]."""
    lo = np.stack([np.stack([nodes["a"][:, 0], nodes["a"][:, 2], nodes["c"][:, 0]], 1),
                   np.stack([nodes["b"][:, 0], nodes["b"][:, 2], nodes["c"][:, 2]], 1)], 1)
    hi = np.stack([np.stack([nodes["a"][:, 1], nodes["a"][:, 3], nodes["c"][:, 1]], 1),
                   np.stack([nodes["b"][:, 1], nodes["b"][:, 3], nodes["c"][:, 3]], 1)], 1)
    return lo, hi


class BatchGraph:
    """A captured plain batch (hsr_batch_graph_*); keeps its backend alive."""

    def __init__(self, handle, backend):
        self._h = handle
        self._backend = backend

    def launch(self, stream=None):
        _lib.check(_lib.lib().hsr_batch_graph_launch(self._h, ctypes.c_void_p(stream)))

    def status(self):
        _lib.check(_lib.lib().hsr_batch_graph_status(self._h))

    def close(self):
        if self._h is not None and self._h.value:
            _lib.lib().hsr_batch_graph_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class _GB300:
    """Namespace mirroring hussar::gb300 (the drop-in for hussar::cpu / hussar::gpu)."""

    class Backend:
        """Backend(mesh, integrator) + run(scene, budget, interruptFlag): the backend
        concept of arch/cpu.h:17-63 and arch/gpu.h:17-47. The mesh is copied to the
        device and its BVH built here; the integrator is held by reference."""

        def __init__(self, mesh, integrator):
            L = _lib.lib()
            v = np.ascontiguousarray(mesh.vertexBuffer, np.float32)
            i = np.ascontiguousarray(mesh.indexBuffer, np.int32)
            h = ctypes.c_void_p()
            _lib.check(L.hsr_scene_create(_lib.ptr(v), len(v), _lib.ptr(i), len(i), ctypes.byref(h)))
            self._scene = h
            self._integrator = integrator

        def __del__(self):
            h = getattr(self, "_scene", None)
            if h is not None and h.value:
                try:
                    _lib.lib().hsr_scene_destroy(h)
                except Exception:
                    pass
                self._scene = None

        @property
        def handle(self):
            return self._scene

        def run(self, scene, budget, interruptFlag=None):
            """Adds samples sampleIndexOffset + [0, budget) into the integrator's frame."""
            it = self._integrator
            L = _lib.lib()
            fc = it.frame.config()
            buf = np.ascontiguousarray(it.frame.data.view(np.float32).reshape(-1))
            tw = ctypes.c_double(it.totalWeight)
            flag = None
            if interruptFlag is not None:
                flag = np.array([1 if interruptFlag() else 0], np.int32) if callable(interruptFlag) else \
                    np.array([1 if interruptFlag else 0], np.int32)
            _lib.check(L.hsr_backend_run(self._scene, ctypes.byref(scene.rfConfig.to_c()), ctypes.byref(fc.to_c()),
                                         ctypes.byref(scene.tx.to_c()), ctypes.byref(scene.rx.to_c()),
                                         ctypes.byref(it.flags_c()), int(budget), int(it.sampleIndexOffset),
                                         float(it.currentSampleWeight), int(it.phaseMode), _lib.ptr(buf),
                                         ctypes.byref(tw), _lib.ptr(flag)))
            it.frame.data = buf.view(np.complex64).reshape(it.frame.data.shape)
            it.totalWeight = tw.value

        def run_path_tracer(self, scene, samples, interruptFlag=None):
            """The whole PathTracer::run schedule on the device (hsr_path_tracer_run):
            sets the integrator's frame and total weight."""
            it = self._integrator
            fc = it.frame.config()
            buf = np.zeros(2 * fc.sampleCount(), np.float32)
            tw = ctypes.c_double(0.0)
            flag = None
            if interruptFlag is not None:
                flag = np.array([1 if (interruptFlag() if callable(interruptFlag) else interruptFlag) else 0],
                                np.int32)
            _lib.check(_lib.lib().hsr_path_tracer_run(
                self._scene, ctypes.byref(scene.rfConfig.to_c()), ctypes.byref(fc.to_c()),
                ctypes.byref(scene.tx.to_c()), ctypes.byref(scene.rx.to_c()), ctypes.byref(it.flags_c()),
                int(samples), int(it.phaseMode), _lib.ptr(buf), ctypes.byref(tw), _lib.ptr(flag)))
            it.frame.data = buf.view(np.complex64).reshape(it.frame.data.shape)
            it.totalWeight = tw.value

        def refit(self, mesh):
            """New vertex positions of the same mesh (hsr_scene_refit): the BVH keeps its
            tree and refits its boxes."""
            v = np.ascontiguousarray(mesh.vertexBuffer, np.float32)
            _lib.check(_lib.lib().hsr_scene_refit(self._scene, _lib.ptr(v), len(v)))

        def rebuild(self, mesh):
            """A new mesh under this backend's scene handle (hsr_scene_rebuild)."""
            v = np.ascontiguousarray(mesh.vertexBuffer, np.float32)
            i = np.ascontiguousarray(mesh.indexBuffer, np.int32)
            _lib.check(_lib.lib().hsr_scene_rebuild(self._scene, _lib.ptr(v), len(v), _lib.ptr(i), len(i)))

        def footprint(self):
            out = ctypes.c_int64()
            _lib.check(_lib.lib().hsr_scene_footprint(self._scene, ctypes.byref(out)))
            return out.value

        def bvh_stats(self):
            n = ctypes.c_int64()
            d = ctypes.c_int32()
            lv = ctypes.c_int64()
            _lib.check(_lib.lib().hsr_scene_bvh_stats(self._scene, ctypes.byref(n), ctypes.byref(d),
                                                       ctypes.byref(lv)))
            return {"nodes": n.value, "max_depth": d.value, "leaves": lv.value}

        def device_bvh(self):
            """The device BVH (tests): (nodes, tris), nodes a DNODE_DTYPE array (root 0),
            tris [triangles, 12] float32 records in slot order."""
            st = self.bvh_stats()
            nodes = np.zeros(st["nodes"], dtype=DNODE_DTYPE)
            tris = np.zeros((st["leaves"], 12), np.float32)
            _lib.check(_lib.lib().hsr_debug_bvh(self._scene, _lib.ptr(nodes), len(nodes), _lib.ptr(tris), len(tris)))
            return nodes, tris

        def intersect(self, origins, directions, tfar=None):
            """Closest-hit queries (RT::intersect): returns t, p, n, prim."""
            o = np.ascontiguousarray(origins, np.float32).reshape(-1, 3)
            d = np.ascontiguousarray(directions, np.float32).reshape(-1, 3)
            n = len(o)
            tf = np.full(n, np.inf, np.float32) if tfar is None else np.ascontiguousarray(tfar, np.float32)
            t = np.zeros(n, np.float32)
            p = np.zeros((n, 3), np.float32)
            nn = np.zeros((n, 3), np.float32)
            prim = np.zeros(n, np.int32)
            _lib.check(_lib.lib().hsr_intersect(self._scene, n, _lib.ptr(o), _lib.ptr(d), _lib.ptr(tf),
                                                 _lib.ptr(t), _lib.ptr(p), _lib.ptr(nn), _lib.ptr(prim)))
            return t, p, nn, prim

        def visible(self, origins, directions, tfar):
            """Occlusion queries (RT::visible): 1 where nothing lies in (5e-5, tfar]."""
            o = np.ascontiguousarray(origins, np.float32).reshape(-1, 3)
            d = np.ascontiguousarray(directions, np.float32).reshape(-1, 3)
            tf = np.ascontiguousarray(tfar, np.float32).reshape(-1)
            vis = np.zeros(len(o), np.int32)
            _lib.check(_lib.lib().hsr_visible(self._scene, len(o), _lib.ptr(o), _lib.ptr(d), _lib.ptr(tf),
                                               _lib.ptr(vis)))
            return vis

        def simulate_batch(self, rf, samples_per_chirp, integrator, tx, rx, budget, index_offset=None,
                           phase_mode=_lib.HSR_PHASE_REFERENCE_FP32, splat_mode=_lib.HSR_SPLAT_DIRICHLET16,
                           stream=None):
            """Many poses in one persistent launch (host arrays in and out).
            tx, rx: sequences of NFAntenna; budget: int per pose. Returns complex64
            rows (poses x samples_per_chirp): each pose's fetchFrame() row."""
            P = len(tx)
            txa = (_lib.AntennaC * P)(*[a.to_c() for a in tx])
            rxa = (_lib.AntennaC * P)(*[a.to_c() for a in rx])
            b = np.ascontiguousarray(budget, np.int64)
            off = np.zeros(P, np.int64) if index_offset is None else np.ascontiguousarray(index_offset, np.int64)
            out = np.zeros((P, samples_per_chirp), np.complex64)
            _lib.check(_lib.lib().hsr_simulate_batch(
                self._scene, ctypes.byref(rf.to_c()), int(samples_per_chirp), ctypes.byref(integrator.flags_c()),
                P, ctypes.cast(txa, ctypes.c_void_p), ctypes.cast(rxa, ctypes.c_void_p), _lib.ptr(b), _lib.ptr(off),
                int(phase_mode), int(splat_mode), _lib.ptr(out), ctypes.c_void_p(stream)))
            return out

        def simulate_frame(self, rf, frame_config, integrator, tx_array, rx_array, budget, index_offset=0,
                           phase_mode=_lib.HSR_PHASE_REFERENCE_FP32, splat_mode=_lib.HSR_SPLAT_DIRICHLET16,
                           stream=None):
            """hsr_simulate_frame: a MIMO radar cube [chirp][sample][channel] (complex64) of
            len(tx_array) x len(rx_array) virtual channels (channel c = TX c // n_rx, RX
            c % n_rx), each a run of `budget` samples, traced as one batch."""
            T, R = len(tx_array), len(rx_array)
            txa = (_lib.AntennaC * T)(*[a.to_c() for a in tx_array])
            rxa = (_lib.AntennaC * R)(*[a.to_c() for a in rx_array])
            fc = frame_config.to_c()
            out = np.zeros((fc.chirpCount, fc.samplesPerChirp, fc.channelCount), np.complex64)
            _lib.check(_lib.lib().hsr_simulate_frame(
                self._scene, ctypes.byref(rf.to_c()), ctypes.byref(fc), ctypes.byref(integrator.flags_c()), T,
                ctypes.cast(txa, ctypes.c_void_p), R, ctypes.cast(rxa, ctypes.c_void_p), int(budget), int(index_offset),
                int(phase_mode), int(splat_mode), _lib.ptr(out), ctypes.c_void_p(stream)))
            return out

        def simulate_batch_ff(self, rf, samples_per_chirp, integrator, tx, rx, budget, index_offset=None,
                              phase_mode=_lib.HSR_PHASE_REFERENCE_FP32):
            """Far-field runs (hsr_simulate_batch_ff): tx, rx sequences of FFAntenna, one
            per pose; returns each pose's fetchFrame() row (complex64)."""
            P = len(tx)
            txa = (_lib.FfAntennaC * P)(*[a.to_c() for a in tx])
            rxa = (_lib.FfAntennaC * P)(*[a.to_c() for a in rx])
            b = np.ascontiguousarray(budget, np.int64)
            off = np.zeros(P, np.int64) if index_offset is None else np.ascontiguousarray(index_offset, np.int64)
            out = np.zeros((P, samples_per_chirp), np.complex64)
            _lib.check(_lib.lib().hsr_simulate_batch_ff(
                self._scene, ctypes.byref(rf.to_c()), int(samples_per_chirp), ctypes.byref(integrator.flags_c()),
                P, ctypes.cast(txa, ctypes.c_void_p), ctypes.cast(rxa, ctypes.c_void_p), _lib.ptr(b), _lib.ptr(off),
                int(phase_mode), _lib.ptr(out)))
            return out

        def batch_graph(self, rf, samples_per_chirp, integrator, pose_count, d_tx, d_rx, d_budget, d_offset,
                        d_out_rows, phase_mode=_lib.HSR_PHASE_REFERENCE_FP32, splat_mode=_lib.HSR_SPLAT_DIRICHLET16):
            """The plain batch over device buffers (addresses as integers) captured into a
            CUDA graph (hsr_batch_graph_create); BatchGraph.launch(stream) replays it."""
            h = ctypes.c_void_p()
            vp = ctypes.c_void_p
            _lib.check(_lib.lib().hsr_batch_graph_create(
                self._scene, ctypes.byref(rf.to_c()), int(samples_per_chirp), ctypes.byref(integrator.flags_c()),
                int(pose_count), vp(d_tx), vp(d_rx), vp(d_budget), vp(d_offset), int(phase_mode), int(splat_mode),
                vp(d_out_rows), ctypes.byref(h)))
            return BatchGraph(h, self)

        def autotune(self, rf, samples_per_chirp, integrator, tx, rx, budget, index_offset=None,
                     phase_mode=_lib.HSR_PHASE_REFERENCE_FP32, splat_mode=_lib.HSR_SPLAT_DIRICHLET16):
            """hsr_autotune_batch: times this batch under candidate launch shapes, keeps the
            fastest for later plain runs on this scene and returns it as a dict."""
            P = len(tx)
            txa = (_lib.AntennaC * P)(*[a.to_c() for a in tx])
            rxa = (_lib.AntennaC * P)(*[a.to_c() for a in rx])
            b = np.ascontiguousarray(budget, np.int64)
            off = np.zeros(P, np.int64) if index_offset is None else np.ascontiguousarray(index_offset, np.int64)
            out = _lib.LaunchConfigC()
            _lib.check(_lib.lib().hsr_autotune_batch(
                self._scene, ctypes.byref(rf.to_c()), int(samples_per_chirp), ctypes.byref(integrator.flags_c()), P,
                ctypes.cast(txa, ctypes.c_void_p), ctypes.cast(rxa, ctypes.c_void_p), _lib.ptr(b), _lib.ptr(off),
                int(phase_mode), int(splat_mode), ctypes.byref(out)))
            return {name: getattr(out, name) for name, _ in _lib.LaunchConfigC._fields_}

        def set_launch_config(self, tile=0, ctas_per_sm=0, queue_threshold=0, field_on_hit=0, coherent_order=0,
                              default=False):
            """Sets the scene's launch shape (default=True: back to the default shape)."""
            c = _lib.LaunchConfigC(int(tile), int(ctas_per_sm), int(queue_threshold), 0.0, 0.0, int(field_on_hit),
                                   int(coherent_order))
            _lib.check(_lib.lib().hsr_set_launch_config(self._scene, None if default else ctypes.byref(c)))

        def traversal_counts(self, rf, samples_per_chirp, integrator, tx, rx, budget, index_offset=None):
            """Exact traversal work of one batch launch (counting instantiation):
            dict(nodes, tris, rays, bytes) with 64 B per BVH node and 48 B per triangle."""
            P = len(tx)
            txa = (_lib.AntennaC * P)(*[a.to_c() for a in tx])
            rxa = (_lib.AntennaC * P)(*[a.to_c() for a in rx])
            b = np.ascontiguousarray(budget, np.int64)
            off = np.zeros(P, np.int64) if index_offset is None else np.ascontiguousarray(index_offset, np.int64)
            out = np.zeros(3, np.int64)
            _lib.check(_lib.lib().hsr_debug_traversal_counts(
                self._scene, ctypes.byref(rf.to_c()), int(samples_per_chirp), ctypes.byref(integrator.flags_c()), P,
                ctypes.cast(txa, ctypes.c_void_p), ctypes.cast(rxa, ctypes.c_void_p), _lib.ptr(b), _lib.ptr(off),
                _lib.ptr(out)))
            nodes, tris, rays = (int(x) for x in out)
            return {"nodes": nodes, "tris": tris, "rays": rays, "bytes": 64 * nodes + 48 * tris}

        def debug_records(self, scene, integrator, samples_per_chirp, budget, index_offset=0, max_records=None):
            """Per-sample next-event records (tests): structured array [budget, max_records]."""
            mr = max_records or (integrator.maxDepth + 1)
            rec = np.zeros((budget, mr), dtype=_lib.RECORD_DTYPE)
            _lib.check(_lib.lib().hsr_debug_records(
                self._scene, ctypes.byref(scene.rfConfig.to_c()), int(samples_per_chirp),
                ctypes.byref(integrator.flags_c()), ctypes.byref(scene.tx.to_c()), ctypes.byref(scene.rx.to_c()),
                int(budget), int(index_offset), int(mr), _lib.ptr(rec)))
            return rec

        def last_kernel_ms(self):
            out = ctypes.c_float()
            _lib.check(_lib.lib().hsr_last_kernel_ms(self._scene, ctypes.byref(out)))
            return out.value

    class Guide:
        """A device guiding tree on a backend's scene (hsr_guide_*): GuidingWrapper's
        reset/step (path.h:47-50, 119-126) plus one guided iteration of PathTracer::run
        (hsr_backend_run_guided) into an integrator's frame."""

        MAX_NODES = 2048

        def __init__(self, backend):
            h = ctypes.c_void_p()
            _lib.check(_lib.lib().hsr_guide_create(backend.handle, ctypes.byref(h)))
            self._h = h
            self._backend = backend

        def close(self):
            if self._h is not None and self._h.value:
                _lib.lib().hsr_guide_destroy(self._h)
                self._h = None

        def __del__(self):
            try:
                self.close()
            except Exception:
                pass

        def reset(self):
            _lib.check(_lib.lib().hsr_guide_reset(self._h))

        def step(self):
            _lib.check(_lib.lib().hsr_guide_step(self._h))

        def read(self):
            """(count, samp_child, samp_p, train_child, train_acc2) as host arrays."""
            n = self.MAX_NODES
            sc, sp = np.zeros(n, np.int32), np.zeros(n, np.float32)
            tc, acc = np.zeros(n, np.int32), np.zeros(n, np.float32)
            cnt = ctypes.c_int32()
            _lib.check(_lib.lib().hsr_guide_read(self._h, ctypes.byref(cnt), _lib.ptr(sc), _lib.ptr(sp),
                                                 _lib.ptr(tc), _lib.ptr(acc)))
            return cnt.value, sc, sp, tc, acc

        def write(self, count, samp_child, samp_p, train_child, train_acc2):
            arr = [np.ascontiguousarray(samp_child, np.int32), np.ascontiguousarray(samp_p, np.float32),
                   np.ascontiguousarray(train_child, np.int32), np.ascontiguousarray(train_acc2, np.float32)]
            if any(len(a) != self.MAX_NODES for a in arr):
                raise ValueError("guide arrays hold %d entries" % self.MAX_NODES)
            _lib.check(_lib.lib().hsr_guide_write(self._h, int(count), *(_lib.ptr(a) for a in arr)))

        def run_iteration(self, integrator, scene, budget, train):
            """One guided backend run: samples integrator.sampleIndexOffset + [0, budget)
            with the integrator's sample weight, added into its frame and total weight."""
            it = integrator
            fc = it.frame.config()
            buf = np.ascontiguousarray(it.frame.data.view(np.float32).reshape(-1))
            tw = ctypes.c_double(it.totalWeight)
            _lib.check(_lib.lib().hsr_backend_run_guided(
                self._backend.handle, ctypes.byref(scene.rfConfig.to_c()), ctypes.byref(fc.to_c()),
                ctypes.byref(scene.tx.to_c()), ctypes.byref(scene.rx.to_c()), ctypes.byref(it.flags_c()),
                int(budget), int(it.sampleIndexOffset), float(it.currentSampleWeight), 1 if train else 0, self._h,
                int(it.phaseMode), _lib.ptr(buf), ctypes.byref(tw), None))
            it.frame.data = buf.view(np.complex64).reshape(it.frame.data.shape)
            it.totalWeight = tw.value


gb300 = _GB300()
