"""ctypes binding of the C ABI in include/hsr_gb300.h (libhsr_gb300.so).

The library is loaded from this package directory only. If it is missing, every call
fails loudly: there is no CPU fallback anywhere in the product.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libhsr_gb300.so")

HSR_OK = 0
HSR_ERR_INVALID_ARGUMENT = 1
HSR_ERR_CUDA = 2
HSR_ERR_OUT_OF_MEMORY = 3
HSR_ERR_INTERRUPTED = 4
HSR_ERR_DEVICE = 5
HSR_ERR_NOT_SUPPORTED = 6
HSR_ERR_NO_DEVICE = 7
HSR_ERR_TIMEOUT = 8

HSR_PHASE_REFERENCE_FP32 = 0
HSR_PHASE_SPLIT_FP64 = 1
HSR_SPLAT_DIRICHLET16 = 0
HSR_SPLAT_FINE_SYNTH = 1

STATUS_NAMES = {
    0: "HSR_OK", 1: "HSR_ERR_INVALID_ARGUMENT", 2: "HSR_ERR_CUDA", 3: "HSR_ERR_OUT_OF_MEMORY",
    4: "HSR_ERR_INTERRUPTED", 5: "HSR_ERR_DEVICE", 6: "HSR_ERR_NOT_SUPPORTED", 7: "HSR_ERR_NO_DEVICE",
    8: "HSR_ERR_TIMEOUT",
}


class HsrError(RuntimeError):
    """A non-OK hsr_status; .status holds the code."""

    def __init__(self, status, message):
        super().__init__("%s: %s" % (STATUS_NAMES.get(status, status), message))
        self.status = status


class InterruptedError_(HsrError):
    pass


class RFConfigC(ctypes.Structure):
    _fields_ = [(n, ctypes.c_float) for n in
                ("startFreq", "freqSlope", "adcRate", "idleTime", "rampTime", "antennaDelay")]


class FrameConfigC(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int32) for n in ("chirpCount", "samplesPerChirp", "channelCount")]


class AntennaC(ctypes.Structure):
    _fields_ = [("position", ctypes.c_float * 3), ("rotation", ctypes.c_float * 9)]


class FfAntennaC(ctypes.Structure):
    _fields_ = [("direction", ctypes.c_float * 3), ("polarization", ctypes.c_float * 6),
                ("scene_center", ctypes.c_float * 3), ("radius", ctypes.c_float)]


class FlagsC(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int32) for n in
                ("onlyIndirect", "maxDepth", "useGeometricalOptics", "poDiffraction", "doGuiding",
                 "clearBeforeIteration", "correctPhase", "filterGuiding", "doFiltering", "filteringSphere",
                 "produceDebugImage")] + \
              [(n, ctypes.c_float) for n in ("filteringMin", "filteringMax", "filteringRadius")]


class ServerConfigC(ctypes.Structure):
    _fields_ = [("max_slots", ctypes.c_int32), ("max_samples_per_chirp", ctypes.c_int32),
                ("memory_bytes", ctypes.c_int64), ("tick_ms", ctypes.c_float), ("phase_mode", ctypes.c_int32),
                ("flags", FlagsC)]


class RequestC(ctypes.Structure):
    _fields_ = [("scene", ctypes.c_int32), ("samples_per_chirp", ctypes.c_int32), ("rf", RFConfigC),
                ("tx", AntennaC), ("rx", AntennaC), ("budget", ctypes.c_int64), ("index_offset", ctypes.c_int64),
                ("out_row", ctypes.c_void_p)]


class RequestResultC(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int32), ("ticks", ctypes.c_int32), ("queue_ms", ctypes.c_double),
                ("latency_ms", ctypes.c_double)]


class ServerStatsC(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int64) for n in ("submitted", "completed", "failed", "ticks", "samples")] + \
               [(n, ctypes.c_double) for n in ("device_ms", "p50_ms", "p99_ms", "max_ms")] + \
               [("max_batch", ctypes.c_int32), ("max_resident", ctypes.c_int32)] + \
               [(n, ctypes.c_int64) for n in ("admitted_while_busy", "memory_bytes_peak", "scene_bytes")]


class LaunchConfigC(ctypes.Structure):
    _fields_ = [("tile", ctypes.c_int32), ("ctas_per_sm", ctypes.c_int32), ("queue_threshold", ctypes.c_int32),
                ("trace_ms", ctypes.c_float), ("default_trace_ms", ctypes.c_float), ("field_on_hit", ctypes.c_int32),
                ("coherent_order", ctypes.c_int32)]


# PathRecord in hsr_trace.cu / hsr_debug_records
RECORD_DTYPE = [("depth", "<i4"), ("splatted", "<i4"), ("time", "<f4"), ("v_re", "<f4"), ("v_im", "<f4"),
                ("dphase", "<f4"), ("bin", "<f4"), ("value_re", "<f4"), ("value_im", "<f4")]

_lib = None
ABI_VERSION = 5  # HSR_ABI_VERSION of include/hsr_gb300.h that these ctypes mirrors follow


def lib():
    """Loads libhsr_gb300.so (once). Raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError("libhsr_gb300.so is not built (run hussar_gb300.build.build()); "
                           "this backend has no CPU fallback")
    L = ctypes.CDLL(LIB_PATH)
    P = ctypes.POINTER
    vp = ctypes.c_void_p
    L.hsr_abi_version.restype = ctypes.c_int32
    if L.hsr_abi_version() != ABI_VERSION:  # a stale build: the struct mirrors would not match
        raise RuntimeError("libhsr_gb300.so has ABI %d, this package expects %d: rebuild it"
                           % (L.hsr_abi_version(), ABI_VERSION))
    L.hsr_last_error.restype = ctypes.c_char_p
    L.hsr_launch_count.restype = ctypes.c_int64
    L.hsr_debug_alloc_count.restype = ctypes.c_int64
    L.hsr_default_flags.argtypes = [P(FlagsC)]
    L.hsr_default_flags.restype = None
    L.hsr_default_server_config.argtypes = [P(ServerConfigC)]
    L.hsr_default_server_config.restype = None
    sigs = {
        "hsr_scene_create": [vp, ctypes.c_int64, vp, ctypes.c_int64, P(vp)],
        "hsr_scene_destroy": [vp],
        "hsr_scene_footprint": [vp, P(ctypes.c_int64)],
        "hsr_scene_bvh_stats": [vp, P(ctypes.c_int64), P(ctypes.c_int32), P(ctypes.c_int64)],
        "hsr_intersect": [vp, ctypes.c_int64, vp, vp, vp, vp, vp, vp, vp],
        "hsr_visible": [vp, ctypes.c_int64, vp, vp, vp, vp],
        "hsr_backend_run": [vp, P(RFConfigC), P(FrameConfigC), P(AntennaC), P(AntennaC), P(FlagsC),
                            ctypes.c_int64, ctypes.c_int64, ctypes.c_float, ctypes.c_int32, vp,
                            P(ctypes.c_double), vp],
        "hsr_path_tracer_run": [vp, P(RFConfigC), P(FrameConfigC), P(AntennaC), P(AntennaC), P(FlagsC),
                                ctypes.c_int64, ctypes.c_int32, vp, P(ctypes.c_double), vp],
        "hsr_simulate_batch_device": [vp, P(RFConfigC), ctypes.c_int32, P(FlagsC), ctypes.c_int32, vp, vp, vp,
                                      vp, ctypes.c_int32, ctypes.c_int32, vp, vp],
        "hsr_simulate_batch": [vp, P(RFConfigC), ctypes.c_int32, P(FlagsC), ctypes.c_int32, vp, vp, vp, vp,
                               ctypes.c_int32, ctypes.c_int32, vp, vp],
        "hsr_simulate_batch_device_noalloc": [vp, P(RFConfigC), ctypes.c_int32, P(FlagsC), ctypes.c_int32, vp, vp,
                                              vp, vp, ctypes.c_int32, vp, vp],
        "hsr_scene_status": [vp, vp, P(ctypes.c_uint32)],
        "hsr_read_obj": [ctypes.c_char_p, ctypes.c_int64, vp, ctypes.c_int64, vp, ctypes.c_int64,
                         P(ctypes.c_int64), P(ctypes.c_int64), P(ctypes.c_int64)],
        "hsr_simulate_frame": [vp, P(RFConfigC), P(FrameConfigC), P(FlagsC), ctypes.c_int32, vp, ctypes.c_int32, vp,
                               ctypes.c_int64, ctypes.c_int64, ctypes.c_int32, ctypes.c_int32, vp, vp],
        "hsr_guide_create": [vp, P(vp)],
        "hsr_guide_reset": [vp],
        "hsr_guide_step": [vp],
        "hsr_guide_destroy": [vp],
        "hsr_guide_read": [vp, P(ctypes.c_int32), vp, vp, vp, vp],
        "hsr_guide_write": [vp, ctypes.c_int32, vp, vp, vp, vp],
        "hsr_backend_run_guided": [vp, P(RFConfigC), P(FrameConfigC), P(AntennaC), P(AntennaC), P(FlagsC),
                                   ctypes.c_int64, ctypes.c_int64, ctypes.c_float, ctypes.c_int32, vp,
                                   ctypes.c_int32, vp, P(ctypes.c_double), vp],
        "hsr_noalloc_status": [vp, P(ctypes.c_uint32)],
        "hsr_debug_records": [vp, P(RFConfigC), ctypes.c_int32, P(FlagsC), P(AntennaC), P(AntennaC),
                              ctypes.c_int64, ctypes.c_int64, ctypes.c_int32, vp],
        "hsr_debug_traversal_counts": [vp, P(RFConfigC), ctypes.c_int32, P(FlagsC), ctypes.c_int32, vp, vp, vp,
                                       vp, vp],
        "hsr_set_path_kernel": [ctypes.c_int32],
        "hsr_set_synth_engine": [ctypes.c_int32],
        "hsr_set_bvh_builder": [ctypes.c_int32],
        "hsr_set_bvh_leaf_size": [ctypes.c_int32],
        "hsr_set_bvh_optimize": [ctypes.c_int32],
        "hsr_scene_refit": [vp, vp, ctypes.c_int64],
        "hsr_scene_rebuild": [vp, vp, ctypes.c_int64, vp, ctypes.c_int64],
        "hsr_last_kernel_ms": [vp, P(ctypes.c_float)],
        "hsr_server_create": [P(ServerConfigC), P(vp)],
        "hsr_server_add_scene": [vp, vp, P(ctypes.c_int32)],
        "hsr_server_submit": [vp, P(RequestC), P(ctypes.c_uint64)],
        "hsr_server_wait": [vp, ctypes.c_uint64, ctypes.c_int32, P(RequestResultC)],
        "hsr_server_get_stats": [vp, P(ServerStatsC)],
        "hsr_server_reset_stats": [vp],
        "hsr_server_destroy": [vp],
        "hsr_debug_plan_tick": [ctypes.c_int32, vp, ctypes.c_int64, ctypes.c_int32, vp],
        "hsr_debug_bvh": [vp, vp, ctypes.c_int64, vp, ctypes.c_int64],
        "hsr_debug_halton": [vp, ctypes.c_int64, ctypes.c_int32, vp],
        "hsr_debug_sincos_sweep": [ctypes.c_float, ctypes.c_float, vp, vp, vp],
        "hsr_simulate_batch_ff": [vp, P(RFConfigC), ctypes.c_int32, P(FlagsC), ctypes.c_int32, vp, vp, vp, vp,
                                  ctypes.c_int32, vp],
        "hsr_autotune_batch": [vp, P(RFConfigC), ctypes.c_int32, P(FlagsC), ctypes.c_int32, vp, vp, vp, vp,
                               ctypes.c_int32, ctypes.c_int32, P(LaunchConfigC)],
        "hsr_set_launch_config": [vp, P(LaunchConfigC)],
        "hsr_get_launch_config": [vp, P(LaunchConfigC)],
        "hsr_measure_l2_read": [ctypes.c_int64, ctypes.c_int32, P(ctypes.c_double)],
        "hsr_batch_graph_create": [vp, P(RFConfigC), ctypes.c_int32, P(FlagsC), ctypes.c_int32, vp, vp, vp, vp,
                                   ctypes.c_int32, ctypes.c_int32, vp, P(vp)],
        "hsr_batch_graph_launch": [vp, vp],
        "hsr_batch_graph_status": [vp],
        "hsr_batch_graph_destroy": [vp],
    }
    for name, args in sigs.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = ctypes.c_int
    _lib = L
    return L


def check(status):
    """Raises HsrError for a non-OK status with the library's message."""
    if status != HSR_OK:
        msg = lib().hsr_last_error().decode("utf-8", "replace")
        if status == HSR_ERR_INTERRUPTED:
            raise InterruptedError_(status, msg)
        raise HsrError(status, msg)


def ptr(arr):
    """Address of a contiguous numpy array (or None)."""
    if arr is None:
        return None
    return ctypes.c_void_p(arr.ctypes.data)
