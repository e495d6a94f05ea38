"""The allocation-free entry point, hsr_simulate_batch_device_noalloc.

It exists for callers that cannot allocate device memory while they simulate (a
real-time loop, work recorded into a larger asynchronous pipeline, a framework whose
memory pool must own every allocation): its scratch is a fixed array inside the
library. Its output must equal that of the allocating entry point
(hsr_simulate_batch_device) on the same device inputs, on two calls in a row (the
second call must not see the first call's leftovers). This file is collected last so
that a run stopping at the first failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-5  # float atomics in the range accumulation: order-dependent rounding only


def rel_l2(a, b):
    a = np.asarray(a, np.complex128)
    b = np.asarray(b, np.complex128)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.mark.parametrize("go", [1, 0], ids=["wavefront-GO", "per-thread-nonGO"])
@pytest.mark.parametrize("phase", ["reference_fp32", "split_fp64"])
def test_no_alloc_matches_allocating_entry_point(product_lib, phase, go):
    """Two allocation-free calls in a row against the allocating entry point on the same
    device inputs (uneven budgets), in both phase modes, on the wavefront kernel (GO mode)
    and the one-thread-per-sample kernel (non-GO mode). The second call allocates nothing
    (the library's allocation count and the device's free memory stay put) and the
    allocation-free status query reports a clean run."""
    torch = pytest.importorskip("torch")
    from hussar_gb300 import PathTracer, _lib, gb300, scenes

    L = product_lib
    w = scenes.dihedral_workload(poses=12, samples_per_pose=1 << 16)
    P, N = 12, w.frame.samplesPerChirp
    t = PathTracer()
    t.doGuiding = False
    t.maxDepth = w.max_depth
    t.useGeometricalOptics = bool(go)
    be = gb300.Backend(w.mesh, None)
    dev = torch.device("cuda")
    stream = torch.cuda.current_stream(dev)
    mode = getattr(_lib, "HSR_PHASE_" + phase.upper())

    def to_dev(arr):
        return torch.frombuffer(bytearray(bytes(arr)), dtype=torch.uint8).to(dev)

    d_tx = to_dev((_lib.AntennaC * P)(*[a.to_c() for a in w.tx]))
    d_rx = to_dev((_lib.AntennaC * P)(*[a.to_c() for a in w.rx]))
    budget = np.array([(1 << 16) - 37 * k for k in range(P)], np.int64)  # uneven budgets
    if not go:
        budget //= 8  # the non-GO estimator traces random directions: fewer samples suffice
    d_budget = torch.from_numpy(budget).to(dev)
    d_offset = torch.zeros(P, dtype=torch.int64, device=dev)
    rf, fl = w.rf.to_c(), t.flags_c()
    ptr = lambda x: ctypes.c_void_p(x.data_ptr())
    sp = ctypes.c_void_p(stream.cuda_stream)

    d_ref = torch.zeros(2 * P * N, dtype=torch.float32, device=dev)
    _lib.check(L.hsr_simulate_batch_device(be.handle, ctypes.byref(rf), N, ctypes.byref(fl), P, ptr(d_tx),
                                           ptr(d_rx), ptr(d_budget), ptr(d_offset), mode,
                                           _lib.HSR_SPLAT_DIRICHLET16, ptr(d_ref), sp))
    bits = ctypes.c_uint32(7)
    _lib.check(L.hsr_scene_status(be.handle, sp, ctypes.byref(bits)))
    assert bits.value == 0
    outs = [torch.full((2 * P * N,), float("nan"), dtype=torch.float32, device=dev) for _ in range(2)]
    torch.cuda.synchronize()
    allocs, free = [], []
    for d_out in outs:
        allocs.append(L.hsr_debug_alloc_count())
        free.append(torch.cuda.mem_get_info()[0])
        _lib.check(L.hsr_simulate_batch_device_noalloc(
            be.handle, ctypes.byref(rf), N, ctypes.byref(fl), P, ptr(d_tx), ptr(d_rx), ptr(d_budget), ptr(d_offset),
            mode, ptr(d_out), sp))
        bits = ctypes.c_uint32(7)
        _lib.check(L.hsr_noalloc_status(sp, ctypes.byref(bits)))
        assert bits.value == 0
    torch.cuda.synchronize()
    # the second call (the first may look the array's address up) allocates nothing
    assert L.hsr_debug_alloc_count() == allocs[1]
    assert torch.cuda.mem_get_info()[0] == free[1]
    ref = d_ref.cpu().numpy().view(np.complex64).reshape(P, N)
    assert np.linalg.norm(ref) > 0
    for d_out in outs:
        got = d_out.cpu().numpy().view(np.complex64).reshape(P, N)
        assert np.isfinite(got).all()
        for p in range(P):
            if np.linalg.norm(ref[p]) == 0:
                assert np.linalg.norm(got[p]) == 0
            else:
                assert rel_l2(got[p], ref[p]) <= RTOL, p


def test_no_alloc_rejects_sizes_beyond_its_scratch(product_lib):
    from hussar_gb300 import PathTracer, _lib, gb300, scenes

    L = product_lib
    w = scenes.dihedral_workload(poses=2, samples_per_pose=1024)
    t = PathTracer()
    t.doGuiding = False
    be = gb300.Backend(w.mesh, None)
    dummy = ctypes.c_void_p(1)  # never dereferenced: the size check comes first
    st = L.hsr_simulate_batch_device_noalloc(be.handle, ctypes.byref(w.rf.to_c()), 4096, ctypes.byref(t.flags_c()),
                                             1, dummy, dummy, dummy, dummy, _lib.HSR_PHASE_REFERENCE_FP32, dummy,
                                             None)
    assert st == _lib.HSR_ERR_INVALID_ARGUMENT
    assert b"fixed size" in L.hsr_last_error()
    st = L.hsr_simulate_batch_device_noalloc(be.handle, ctypes.byref(w.rf.to_c()), 256, ctypes.byref(t.flags_c()),
                                             65, dummy, dummy, dummy, dummy, _lib.HSR_PHASE_REFERENCE_FP32, dummy,
                                             None)
    assert st == _lib.HSR_ERR_INVALID_ARGUMENT
