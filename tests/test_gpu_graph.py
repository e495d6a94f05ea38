"""A plain batch captured into a CUDA graph (hsr_batch_graph_*): each launch replays the
whole batch over the same device buffers and reads their current contents. Rows equal
the direct entry point's (the same samples; FP64 atomics add in a different order)."""
import ctypes

import numpy as np
import pytest

from hussar_gb300 import PathTracer, _lib, gb300, scenes

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    a = np.asarray(a, np.complex128)
    b = np.asarray(b, np.complex128)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def test_graph_replays_match_direct_runs(product_lib):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda", 0)
    w = scenes.dihedral_workload(poses=24)
    t = PathTracer()
    t.doGuiding = False
    t.maxDepth = w.max_depth
    be = gb300.Backend(w.mesh, None)
    P, N = len(w.tx), w.frame.samplesPerChirp
    tx = (_lib.AntennaC * P)(*[a.to_c() for a in w.tx])
    rx = (_lib.AntennaC * P)(*[a.to_c() for a in w.rx])
    d_tx = torch.frombuffer(bytearray(bytes(tx)), dtype=torch.uint8).to(dev)
    d_rx = torch.frombuffer(bytearray(bytes(rx)), dtype=torch.uint8).to(dev)
    budget = np.full(P, 1 << 14, np.int64)
    offset = np.zeros(P, np.int64)
    d_budget = torch.from_numpy(budget.copy()).to(dev)
    d_offset = torch.from_numpy(offset.copy()).to(dev)
    d_out = torch.zeros(2 * P * N, dtype=torch.float32, device=dev)
    g = be.batch_graph(w.rf, N, t, P, d_tx.data_ptr(), d_rx.data_ptr(), d_budget.data_ptr(), d_offset.data_ptr(),
                       d_out.data_ptr())
    stream = torch.cuda.current_stream(dev)
    for _ in range(3):
        g.launch(stream.cuda_stream)
    g.status()
    rows = d_out.cpu().numpy().view(np.complex64).reshape(P, N)
    ref = be.simulate_batch(w.rf, N, t, w.tx, w.rx, budget)
    for k in range(P):
        if np.linalg.norm(ref[k]) > 0:
            assert rel_l2(rows[k], ref[k]) <= 1e-6, k
    # change budgets and offsets in place: the next replay traces the new work
    budget[3] *= 4
    offset[5] = 1 << 20
    d_budget.copy_(torch.from_numpy(budget))
    d_offset.copy_(torch.from_numpy(offset))
    g.launch(stream.cuda_stream)
    g.status()
    rows = d_out.cpu().numpy().view(np.complex64).reshape(P, N)
    ref = be.simulate_batch(w.rf, N, t, w.tx, w.rx, budget, index_offset=offset)
    assert rel_l2(rows[3], ref[3]) <= 1e-6 and rel_l2(rows[5], ref[5]) <= 1e-6
    g.close()


def test_graph_rejects_guiding(product_lib):
    w = scenes.dihedral_workload(poses=2)
    t = PathTracer()
    t.doGuiding = True
    be = gb300.Backend(w.mesh, None)
    h = ctypes.c_void_p()
    st = product_lib.hsr_batch_graph_create(be.handle, ctypes.byref(w.rf.to_c()), 256, ctypes.byref(t.flags_c()), 2,
                                            ctypes.c_void_p(16), ctypes.c_void_p(16), ctypes.c_void_p(16),
                                            ctypes.c_void_p(16), 0, 0, ctypes.c_void_p(16), ctypes.byref(h))
    assert st == _lib.HSR_ERR_NOT_SUPPORTED


def test_graph_with_split_phase_and_synthesis(product_lib):
    """The batched form of the 1 M-triangle boxes configuration inside a graph: split-FP64
    phase and the tensor-core synthesis of the fine range histogram, replayed twice, each
    replay equal to the direct call (same samples; only FP64 atomic order differs). A
    direct call with another N on the same scene in between (which rebuilds the scene's
    twiddle operand) leaves the graph's own operand intact."""
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda", 0)
    w = scenes.boxes_workload(poses=32, min_log2=14, max_log2=16)
    t = PathTracer()
    t.doGuiding = False
    t.maxDepth = w.max_depth
    be = gb300.Backend(w.mesh, None)
    P, N = len(w.tx), w.frame.samplesPerChirp
    tx = (_lib.AntennaC * P)(*[a.to_c() for a in w.tx])
    rx = (_lib.AntennaC * P)(*[a.to_c() for a in w.rx])
    d_tx = torch.frombuffer(bytearray(bytes(tx)), dtype=torch.uint8).to(dev)
    d_rx = torch.frombuffer(bytearray(bytes(rx)), dtype=torch.uint8).to(dev)
    d_budget = torch.from_numpy(w.budget.copy()).to(dev)
    d_offset = torch.zeros(P, dtype=torch.int64, device=dev)
    d_out = torch.zeros(2 * P * N, dtype=torch.float32, device=dev)
    g = be.batch_graph(w.rf, N, t, P, d_tx.data_ptr(), d_rx.data_ptr(), d_budget.data_ptr(), d_offset.data_ptr(),
                       d_out.data_ptr(), phase_mode=_lib.HSR_PHASE_SPLIT_FP64, splat_mode=_lib.HSR_SPLAT_FINE_SYNTH)
    stream = torch.cuda.current_stream(dev)
    ref = be.simulate_batch(w.rf, N, t, w.tx, w.rx, w.budget, phase_mode=_lib.HSR_PHASE_SPLIT_FP64,
                            splat_mode=_lib.HSR_SPLAT_FINE_SYNTH)
    for rep in range(2):
        if rep == 1:  # another N on the scene: its own operand is rebuilt, the graph's is not
            be.simulate_batch(w.rf, 128, t, w.tx[:2], w.rx[:2], w.budget[:2], phase_mode=_lib.HSR_PHASE_SPLIT_FP64,
                              splat_mode=_lib.HSR_SPLAT_FINE_SYNTH)
        d_out.zero_()
        g.launch(stream.cuda_stream)
        g.status()
        rows = d_out.cpu().numpy().view(np.complex64).reshape(P, N)
        nz = [k for k in range(P) if np.linalg.norm(ref[k]) > 0]
        assert len(nz) > P // 2
        for k in nz:
            assert rel_l2(rows[k], ref[k]) <= 1e-5, (rep, k)
    g.close()
