"""Far-field runs (hsr_simulate_batch_ff: FFAntenna TX and RX, emitter.h:226-291) on the
GPU against the oracle's restatement on the same samples: the FP32 reference phase
within 1e-4 relative L2 per pose (GO and non-GO modes), the split-FP64 phase within 1e-3
of the FP64 oracle; guiding and degenerate antennas are refused."""
import ctypes

import numpy as np
import pytest

from hussar_gb300 import HSR_PHASE_SPLIT_FP64, HsrError, PathTracer, _lib, gb300, scenes

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    return float(np.linalg.norm(np.asarray(a, np.complex128) - b) / np.linalg.norm(b))


@pytest.fixture(scope="module")
def ff(product_lib, oracle_lib):
    w = scenes.dihedral_ff_workload(poses=9, samples_per_pose=1 << 16)
    return w, gb300.Backend(w.mesh, None), oracle_lib.Scene(w.mesh)


def tracer(go=True):
    t = PathTracer()
    t.doGuiding = False
    t.maxDepth = 2
    t.useGeometricalOptics = go
    return t


@pytest.mark.parametrize("go", [True, False], ids=["go", "non-go"])
def test_far_field_matches_oracle(ff, go):
    w, be, ora = ff
    t = tracer(go)
    budget = w.budget if go else np.full(len(w.tx), 1 << 14, np.int64)
    rows = be.simulate_batch_ff(w.rf, 256, t, w.tx, w.rx, budget)
    for k in range(len(w.tx)):
        ref = ora.fetch_row_ff(w.rf, 256, w.tx[k], w.rx[k], t, int(budget[k]))
        assert rel_l2(rows[k], ref) <= 1e-4, k


def test_far_field_split_phase_near_fp64(ff):
    w, be, ora = ff
    t = tracer()
    rows = be.simulate_batch_ff(w.rf, 256, t, w.tx, w.rx, w.budget, phase_mode=HSR_PHASE_SPLIT_FP64)
    for k in (0, 4, 8):
        ref = ora.fetch_row_ff(w.rf, 256, w.tx[k], w.rx[k], t, int(w.budget[k]), precision=65)
        assert rel_l2(rows[k], ref) <= 1e-3, k


def test_far_field_index_offset_and_refusals(ff):
    w, be, ora = ff
    t = tracer()
    off = np.full(len(w.tx), 12345, np.int64)
    rows = be.simulate_batch_ff(w.rf, 256, t, w.tx[:2], w.rx[:2], w.budget[:2] // 4, index_offset=off[:2])
    ref = ora.fetch_row_ff(w.rf, 256, w.tx[1], w.rx[1], t, int(w.budget[1] // 4), offset=12345)
    assert rel_l2(rows[1], ref) <= 1e-4
    g = tracer()
    g.doGuiding = True
    with pytest.raises(HsrError) as e:
        be.simulate_batch_ff(w.rf, 256, g, w.tx[:1], w.rx[:1], w.budget[:1])
    assert e.value.status == _lib.HSR_ERR_NOT_SUPPORTED
    bad = w.tx[0].to_c()
    bad.radius = 0.0
    arr = (_lib.FfAntennaC * 1)(bad)
    b = np.array([1024], np.int64)
    o = np.zeros(1, np.int64)
    out = np.zeros(256, np.complex64)
    st = product_lib_call(be, w, t, arr, b, o, out)
    assert st == _lib.HSR_ERR_INVALID_ARGUMENT


def product_lib_call(be, w, t, arr, b, o, out):
    return _lib.lib().hsr_simulate_batch_ff(be.handle, ctypes.byref(w.rf.to_c()), 256, ctypes.byref(t.flags_c()), 1,
                                            ctypes.cast(arr, ctypes.c_void_p), ctypes.cast(arr, ctypes.c_void_p),
                                            _lib.ptr(b), _lib.ptr(o), 0, _lib.ptr(out))
