"""The launch-shape autotuner (hsr_autotune_batch): it times the caller's batch under
candidate shapes (work-item tile, CTAs per SM, queue threshold: 32, 64, 128, 256, the
primary field formed on a hit, the coherent stage order) and keeps the fastest.
A shape changes only the grouping of sums, so rows agree with the default shape up to
summation order (1e-5 relative L2)."""
import numpy as np
import pytest

from hussar_gb300 import NFAntenna, PathTracer, gb300, scenes

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    a = np.asarray(a, np.complex128)
    b = np.asarray(b, np.complex128)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def test_autotune_picks_a_valid_shape_and_keeps_results(product_lib):
    w = scenes.sphere_ground_workload(samples=1 << 20, level=5)
    t = PathTracer()
    t.doGuiding = False
    t.maxDepth = w.max_depth
    be = gb300.Backend(w.mesh, None)
    N = w.frame.samplesPerChirp
    ref = be.simulate_batch(w.rf, N, t, w.tx, w.rx, w.budget)
    best = be.autotune(w.rf, N, t, w.tx, w.rx, w.budget)
    print("autotuned", best)
    assert best["tile"] in (1024, 2048, 4096, 8192, 16384)
    assert best["ctas_per_sm"] in (0, 2, 3, 4) and 1 <= best["queue_threshold"] <= 256
    assert 0 < best["trace_ms"] <= best["default_trace_ms"]
    tuned = be.simulate_batch(w.rf, N, t, w.tx, w.rx, w.budget)
    assert rel_l2(tuned, ref) <= 1e-5
    # explicit shapes at each path-stack capacity (320, 384 and 512 entries) give the same
    # rows too, in both phase modes, and the default can be restored
    for tile, ctas, q, lazy, coh in ((1024, 2, 32, 0, 0), (2048, 3, 100, 0, 1), (1024, 4, 256, 0, 0),
                                     (4096, 4, 200, 0, 1), (1024, 4, 64, 1, 0), (2048, 4, 128, 1, 1),
                                     (1024, 4, 256, 1, 1), (1024, 4, 32, 0, 1)):
        be.set_launch_config(tile=tile, ctas_per_sm=ctas, queue_threshold=q, field_on_hit=lazy, coherent_order=coh)
        assert rel_l2(be.simulate_batch(w.rf, N, t, w.tx, w.rx, w.budget), ref) <= 1e-5, (tile, ctas, q, lazy, coh)
    from hussar_gb300 import HSR_PHASE_SPLIT_FP64
    be.set_launch_config(default=True)
    ref_split = be.simulate_batch(w.rf, N, t, w.tx, w.rx, w.budget, phase_mode=HSR_PHASE_SPLIT_FP64)
    for lazy, coh in ((0, 0), (1, 0), (0, 1)):
        be.set_launch_config(tile=1024, ctas_per_sm=4, queue_threshold=256, field_on_hit=lazy, coherent_order=coh)
        split = be.simulate_batch(w.rf, N, t, w.tx, w.rx, w.budget, phase_mode=HSR_PHASE_SPLIT_FP64)
        assert rel_l2(split, ref_split) <= 1e-5, (lazy, coh)
    be.set_launch_config(default=True)
    assert rel_l2(be.simulate_batch(w.rf, N, t, w.tx, w.rx, w.budget), ref) <= 1e-5


def test_field_on_hit_keeps_rows_where_primaries_miss(product_lib):
    """The dihedral (most primary rays miss the reflector): the primary field formed on a
    hit gives the same rows as the eager form, with and without the direct TX -> RX term
    (which needs the field of every primary ray; the RX sits 5 cm above the TX, since the
    monostatic direct term is the reference's 0/0)."""
    w = scenes.dihedral_workload(poses=24, samples_per_pose=1 << 16)
    rx = [NFAntenna(a.position() + np.array([0, 0.05, 0], np.float32), a.rotation()) for a in w.tx]
    be = gb300.Backend(w.mesh, None)
    N = w.frame.samplesPerChirp
    for only_indirect in (True, False):
        t = PathTracer()
        t.doGuiding = False
        t.maxDepth = w.max_depth
        t.onlyIndirect = only_indirect
        be.set_launch_config(default=True)
        ref = be.simulate_batch(w.rf, N, t, w.tx, rx, w.budget)
        assert np.isfinite(ref).all() and (np.linalg.norm(ref, axis=1) > 0).all()
        be.set_launch_config(tile=4096, ctas_per_sm=4, queue_threshold=64, field_on_hit=1)
        got = be.simulate_batch(w.rf, N, t, w.tx, rx, w.budget)
        for k in range(len(w.tx)):
            assert rel_l2(got[k], ref[k]) <= 1e-5, (only_indirect, k)
    be.set_launch_config(default=True)


def test_coherent_order_matches_the_oracle_on_boxes(product_lib):
    """The coherent stage order (samples and popped paths grouped by direction) on the
    batched boxes configuration, against the oracle at 1e-4 as the default order is."""
    from oracle import pyoracle
    w = scenes.boxes_workload(poses=6)
    w.budget = np.minimum(w.budget, 1 << 14)
    t = PathTracer()
    t.doGuiding = False
    t.maxDepth = w.max_depth
    be = gb300.Backend(w.mesh, None)
    N = w.frame.samplesPerChirp
    be.set_launch_config(tile=1024, ctas_per_sm=4, queue_threshold=64, coherent_order=1)
    rows = be.simulate_batch(w.rf, N, t, w.tx, w.rx, w.budget)
    be.set_launch_config(default=True)
    ora = pyoracle.Scene(w.mesh)
    for k in range(len(w.tx)):
        ref = ora.fetch_row(w.rf, N, w.tx[k], w.rx[k], t, int(w.budget[k]))
        assert rel_l2(rows[k], ref) <= 1e-4, k
