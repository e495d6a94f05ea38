"""GPU parity: the CUDA path (through the C ABI) against the oracle on identical Halton
samples. The bar is the parity tolerance: relative L2 of the complex IF signal
<= 1e-4 (the IF signal is the inverse DFT of the frame row, which is unitary, so the
relative L2 is the same in either domain). Integer/index results (hit primitive,
visibility, record structure) must agree exactly."""
import numpy as np
import pytest

from hussar_gb300 import (HSR_PHASE_REFERENCE_FP32, HSR_PHASE_SPLIT_FP64, FrameConfig, HsrError, NFAntenna,
                          PathTracer, Scene, TriangleMesh, gb300, scenes)

pytestmark = pytest.mark.gpu

RTOL_IF = 1e-4  # relative L2 of the complex IF signal


def rel_l2(a, b):
    a = np.asarray(a, np.complex128)
    b = np.asarray(b, np.complex128)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.fixture(params=[0, 1], ids=["wavefront", "per-thread"])
def kernel_kind(request, product_lib):
    """Runs a test with the wavefront kernel and with the one-thread-per-sample kernel."""
    product_lib.hsr_set_path_kernel(request.param)
    yield request.param
    product_lib.hsr_set_path_kernel(0)


def tracer_for(w, guiding=False):
    t = PathTracer()
    t.maxDepth = w.max_depth
    t.doGuiding = guiding
    return t


@pytest.fixture(scope="module")
def dihedral(product_lib, oracle_lib):
    w = scenes.dihedral_workload()
    be = gb300.Backend(w.mesh, None)
    return w, be, oracle_lib.Scene(w.mesh)


@pytest.fixture(scope="module")
def sphere(product_lib, oracle_lib):
    w = scenes.sphere_ground_workload(samples=1 << 16)
    be = gb300.Backend(w.mesh, None)
    return w, be, oracle_lib.Scene(w.mesh)


def test_bvh_stats(sphere):
    w, be, _ = sphere
    st = be.bvh_stats()
    # internal nodes: those left after leaves of up to four triangles are formed
    assert st["leaves"] == 81922 and 81922 // 8 <= st["nodes"] < 81921
    assert 1 <= st["max_depth"] <= 64


def test_ray_queries_match_oracle(sphere):
    w, be, ora = sphere
    rng = np.random.default_rng(5)
    n = 20000
    o = np.concatenate([rng.uniform([-3, 0.05, -3], [3, 2, 3], (n // 2, 3)),
                        np.tile([[10.0, 0.5, 0.0]], (n // 2, 1))]).astype(np.float32)
    d = rng.normal(size=(n, 3))
    d[n // 2:] = np.array([0.0, 0.5, 0.0]) - o[n // 2:] + rng.normal(scale=0.3, size=(n // 2, 3))
    d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    t, p, nn, prim = be.intersect(o, d)
    t2, p2, n2, prim2 = ora.intersect(o, d)
    hit = prim2 >= 0
    assert hit.sum() > n // 4
    assert np.array_equal(prim, prim2)
    assert np.array_equal(t[hit].view(np.uint32), t2[hit].view(np.uint32))
    assert np.array_equal(p[hit].view(np.uint32), p2[hit].view(np.uint32))
    assert np.array_equal(nn[hit].view(np.uint32), n2[hit].view(np.uint32))
    tf = rng.uniform(0.1, 12, n).astype(np.float32)
    assert np.array_equal(be.visible(o, d, tf), ora.visible(o, d, tf))


def test_dihedral_all_poses_full_size(dihedral, kernel_kind):
    """The 4-triangle dihedral sweep at its full size: 91 poses x 2^18 samples."""
    w, be, ora = dihedral
    t = tracer_for(w)
    rows = be.simulate_batch(w.rf, w.frame.samplesPerChirp, t, w.tx, w.rx, w.budget)
    errs = []
    for k in range(len(w.tx)):
        ref = ora.fetch_row(w.rf, w.frame.samplesPerChirp, w.tx[k], w.rx[k], t, int(w.budget[k]))
        if np.linalg.norm(ref) == 0:
            assert np.linalg.norm(rows[k]) == 0
            continue
        errs.append(rel_l2(rows[k], ref))
    assert len(errs) > 80
    assert max(errs) <= RTOL_IF, (max(errs), int(np.argmax(errs)))


def test_dihedral_peak_at_corner_range(dihedral):
    w, be, _ = dihedral
    t = tracer_for(w)
    k = 45  # boresight of the corner
    rows = be.simulate_batch(w.rf, w.frame.samplesPerChirp, t, w.tx[k:k + 1], w.rx[k:k + 1], w.budget[k:k + 1])
    # round trip ~2 m to the corner edge: bin = N * frac((2r/c + delay) * S / adcRate)
    r = np.linalg.norm(w.tx[k].position() - np.array([0, 0.05, 0]))
    dt = 2 * r / 299792458.0 + w.rf.antennaDelay
    expect = w.frame.samplesPerChirp * ((dt * w.rf.freqSlope / w.rf.adcRate) % 1.0)
    assert abs(int(np.argmax(np.abs(rows[0]))) - expect) <= 1.0


def test_records_match_oracle(dihedral):
    """Per-sample next-event estimates: the same events on every sample (bit-identical
    primary directions and hits), times to 1e-6 and values to 1e-5 relative (the phase's
    sin/cos are FP32 here and double-then-rounded in the reference)."""
    w, be, ora = dihedral
    t = tracer_for(w)
    k = 40
    scn = Scene(w.rf, w.tx[k], w.rx[k])
    n = 1 << 16
    g = be.debug_records(scn, t, w.frame.samplesPerChirp, n)
    c = ora.records(w.rf, w.frame, w.tx[k], w.rx[k], t, 0, n)
    same = np.all((g["depth"] == c["depth"]) & (g["splatted"] == c["splatted"]), axis=1)
    assert same.all(), int(np.count_nonzero(~same))
    m = (c["depth"] >= 0) & same[:, None]
    assert m.sum() > 100
    assert np.allclose(g["time"][m], c["time"][m], rtol=1e-6, atol=0)
    m = m & (c["splatted"] == 1)
    assert np.allclose(g["bin"][m], c["bin"][m], rtol=0, atol=1e-3)
    vg = g["value_re"][m] + 1j * g["value_im"][m]
    vc = c["value_re"][m] + 1j * c["value_im"][m]
    assert np.max(np.abs(vg - vc)) <= 1e-5 * np.max(np.abs(vc))


def test_sphere_ground_parity(sphere, kernel_kind):
    w, be, ora = sphere
    t = tracer_for(w)
    rows = be.simulate_batch(w.rf, w.frame.samplesPerChirp, t, w.tx, w.rx, w.budget)
    ref = ora.fetch_row(w.rf, w.frame.samplesPerChirp, w.tx[0], w.rx[0], t, int(w.budget[0]))
    assert np.linalg.norm(ref) > 0
    assert rel_l2(rows[0], ref) <= RTOL_IF


def test_sphere_ground_full_budget(product_lib, oracle_lib, kernel_kind):
    """The sphere+ground configuration at its own budget: 2^22 Halton samples, 3 bounces,
    512 range bins, one launch, against the oracle at 1e-4."""
    w = scenes.sphere_ground_workload(samples=1 << 22)
    be = gb300.Backend(w.mesh, None)
    t = tracer_for(w)
    rows = be.simulate_batch(w.rf, w.frame.samplesPerChirp, t, w.tx, w.rx, w.budget)
    ref = oracle_lib.Scene(w.mesh).fetch_row(w.rf, w.frame.samplesPerChirp, w.tx[0], w.rx[0], t, int(w.budget[0]))
    err = rel_l2(rows[0], ref)
    print("sphere+ground 2^22: rel L2 %.2e" % err)
    assert np.linalg.norm(ref) > 0 and err <= RTOL_IF


def test_sphere_ground_records(sphere):
    w, be, ora = sphere
    t = tracer_for(w)
    scn = Scene(w.rf, w.tx[0], w.rx[0])
    n = 1 << 14
    g = be.debug_records(scn, t, w.frame.samplesPerChirp, n)
    c = ora.records(w.rf, w.frame, w.tx[0], w.rx[0], t, 0, n)
    # identical event structure on every sample, bins to 2e-3 (compared circularly)
    same = np.all(g["depth"] == c["depth"], axis=1)
    assert same.all(), int(np.count_nonzero(~same))
    m = (c["depth"] >= 0) & (c["splatted"] == 1)
    diff = np.abs(g["bin"][m] - c["bin"][m])
    diff = np.minimum(diff, w.frame.samplesPerChirp - diff)
    assert np.all(diff <= 2e-3)


def test_backend_run_api_and_layout(dihedral):
    """The drop-in flow: PathTracer.run(backend, scene, samples) -> fetchFrame(); only
    chirp 0 / channel 0 are written (path.h:130, 291-292)."""
    w, _, ora = dihedral
    t = tracer_for(w)
    t.configureFrame(FrameConfig(2, w.frame.samplesPerChirp, 3))
    be = gb300.Backend(w.mesh, t)
    k = 30
    scn = Scene(w.rf, w.tx[k], w.rx[k])
    t.run(be, scn, 1 << 16)
    f = t.fetchFrame()
    assert t.totalWeight == float(1 << 16)
    assert np.count_nonzero(f.data[1]) == 0 and np.count_nonzero(f.data[:, :, 1:]) == 0
    ref = ora.fetch_row(w.rf, w.frame.samplesPerChirp, w.tx[k], w.rx[k], t, 1 << 16)
    assert rel_l2(f.data[0, :, 0], ref) <= RTOL_IF


def test_index_offset_linearity(dihedral):
    """Two runs over [0,B) and [B,2B) add up to one run over [0,2B) (PathTracer::run
    advances sampleIndexOffset between backend runs, path.h:198)."""
    w, _, _ = dihedral
    t = tracer_for(w)
    t.configureFrame(w.frame)
    be = gb300.Backend(w.mesh, t)
    scn = Scene(w.rf, w.tx[45], w.rx[45])
    B = 1 << 15
    t.clearFrame()
    t.sampleIndexOffset = 0
    be.run(scn, B)
    t.sampleIndexOffset = B
    be.run(scn, B)
    two = t.frame.data.copy()
    t.clearFrame()
    t.sampleIndexOffset = 0
    be.run(scn, 2 * B)
    assert rel_l2(two, t.frame.data) <= 1e-5


def test_split_phase_reduces_error_vs_fp64(sphere, kernel_kind):
    w, be, ora = sphere
    t = tracer_for(w)
    # FP64 oracle on the same samples: the float Halton values of the FP32 run, all else in double
    fp64 = ora.fetch_row(w.rf, w.frame.samplesPerChirp, w.tx[0], w.rx[0], t, int(w.budget[0]), precision=65)
    plain = be.simulate_batch(w.rf, w.frame.samplesPerChirp, t, w.tx, w.rx, w.budget,
                              phase_mode=HSR_PHASE_REFERENCE_FP32)[0]
    split = be.simulate_batch(w.rf, w.frame.samplesPerChirp, t, w.tx, w.rx, w.budget,
                              phase_mode=HSR_PHASE_SPLIT_FP64)[0]
    e_plain, e_split = rel_l2(plain, fp64), rel_l2(split, fp64)
    assert e_split < e_plain
    assert e_split < 1e-2


def test_batch_equals_single_pose_runs(dihedral, kernel_kind):
    w, be, _ = dihedral
    t = tracer_for(w)
    sel = [3, 44, 45, 80]
    budget = np.array([1 << 12, 1 << 15, 3000, 1 << 14], np.int64)
    rows = be.simulate_batch(w.rf, 256, t, [w.tx[i] for i in sel], [w.rx[i] for i in sel], budget)
    for j, i in enumerate(sel):
        one = be.simulate_batch(w.rf, 256, t, [w.tx[i]], [w.rx[i]], budget[j:j + 1])
        if np.linalg.norm(one) == 0:
            assert np.linalg.norm(rows[j]) == 0
        else:
            assert rel_l2(rows[j], one[0]) <= 1e-5


def test_edge_cases(product_lib, oracle_lib, kernel_kind):
    rf, fc = scenes.rf_77ghz(256)
    t = PathTracer()
    t.doGuiding = False
    t.maxDepth = 3
    a = NFAntenna([1.0, 0.05, 0.3], scenes.looking(0.3))
    # empty scene: every ray misses, nothing is splatted
    empty = gb300.Backend(TriangleMesh(), None)
    rows = empty.simulate_batch(rf, 256, t, [a], [a], [4096])
    assert np.count_nonzero(rows) == 0
    # one triangle facing the sensor
    one = TriangleMesh()
    one.append(np.array([[0, -0.2, -0.2], [0, 0.3, -0.2], [0, 0.0, 0.4]], np.float32), [[0, 1, 2]])
    be = gb300.Backend(one, None)
    ora = oracle_lib.Scene(one)
    t.onlyIndirect = True
    rows = be.simulate_batch(rf, 256, t, [a], [a], [1 << 16])
    ref = ora.fetch_row(rf, 256, a, a, t, 1 << 16)
    assert np.linalg.norm(ref) > 0 and rel_l2(rows[0], ref) <= RTOL_IF
    # direct path enabled (onlyIndirect = False) with a bistatic pair
    t.onlyIndirect = False
    b = NFAntenna([1.0, 0.05, 0.35], scenes.looking(0.3))
    rows = be.simulate_batch(rf, 256, t, [a], [b], [1 << 14])
    ref = ora.fetch_row(rf, 256, a, b, t, 1 << 14)
    assert rel_l2(rows[0], ref) <= RTOL_IF
    t.onlyIndirect = True
    # zero budget: fetchFrame divides an empty frame by a zero total weight, 0 * (1/0) = NaN,
    # exactly as the reference's Frame::operator/ does (radar.h:388-392, path.h:453-455)
    rows = be.simulate_batch(rf, 256, t, [a, a], [a, a], [0, 1 << 12])
    assert np.all(np.isnan(rows[0].real)) and np.all(np.isfinite(rows[1]))
    # non-power-of-two range bins exercise the reference's unsigned modulo
    rows = be.simulate_batch(rf, 200, t, [a], [a], [1 << 15])
    ref = ora.fetch_row(rf, 200, a, a, t, 1 << 15)
    assert rel_l2(rows[0], ref) <= RTOL_IF
    # CW radar (freqSlope = 0): everything lands in sample 0 (radar.h:233-235)
    cw = scenes.RFConfig(startFreq=78e9, freqSlope=0.0, adcRate=5e6, idleTime=1e-4, rampTime=5e-5)
    rows = be.simulate_batch(cw, 1, t, [a], [a], [1 << 14])
    ref = ora.fetch_row(cw, 1, a, a, t, 1 << 14)
    assert rel_l2(rows[0], ref) <= RTOL_IF


def test_filtering_and_phase_flags(sphere, kernel_kind):
    """Flag combinations of path.h:153-169 against the oracle, each at 1e-4. Without the
    filtering sphere the frame is dominated by long (tens of metres) ground paths whose
    FP32 phase has a rounding step of ~4e-3 rad, so this holds only with bit-identical
    path geometry (identical primary directions)."""
    w, be, ora = sphere
    base = tracer_for(w)
    combos = [dict(doFiltering=False), dict(filteringSphere=False), dict(correctPhase=True),
              dict(poDiffraction=True), dict(produceDebugImage=True), dict(useGeometricalOptics=False)]
    for c in combos:
        t = tracer_for(w)
        for k, v in c.items():
            setattr(t, k, v)
        B = 1 << 14
        rows = be.simulate_batch(w.rf, w.frame.samplesPerChirp, t, w.tx, w.rx, [B])
        ref = ora.fetch_row(w.rf, w.frame.samplesPerChirp, w.tx[0], w.rx[0], t, B)
        if np.linalg.norm(ref) == 0:
            assert np.linalg.norm(rows[0]) == 0, c
        else:
            assert rel_l2(rows[0], ref) <= RTOL_IF, (c, rel_l2(rows[0], ref))
    del base


def test_interrupt_flag(dihedral):
    w, _, _ = dihedral
    t = tracer_for(w)
    t.configureFrame(w.frame)
    be = gb300.Backend(w.mesh, t)
    with pytest.raises(HsrError) as e:
        be.run(Scene(w.rf, w.tx[0], w.rx[0]), 1024, interruptFlag=True)
    assert e.value.status == 4


def test_kernels_agree(sphere, product_lib):
    """The wavefront and per-thread kernels trace the same samples with the same
    arithmetic; only the order of the float atomics differs."""
    w, be, _ = sphere
    t = tracer_for(w)
    product_lib.hsr_set_path_kernel(0)
    a = be.simulate_batch(w.rf, w.frame.samplesPerChirp, t, w.tx, w.rx, w.budget)
    product_lib.hsr_set_path_kernel(1)
    b = be.simulate_batch(w.rf, w.frame.samplesPerChirp, t, w.tx, w.rx, w.budget)
    product_lib.hsr_set_path_kernel(0)
    assert rel_l2(a, b) <= 1e-5
