"""Fine range histogram + synthesis GEMM (HSR_SPLAT_FINE_SYNTH).

The estimator is the exact (untruncated, finite-N) spectrum of each contribution's IF
chirp; its FP64 oracle is the restatement with Frame::splat<16> replaced by the exact
Dirichlet sum, on the same float Halton samples. The synthesis has a second-order Taylor
remainder (~-70 dB on average); the tolerance below is stated per test."""
import ctypes

import numpy as np
import pytest

from hussar_gb300 import HSR_SPLAT_DIRICHLET16, HSR_SPLAT_FINE_SYNTH, PathTracer, gb300, scenes

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    a = np.asarray(a, np.complex128)
    b = np.asarray(b, np.complex128)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def tracer(w, guiding=False):
    t = PathTracer()
    t.maxDepth = w.max_depth
    t.doGuiding = guiding
    return t


@pytest.fixture
def engine(product_lib):
    def use(e):
        product_lib.hsr_set_synth_engine(e)
    yield use
    product_lib.hsr_set_synth_engine(0)


@pytest.fixture(scope="module")
def dihedral(product_lib, oracle_lib):
    w = scenes.dihedral_workload()
    return w, gb300.Backend(w.mesh, None), oracle_lib.Scene(w.mesh)


@pytest.mark.parametrize("kind", [0, 1], ids=["tensor-cores", "cuda-cores"])
def test_fine_synth_matches_fp64_exact_oracle(dihedral, engine, kind):
    w, be, ora = dihedral
    engine(kind)
    t = tracer(w)
    sel = [10, 45, 80]
    S = 1 << 16
    rows = be.simulate_batch(w.rf, 256, t, [w.tx[i] for i in sel], [w.rx[i] for i in sel], [S] * 3,
                             splat_mode=HSR_SPLAT_FINE_SYNTH)
    for j, k in enumerate(sel):
        ref64 = ora.fetch_row(w.rf, 256, w.tx[k], w.rx[k], t, S, precision=65, exact=True)
        ref32 = ora.fetch_row(w.rf, 256, w.tx[k], w.rx[k], t, S, precision=32, exact=True)
        if np.linalg.norm(ref64) == 0:
            continue
        e32, e64, path = rel_l2(rows[j], ref32), rel_l2(rows[j], ref64), rel_l2(ref32, ref64)
        print("pose", k, "fine-synth vs FP32-exact %.2e, vs FP64-exact %.2e; FP32 path vs FP64 %.2e" % (e32, e64, path))
        # the synthesis (second-order remainder, BF16-split GEMM) against the same FP32 path
        assert e32 <= 1e-3
        # against FP64: the FP32 path's own error plus the synthesis
        assert e64 <= path + 1e-3


def test_engines_agree_on_many_poses(dihedral, engine):
    """300 poses: three 128-row M tiles, the last one partial."""
    w, be, _ = dihedral
    t = tracer(w)
    idx = np.arange(300) % len(w.tx)
    budget = np.full(300, 1 << 12, np.int64)
    engine(0)
    a = be.simulate_batch(w.rf, 256, t, [w.tx[i] for i in idx], [w.rx[i] for i in idx], budget,
                          splat_mode=HSR_SPLAT_FINE_SYNTH)
    engine(1)
    b = be.simulate_batch(w.rf, 256, t, [w.tx[i] for i in idx], [w.rx[i] for i in idx], budget,
                          splat_mode=HSR_SPLAT_FINE_SYNTH)
    assert np.isfinite(a).all()
    nz = np.linalg.norm(b, axis=1) > 0
    assert nz.sum() > 100
    err = max(rel_l2(a[i], b[i]) for i in np.nonzero(nz)[0])
    print("tensor vs cuda cores, worst pose", err)
    assert err <= 2e-5  # three-term BF16 split ~ FP32
    # the same pose repeated gives the same row regardless of its position in the batch
    assert rel_l2(a[45], a[45 + 91]) <= 1e-5


def test_fine_synth_close_to_reference_splat(dihedral):
    """The reference's 33-bin kernel is the truncated large-N limit of the exact one:
    the two estimators agree to the truncation level (a few percent)."""
    w, be, _ = dihedral
    t = tracer(w)
    k = 45
    a = be.simulate_batch(w.rf, 256, t, [w.tx[k]], [w.rx[k]], [1 << 18], splat_mode=HSR_SPLAT_FINE_SYNTH)[0]
    b = be.simulate_batch(w.rf, 256, t, [w.tx[k]], [w.rx[k]], [1 << 18], splat_mode=HSR_SPLAT_DIRICHLET16)[0]
    err = rel_l2(b, a)
    print("splat16 vs exact synthesis", err)
    assert 1e-3 < err < 0.2
    assert np.argmax(np.abs(a)) == np.argmax(np.abs(b))


def test_fine_synth_non_power_of_two_bins(product_lib, oracle_lib):
    rf, _ = scenes.rf_77ghz(200)
    w = scenes.dihedral_workload(poses=5)
    be = gb300.Backend(w.mesh, None)
    ora = oracle_lib.Scene(w.mesh)
    t = tracer(w)
    rows = be.simulate_batch(rf, 200, t, w.tx[2:3], w.rx[2:3], [1 << 16], splat_mode=HSR_SPLAT_FINE_SYNTH)
    ref = ora.fetch_row(rf, 200, w.tx[2], w.rx[2], t, 1 << 16, precision=65, exact=True)
    assert rel_l2(rows[0], ref) <= 2e-3


def test_fine_synth_guided(dihedral):
    w, be, _ = dihedral
    k = 45
    ref = be.simulate_batch(w.rf, 256, tracer(w), [w.tx[k]], [w.rx[k]], [1 << 24],
                            splat_mode=HSR_SPLAT_FINE_SYNTH)[0]
    g = be.simulate_batch(w.rf, 256, tracer(w, True), [w.tx[k]], [w.rx[k]], [1 << 18],
                          splat_mode=HSR_SPLAT_FINE_SYNTH)[0]
    assert rel_l2(g, ref) < 0.05


@pytest.mark.parametrize("N", [64, 128, 512, 1000])
def test_fine_synth_column_tilings(product_lib, oracle_lib, engine, N):
    """Every column tiling of the tensor-core GEMM: N <= 128 (one 256-column half per
    CTA), 512 and 1000 (two and four groups of two halves), with a partial row tile (3
    poses): against the FP64 exact oracle, and the two engines against each other."""
    rf, _ = scenes.rf_77ghz(N)
    w = scenes.dihedral_workload(poses=5)
    be = gb300.Backend(w.mesh, None)
    ora = oracle_lib.Scene(w.mesh)
    t = tracer(w)
    sel = [1, 2, 3]
    engine(0)
    rows = be.simulate_batch(rf, N, t, [w.tx[k] for k in sel], [w.rx[k] for k in sel], [1 << 16] * 3,
                             splat_mode=HSR_SPLAT_FINE_SYNTH)
    engine(1)
    rows_cc = be.simulate_batch(rf, N, t, [w.tx[k] for k in sel], [w.rx[k] for k in sel], [1 << 16] * 3,
                                splat_mode=HSR_SPLAT_FINE_SYNTH)
    for i, k in enumerate(sel):
        ref = ora.fetch_row(rf, N, w.tx[k], w.rx[k], t, 1 << 16, precision=65, exact=True)
        assert rel_l2(rows[i], ref) <= 2e-3, (N, k)
        assert rel_l2(rows[i], rows_cc[i]) <= 1e-5, (N, k)
