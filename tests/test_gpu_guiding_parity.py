"""Device path guiding against the oracle's restatement of the same tree (the product's
2-D tree behind GuidingWrapper, path.h:17-131; the reference's own BTree lives in the
libguiding submodule, which is not part of the reference sources).

- step (GuidingWrapper::step, path.h:119-126): from the device's own training sums, the
  device's new sampling tree, probabilities and training topology equal the oracle's
  bit for bit;
- sample and train (path.h:265-270, 448-450): one guided iteration from the same tree
  gives the same frame (1e-4 relative L2) and the same leaf sums (float atomics on the
  device against one-thread sums in the oracle: 1e-4 relative);
- schedule (PathTracer::run, path.h:171-224): the whole guided run matches the oracle's
  whole guided run (its own trees, trained from its own sums) within 1e-4.
All in the reference's FP32 phase, where the device arithmetic rounds as the oracle's."""
import numpy as np
import pytest

from hussar_gb300 import PathTracer, Scene, gb300, scenes

pytestmark = pytest.mark.gpu

POSE = 30
TOL = 1e-4  # relative L2 of the complex frame; relative difference of a leaf sum


def rel_l2(a, b):
    a = np.asarray(a, np.complex128)
    b = np.asarray(b, np.complex128)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def tracer(w):
    t = PathTracer()
    t.maxDepth = w.max_depth
    t.doGuiding = True
    t.configureFrame(w.frame)
    return t


@pytest.fixture(scope="module")
def setup(product_lib):
    from oracle import pyoracle
    w = scenes.dihedral_workload()
    return w, gb300.Backend(w.mesh, None), pyoracle.Scene(w.mesh)


def device_state(g):
    from oracle import pyoracle
    return pyoracle.GuideState(*g.read())


def train_once(g, t, sc, budget, train=True):
    t.clearFrame()
    t.sampleIndexOffset = 0
    g.run_iteration(t, sc, budget, train)
    return t.frame.data[0, :, 0].copy(), t.totalWeight


def test_step_matches_oracle_bit_exact(setup):
    from oracle import pyoracle
    w, be, _ = setup
    t = tracer(w)
    sc = Scene(w.rf, w.tx[POSE], w.rx[POSE])
    g = gb300.Guide(be)
    og = pyoracle.Guide()
    counts = []
    for it in range(5):
        train_once(g, t, sc, 1 << 15)
        pre = device_state(g)
        g.step()
        got = device_state(g)
        og.set(pre)
        og.step()
        want = og.get()
        n, m = want.count, pre.count
        assert got.count == n, it
        np.testing.assert_array_equal(got.train_child[:n], want.train_child[:n])
        np.testing.assert_array_equal(got.samp_child[:m], want.samp_child[:m])
        assert got.samp_p[:m].tobytes() == want.samp_p[:m].tobytes(), it
        assert not got.acc2[:n].any()
        counts.append(n)
    print("training tree nodes after each step:", counts)
    assert counts[-1] > 16  # the tree refined


def test_guided_iteration_matches_oracle(setup):
    """Sampling through a trained tree and training into it: one iteration on the device
    and in the oracle from the same state."""
    from oracle import pyoracle
    w, be, ora = setup
    t = tracer(w)
    sc = Scene(w.rf, w.tx[POSE], w.rx[POSE])
    g = gb300.Guide(be)
    for _ in range(3):
        train_once(g, t, sc, 1 << 15)
        g.step()
    start = device_state(g)
    assert (start.samp_child >= 0).sum() > 4  # a tree that warps samples
    og = pyoracle.Guide()
    og.set(start)
    budget = 1 << 16
    row, tw = train_once(g, t, sc, budget, train=True)
    fr, ow = og.run_pass(ora, w.rf, w.frame, w.tx[POSE], w.rx[POSE], t, budget, train=True)
    e = rel_l2(row, fr[0, :, 0])
    got, want = device_state(g), og.get()
    leaves = [n for n in want.reachable("train") if want.train_child[n] < 0]
    a = got.acc2[leaves].astype(np.float64)
    b = want.acc2[leaves].astype(np.float64)
    worst = float(np.max(np.abs(a - b)) / np.max(np.abs(b)))
    print("guided iteration: frame rel L2 %.2e, leaf sums worst %.2e over %d leaves" % (e, worst, len(leaves)))
    assert tw == ow
    assert e <= TOL
    assert np.count_nonzero(b) > 4 and worst <= TOL


@pytest.mark.parametrize("samples,clear", [(1 << 17, True), (100_000, False)])
def test_guided_schedule_matches_oracle(setup, samples, clear):
    from oracle import pyoracle
    w, _, ora = setup
    t = tracer(w)
    t.clearBeforeIteration = clear
    be = gb300.Backend(w.mesh, t)
    sc = Scene(w.rf, w.tx[POSE], w.rx[POSE])
    t.run(be, sc, samples)
    og = pyoracle.Guide()
    fr, ow = og.path_tracer_run(ora, w.rf, w.frame, w.tx[POSE], w.rx[POSE], t, samples)
    e = rel_l2(t.frame.data[0, :, 0], fr[0, :, 0])
    print("guided schedule %d samples (clear %s): rel L2 vs oracle %.2e, final tree %d nodes"
          % (samples, clear, e, og.get().count))
    assert t.totalWeight == pytest.approx(ow, rel=1e-12)
    assert e <= TOL
