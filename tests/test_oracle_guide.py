"""The oracle's restatement of the guiding tree (GuidingWrapper, path.h:17-131, over the
product's 2-D tree) checked on the CPU: the mixture density, the warp, the step's build
and refinement, and PathTracer::run's guided schedule (path.h:171-224)."""
import numpy as np
import pytest

from oracle import pyoracle


def tree_density(st, y0, y1):
    """The sampling tree's density at y relative to uniform, by descent (numpy float32)."""
    pdf, node, depth = np.float32(1), 0, 0
    lo, half = [np.float32(0), np.float32(0)], [np.float32(1), np.float32(1)]
    y = [np.float32(y0), np.float32(y1)]
    while depth < 24 and st.samp_child[node] >= 0:
        ax = depth & 1
        half[ax] = half[ax] * np.float32(0.5)
        p = st.samp_p[node]
        if y[ax] < lo[ax] + half[ax]:
            pdf = pdf * (np.float32(2) * p)
            node = st.samp_child[node]
        else:
            pdf = pdf * (np.float32(2) * (np.float32(1) - p))
            lo[ax] = lo[ax] + half[ax]
            node = st.samp_child[node] + 1
        depth += 1
    return float(pdf)


def trained_state():
    """A tree stepped twice from second-moment sums concentrated near (0.8, 0.3)."""
    g = pyoracle.Guide()
    for _ in range(2):
        st = g.get()
        rng = np.random.default_rng(1)
        for n in st.reachable("train"):
            if st.train_child[n] < 0:
                st.acc2[n] = np.float32(rng.uniform(0.0, 1e-3))
        # the leaf holding (0.8, 0.3) carries most of the energy
        node, depth, lo, half = 0, 0, [0.0, 0.0], [1.0, 1.0]
        while st.train_child[node] >= 0:
            ax = depth & 1
            half[ax] *= 0.5
            x = (0.8, 0.3)[ax]
            if x < lo[ax] + half[ax]:
                node = st.train_child[node]
            else:
                lo[ax] += half[ax]
                node = st.train_child[node] + 1
            depth += 1
        st.acc2[node] = np.float32(5.0)
        g.set(st)
        g.step()
    return g


def test_root_tree_is_the_uniform_mixture():
    g = pyoracle.Guide()
    y0, y1, pdf = g.sample(0.55, 0.25)
    assert pdf == pytest.approx(1.0, abs=1e-6)
    assert y0 == pytest.approx((0.55 - 0.1) / 0.9, rel=1e-6) and y1 == pytest.approx(0.25)
    y0, y1, pdf = g.sample(0.05, 0.25)  # the uniform branch rescales x0 only
    assert y0 == pytest.approx(0.5, rel=1e-6) and y1 == pytest.approx(0.25)


def test_step_builds_and_refines():
    g = trained_state()
    st = g.get()
    assert st.count > 9
    # links stay inside the arrays and point past their node
    for n in st.reachable("train"):
        c = st.train_child[n]
        assert c == -1 or n < c < pyoracle.GUIDE_NODES - 1
    # the sampling tree's first-child probabilities are energy shares in [0, 1]
    inner = [n for n in st.reachable("samp") if st.samp_child[n] >= 0]
    assert inner and all(0.0 <= st.samp_p[n] <= 1.0 for n in inner)
    # the statistics restart
    assert not st.acc2.any()
    # the region around (0.8, 0.3) is sampled more densely than uniform
    assert tree_density(st, 0.8, 0.3) > 4.0
    assert tree_density(st, 0.1, 0.9) < 1.0


def test_warp_reports_the_mixture_density_of_its_output():
    g = trained_state()
    st = g.get()
    rng = np.random.default_rng(2)
    for x0, x1 in rng.random((400, 2)):
        y0, y1, pdf = g.sample(x0, x1)
        assert 0.0 <= y0 < 1.0 and 0.0 <= y1 < 1.0
        if x0 >= 0.1:  # the tree branch: pdf = 0.9 * tree density at the warped point + 0.1
            want = 0.9 * tree_density(st, y0, y1) + 0.1
            assert pdf == pytest.approx(want, rel=1e-5)


def test_tree_density_integrates_to_one():
    st = trained_state().get()
    n = 256
    grid = (np.arange(n) + 0.5) / n
    mean = np.mean([tree_density(st, a, b) for a in grid[::4] for b in grid])
    assert mean == pytest.approx(1.0, rel=2e-3)


def test_set_rejects_bad_count():
    g = pyoracle.Guide()
    st = g.get()
    st.count = 0
    with pytest.raises(ValueError):
        g.set(st)


@pytest.mark.parametrize("samples", [1000, 16384, 40000, 1 << 17])
def test_guided_schedule_total_weight(samples):
    """The oracle's PathTracer::run: total weight of the last (cleared) iteration."""
    from hussar_gb300 import PathTracer, scenes
    w = scenes.dihedral_workload(poses=3)
    t = PathTracer()
    t.maxDepth = w.max_depth
    t.doGuiding = True
    ora = pyoracle.Scene(w.mesh)
    fr, tw = pyoracle.Guide().path_tracer_run(ora, w.rf, w.frame, w.tx[1], w.rx[1], t, samples)
    milestone, remaining, last = 16384, samples, 0
    while True:
        milestone = min(milestone, remaining)
        last = milestone
        remaining -= milestone
        if remaining == 0:
            break
        milestone *= 2
        if remaining < milestone * 2:
            milestone = remaining
    assert tw == last
    assert np.isfinite(fr).all() and np.abs(fr).sum() > 0
