"""The urban MIMO configuration: ~5 M triangles of building and car boxes, one sensor on a
street with a 3 TX x 4 RX array at half-wavelength spacing (12 virtual channels, each a
(TX, RX) pose of one batch), up to 5 bounces. The plain (unguided) FP32 path of every
channel against the oracle at 1e-4 relative L2, at a budget capped so the CPU oracle
finishes in seconds."""
import numpy as np
import pytest

from hussar_gb300 import PathTracer, gb300, scenes

pytestmark = pytest.mark.gpu

BUDGET = 1 << 18


def rel_l2(a, b):
    a = np.asarray(a, np.complex128)
    b = np.asarray(b, np.complex128)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.fixture(scope="module")
def urban(product_lib, oracle_lib):
    w = scenes.urban_mimo_workload(samples=BUDGET)
    return w, gb300.Backend(w.mesh, None), oracle_lib.Scene(w.mesh)


def test_urban_mimo_channels_match_oracle(urban):
    w, be, ora = urban
    t = PathTracer()
    t.doGuiding = False
    t.maxDepth = w.max_depth
    N = w.frame.samplesPerChirp
    rows = be.simulate_batch(w.rf, N, t, w.tx, w.rx, w.budget)
    assert rows.shape == (12, N)
    errs = []
    for k in range(len(w.tx)):
        ref = ora.fetch_row(w.rf, N, w.tx[k], w.rx[k], t, int(w.budget[k]))
        assert np.linalg.norm(ref) > 0, k
        errs.append(rel_l2(rows[k], ref))
    print("urban MIMO 12 channels at 2^18: max rel L2 %.2e" % max(errs))
    assert max(errs) <= 1e-4, errs
    # virtual channels half a wavelength apart see the scene with different phases
    assert rel_l2(rows[0], rows[-1]) > 0.05


def test_urban_mimo_radar_cube(urban):
    """hsr_simulate_frame: the 3 TX x 4 RX array's radar cube [128 chirps][256 samples][12
    channels] in one call: channel c pairs TX c // 4 with RX c % 4 and equals that pose's
    batch row (the same samples), the static scene's energy sits in chirp 0 (Doppler bin
    0) and every other chirp is zero."""
    w, be, _ = urban
    t = PathTracer()
    t.doGuiding = False
    t.maxDepth = w.max_depth
    N = w.frame.samplesPerChirp
    cube = be.simulate_frame(w.rf, w.frame, t, w.tx_array, w.rx_array, BUDGET)
    assert cube.shape == (128, N, 12)
    rows = be.simulate_batch(w.rf, N, t, w.tx, w.rx, w.budget)
    for c in range(12):
        assert rel_l2(cube[0, :, c], rows[c]) <= 1e-5, c
    assert np.count_nonzero(cube[1:]) == 0
