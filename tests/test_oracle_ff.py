"""The far-field (FFAntenna, emitter.h:226-291) restatement of the oracle on the CPU:
the monostatic dihedral sweep is symmetric about 45 degrees (the reflector is symmetric
under x <-> z), strongest at 45 degrees, peaks at the round-trip range of the disk
planes, and its FP32 run agrees with the FP64 one on the same samples."""
import numpy as np
import pytest

from hussar_gb300 import FFAntenna, PathTracer, scenes


@pytest.fixture(scope="module")
def sweep(oracle_lib):
    w = scenes.dihedral_ff_workload(poses=5, samples_per_pose=1 << 14)
    t = PathTracer()
    t.doGuiding = False
    t.maxDepth = 2
    ora = oracle_lib.Scene(w.mesh)
    rows32 = [ora.fetch_row_ff(w.rf, 256, w.tx[k], w.rx[k], t, 1 << 14, precision=32) for k in range(5)]
    rows65 = [ora.fetch_row_ff(w.rf, 256, w.tx[k], w.rx[k], t, 1 << 14, precision=65) for k in range(5)]
    return w, np.array(rows32), np.array(rows65)


def test_far_field_sweep_symmetric_and_peaked(sweep):
    w, rows, _ = sweep
    mag = np.linalg.norm(rows, axis=1)
    assert mag[2] == mag.max()
    for k in range(2):
        assert abs(mag[k] - mag[4 - k]) <= 0.02 * mag[k]
    # peak bin: round trip between the disk planes, 0.1 m from the reflector's centre
    assert 4 <= int(np.argmax(np.abs(rows[2]))) <= 8


def test_far_field_fp32_matches_fp64(sweep):
    _, r32, r65 = sweep
    for k in range(5):
        assert np.linalg.norm(r32[k] - r65[k]) / np.linalg.norm(r65[k]) <= 1e-3


def test_far_field_antenna_checks():
    with pytest.raises(ValueError):
        FFAntenna([1, 1, 0], [0, 1, 0], [0, 0, 0], 1.0)  # not normalised
    with pytest.raises(ValueError):
        FFAntenna([1, 0, 0], [1, 0, 0], [0, 0, 0], 1.0)  # H along the direction
    with pytest.raises(ValueError):
        FFAntenna([1, 0, 0], [0, 1, 0], [0, 0, 0], 0.0)
