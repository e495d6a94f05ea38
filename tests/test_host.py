"""Host-side API mirrors: mesh building order, antenna checks, frames, workloads."""
import numpy as np
import pytest

from hussar_gb300 import Frame, FrameConfig, NFAntenna, PathTracer, RFConfig, TriangleMesh, scenes


def test_add_quad_vertex_order():
    m = TriangleMesh()
    m.addQuad([1, 2, 3], [1, 0, 0], [0, 1, 0])  # mesh.h:30-40
    assert np.array_equal(m.vertexBuffer, np.array([[1, 2, 3], [2, 2, 3], [2, 3, 3], [1, 3, 3]], np.float32))
    assert np.array_equal(m.indexBuffer, np.array([[0, 1, 2], [0, 2, 3]]))


def test_add_box_twelve_triangles_closed():
    m = TriangleMesh()
    m.addBox([0, 0, 0], [1, 2, 3])
    v, f = m.vertexBuffer, m.indexBuffer
    assert len(f) == 12 and len(v) == 24
    assert v.min(0).tolist() == [0, 0, 0] and v.max(0).tolist() == [1, 2, 3]
    # every face lies on a box face: each triangle's vertices share one coordinate at a bound
    for t in f:
        p = v[t]
        assert any(np.all(p[:, a] == p[0, a]) and p[0, a] in (0, [1, 2, 3][a]) for a in range(3))


def test_vectorised_boxes_match_addbox():
    mesh = scenes.boxes_mesh(seed=7, count=5)
    ref = TriangleMesh()
    rng = np.random.default_rng(7)
    size = rng.uniform(0.2, 5.0, (5, 3))
    pos = rng.uniform(-50, 50, (5, 2))
    for k in range(5):
        mn64 = np.array([pos[k, 0], 0, pos[k, 1]], np.float64)
        ref.addBox(mn64.astype(np.float32), (mn64 + size[k]).astype(np.float32))
    ref.addQuad([-50, 0, -50], [100, 0, 0], [0, 0, 100])
    assert np.array_equal(mesh.indexBuffer, ref.indexBuffer)
    assert np.array_equal(mesh.vertexBuffer, ref.vertexBuffer)


def test_icosphere_counts_and_radius():
    v, f = scenes.icosphere(3, 0.5, (0, 0.5, 0))
    assert len(f) == 20 * 4 ** 3
    r = np.linalg.norm(v - np.array([0, 0.5, 0], np.float32), axis=1)
    assert np.allclose(r, 0.5, atol=1e-6)
    w = scenes.sphere_ground_workload(samples=16, level=6)
    assert w.mesh.triangleCount() == 81922


def test_antenna_rejects_non_rotation():
    with pytest.raises(ValueError):
        NFAntenna([0, 0, 0], np.diag([1.0, 1.0, 2.0]))
    a = NFAntenna([0, 0, 0], scenes.looking(0.3))
    assert abs(np.linalg.det(a.rotation().astype(np.float64)) - 1) < 1e-5


def test_looking_boresight():
    for yaw in (0.0, 0.7, 2.0):
        R = scenes.looking(yaw)
        assert np.allclose(R[:, 2], [-np.cos(yaw), 0, -np.sin(yaw)], atol=1e-6)


def test_pathtracer_defaults_and_frame():
    t = PathTracer()
    assert t.maxDepth == 10 and t.doGuiding and t.onlyIndirect and t.filteringRadius == 160
    t.configureFrame(FrameConfig(2, 8, 3))
    assert t.frame.data.shape == (2, 8, 3) and t.frame.sampleCount() == 48
    t.frame.data[0, 3, 0] = 2 + 4j
    t.totalWeight = 4.0
    f = t.fetchFrame()
    assert f.data[0, 3, 0] == np.complex64(0.5 + 1j)
    assert f.argmax() == (0, 3, 0)


def test_rf_bandwidth_float():
    rf, fc = scenes.rf_77ghz()
    assert rf.bandwidth() == float(np.float32(rf.freqSlope) * np.float32(rf.rampTime))
    assert fc.samplesPerChirp == 256
