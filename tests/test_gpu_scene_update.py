"""Scene changes for resident scenes: hsr_scene_refit (new vertex positions, the BVH's
boxes refitted over its tree) and hsr_scene_rebuild (a new mesh under the same handle).
Ray-query answers do not depend on the tree, so a refitted or rebuilt scene must answer
bit for bit as a scene freshly created from the same mesh, and its frames must match the
oracle's as the plain path's do."""
import numpy as np
import pytest

from hussar_gb300 import PathTracer, TriangleMesh, gb300, scenes

pytestmark = pytest.mark.gpu


def rays(mesh, n, seed):
    rng = np.random.default_rng(seed)
    v = np.asarray(mesh.vertexBuffer, np.float32)
    o = rng.uniform(v.min(0), v.max(0), (n, 3)).astype(np.float32)
    d = rng.normal(size=(n, 3))
    return o, (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)


def moved(mesh, seed, scale=0.3):
    """The same triangles with every box shifted and stretched (vertices of one box move
    together, so the triangles stay valid)."""
    rng = np.random.default_rng(seed)
    v = np.asarray(mesh.vertexBuffer, np.float32).copy()
    box = np.arange(len(v)) // 24  # addBox: six quads of four vertices
    shift = rng.normal(scale=scale, size=(box.max() + 1, 3)).astype(np.float32)
    v = v + shift[box]
    return TriangleMesh(v, np.asarray(mesh.indexBuffer, np.int32))


def same_answers(a, b, o, d):
    ra, rb = a.intersect(o, d), b.intersect(o, d)
    for x, y in zip(ra, rb):
        assert np.array_equal(np.asarray(x).view(np.uint8), np.asarray(y).view(np.uint8))
    tf = np.full(len(o), 5.0, np.float32)
    assert np.array_equal(a.visible(o, d, tf), b.visible(o, d, tf))


def test_refit_answers_as_a_fresh_scene(product_lib):
    mesh = scenes.boxes_mesh(seed=6, count=3000, extent=40.0)
    be = gb300.Backend(mesh, None)
    for k in range(3):
        m2 = moved(mesh, 100 + k)
        be.refit(m2)
        o, d = rays(m2, 20000, k)
        same_answers(be, gb300.Backend(m2, None), o, d)
    st = be.bvh_stats()
    assert st["leaves"] == mesh.triangleCount()


def test_refit_frames_match_the_oracle(product_lib):
    from oracle import pyoracle
    w = scenes.dihedral_workload(poses=5)
    be = gb300.Backend(w.mesh, None)
    # the dihedral rotated by 20 degrees about y and lifted 5 cm
    c, s = np.cos(np.deg2rad(20.0)), np.sin(np.deg2rad(20.0))
    R = np.array([[c, 0, s], [0, 1, 0], [-s, 0, c]], np.float32)
    v = (np.asarray(w.mesh.vertexBuffer, np.float32) @ R.T + np.float32([0, 0.05, 0])).astype(np.float32)
    m2 = TriangleMesh(v, np.asarray(w.mesh.indexBuffer, np.int32))
    be.refit(m2)
    t = PathTracer()
    t.doGuiding = False
    t.maxDepth = w.max_depth
    rows = be.simulate_batch(w.rf, 256, t, w.tx, w.rx, np.full(len(w.tx), 1 << 16, np.int64))
    ora = pyoracle.Scene(m2)
    for k in range(len(w.tx)):
        ref = ora.fetch_row(w.rf, 256, w.tx[k], w.rx[k], t, 1 << 16)
        err = np.linalg.norm(rows[k] - ref) / np.linalg.norm(ref)
        assert err <= 1e-4, (k, err)


def test_rebuild_swaps_the_mesh_under_the_handle(product_lib):
    be = gb300.Backend(scenes.dihedral_mesh(), None)
    m2 = scenes.boxes_mesh(seed=8, count=500, extent=20.0)
    be.rebuild(m2)
    o, d = rays(m2, 10000, 3)
    same_answers(be, gb300.Backend(m2, None), o, d)
    assert be.bvh_stats()["leaves"] == m2.triangleCount()
    # and back to a one-triangle scene, then a refit of it
    one = TriangleMesh(np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32), np.array([[0, 1, 2]], np.int32))
    be.rebuild(one)
    be.refit(TriangleMesh(np.array([[0, 0, 1], [1, 0, 1], [0, 1, 1]], np.float32), np.array([[0, 1, 2]], np.int32)))
    t, p, n, prim = be.intersect(np.array([[0.2, 0.2, 3.0]], np.float32), np.array([[0, 0, -1.0]], np.float32))
    assert prim[0] == 0 and t[0] == np.float32(2.0)


def test_refit_rejects_a_different_vertex_count(product_lib):
    from hussar_gb300 import _lib
    be = gb300.Backend(scenes.dihedral_mesh(), None)
    v = np.zeros((3, 3), np.float32)
    assert _lib.lib().hsr_scene_refit(be.handle, _lib.ptr(v), 3) == _lib.HSR_ERR_INVALID_ARGUMENT
    bad = np.asarray(scenes.dihedral_mesh().vertexBuffer, np.float32).copy()
    bad[0, 0] = np.nan
    assert _lib.lib().hsr_scene_refit(be.handle, _lib.ptr(bad), len(bad)) == _lib.HSR_ERR_INVALID_ARGUMENT


def test_rebuild_refused_while_a_graph_holds_the_scene(product_lib):
    """A captured graph keeps the BVH's device pointers: rebuild waits for it to go."""
    torch = pytest.importorskip("torch")
    from hussar_gb300 import _lib
    dev = torch.device("cuda", 0)
    w = scenes.dihedral_workload(poses=2)
    be = gb300.Backend(w.mesh, None)
    t = PathTracer()
    t.doGuiding = False
    t.maxDepth = w.max_depth
    P, N = 2, 256
    tx = (_lib.AntennaC * P)(*[a.to_c() for a in w.tx])
    rx = (_lib.AntennaC * P)(*[a.to_c() for a in w.rx])
    d_tx = torch.frombuffer(bytearray(bytes(tx)), dtype=torch.uint8).to(dev)
    d_rx = torch.frombuffer(bytearray(bytes(rx)), dtype=torch.uint8).to(dev)
    d_b = torch.full((P,), 1 << 10, dtype=torch.int64, device=dev)
    d_o = torch.zeros(P, dtype=torch.int64, device=dev)
    d_out = torch.zeros(2 * P * N, dtype=torch.float32, device=dev)
    g = be.batch_graph(w.rf, N, t, P, d_tx.data_ptr(), d_rx.data_ptr(), d_b.data_ptr(), d_o.data_ptr(),
                       d_out.data_ptr())
    m2 = scenes.boxes_mesh(seed=9, count=50, extent=5.0)
    v = np.ascontiguousarray(m2.vertexBuffer, np.float32)
    i = np.ascontiguousarray(m2.indexBuffer, np.int32)
    assert _lib.lib().hsr_scene_rebuild(be.handle, _lib.ptr(v), len(v), _lib.ptr(i), len(i)) == \
        _lib.HSR_ERR_INVALID_ARGUMENT
    g.close()
    be.rebuild(m2)
    assert be.bvh_stats()["leaves"] == m2.triangleCount()
