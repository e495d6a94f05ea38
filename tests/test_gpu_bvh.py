"""The device BVH as built on the GPU (PLOC and LBVH topologies, with and without the
insertion passes that follow the build).

Structure: a binary tree over all triangles, root 0, stored depth first; every stored
node is reachable from the root exactly once and the leaves (one to eight triangles in
consecutive slots) hold every triangle slot exactly once. Conservativeness: each stored child box
contains the padded bounding box of every triangle beneath it, with the padding the build
applies (max|x| * 4e-6 + 1e-6 per axis), so the FP32 slab test cannot reject a box that a
hit lies in."""
import numpy as np
import pytest

from hussar_gb300 import TriangleMesh, gb300, scenes
from hussar_gb300.core import child_boxes

pytestmark = pytest.mark.gpu


def padded_boxes(mesh, tris):
    """Padded boxes of the triangles in slot order, from the mesh's own vertices (the
    records carry the original primitive id in v0.w)."""
    prim = tris[:, 3].copy().view(np.int32)
    v = np.asarray(mesh.vertexBuffer, np.float32)[np.asarray(mesh.indexBuffer)[prim]]  # [n, 3, 3]
    v0, v1, v2 = v[:, 0], v[:, 1], v[:, 2]
    mn = np.minimum(v0, np.minimum(v1, v2))
    mx = np.maximum(v0, np.maximum(v1, v2))
    # the build may round m * 4e-6 + 1e-6 once (fused) or twice: check against the smaller pad
    m = np.maximum(np.abs(mn), np.abs(mx))
    pad2 = (m * np.float32(4e-6)).astype(np.float32) + np.float32(1e-6)
    pad1 = (m.astype(np.float64) * np.float64(np.float32(4e-6)) + np.float64(np.float32(1e-6))).astype(np.float32)
    pad = np.minimum(pad1, pad2).astype(np.float32)
    return mn - pad, mx + pad


def leaf_slots(ref):
    """Slots of a leaf reference (child < 0): ((~c) & 7) + 1 triangles from (~c) >> 3."""
    r = ~int(ref)
    return range(r >> 3, (r >> 3) + (r & 7) + 1)


def check_tree(be, mesh):
    nt = mesh.triangleCount()
    nodes, tris = be.device_bvh()
    assert len(tris) == nt and 1 <= len(nodes) <= nt - 1
    child = nodes["child"]
    lo, hi = child_boxes(nodes)
    tlo, thi = padded_boxes(mesh, tris)
    # the nodes reachable from the root (pre-order), then subtree boxes bottom-up
    order, stack, seen_slots = [], [0], []
    while stack:
        i = stack.pop()
        order.append(i)
        for c in child[i]:
            if c >= 0:
                stack.append(int(c))
            else:
                seen_slots.extend(leaf_slots(c))
    # every stored node reachable once (depth-first layout: a node's first child, when
    # internal, is the next node), every triangle slot in exactly one leaf
    assert len(set(order)) == len(order) == len(nodes)
    first = child[:, 0]
    assert np.array_equal(first[first >= 0], np.nonzero(first >= 0)[0] + 1)
    assert np.array_equal(np.sort(np.array(seen_slots)), np.arange(nt))
    sub_lo = np.zeros((nt - 1, 3), np.float32)
    sub_hi = np.zeros((nt - 1, 3), np.float32)
    for i in reversed(order):
        blo, bhi = [], []
        for k in range(2):
            c = int(child[i, k])
            if c >= 0:
                cl, ch = sub_lo[c], sub_hi[c]
            else:
                sl = list(leaf_slots(c))
                cl, ch = tlo[sl].min(0), thi[sl].max(0)
            assert (lo[i, k] <= cl).all() and (hi[i, k] >= ch).all(), (i, k)
            blo.append(cl)
            bhi.append(ch)
        sub_lo[i] = np.minimum(blo[0], blo[1])
        sub_hi[i] = np.maximum(bhi[0], bhi[1])
    leaves = [c for i in order for c in child[i] if c < 0]
    return nodes, len(order), len(leaves)


@pytest.mark.parametrize("passes", [0, 32], ids=["built", "reinserted"])
@pytest.mark.parametrize("leaf", [1, 4, 8])
@pytest.mark.parametrize("builder", [0, 1], ids=["ploc", "lbvh"])
def test_device_bvh_contains_padded_triangles(product_lib, builder, leaf, passes):
    """Each topology as built and after the insertion passes (hsr_set_bvh_optimize)."""
    product_lib.hsr_set_bvh_builder(builder)
    product_lib.hsr_set_bvh_leaf_size(leaf)
    product_lib.hsr_set_bvh_optimize(passes)
    try:
        for mesh in (scenes.dihedral_mesh(), scenes.sphere_ground_workload(level=3).mesh,
                     scenes.boxes_mesh(seed=3, count=2000)):
            be = gb300.Backend(mesh, None)
            _, inner, leaves = check_tree(be, mesh)
            print(mesh.triangleCount(), "triangles, depth", be.bvh_stats()["max_depth"], "reachable nodes", inner,
                  "leaves", leaves)
            if leaf == 1:
                assert leaves == mesh.triangleCount()
    finally:
        product_lib.hsr_set_bvh_builder(0)
        product_lib.hsr_set_bvh_leaf_size(4)
        product_lib.hsr_set_bvh_optimize(32)


@pytest.mark.parametrize("leaf", [1, 8])
def test_ray_queries_do_not_depend_on_leaf_size(product_lib, leaf):
    """The same queries against trees with leaves of one triangle, of up to four (the
    default) and up to eight: bit-identical answers."""
    mesh = scenes.boxes_mesh(seed=4, count=3000)
    rng = np.random.default_rng(7)
    v = np.asarray(mesh.vertexBuffer, np.float32)
    o = rng.uniform(v.min(0), v.max(0), (20000, 3)).astype(np.float32)
    d = rng.normal(size=(20000, 3))
    d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    ref = gb300.Backend(mesh, None).intersect(o, d)
    product_lib.hsr_set_bvh_leaf_size(leaf)
    try:
        got = gb300.Backend(mesh, None).intersect(o, d)
    finally:
        product_lib.hsr_set_bvh_leaf_size(4)
    for a, b in zip(got, ref):
        assert np.array_equal(np.asarray(a).view(np.uint8), np.asarray(b).view(np.uint8))


def test_single_triangle_scene(product_lib):
    m = TriangleMesh()
    m.append(np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32), np.array([[0, 1, 2]], np.int32))
    be = gb300.Backend(m, None)
    st = be.bvh_stats()
    assert st["leaves"] == 1 and st["nodes"] == 1
    t, p, n, prim = be.intersect(np.array([[0.2, 0.2, 1.0]], np.float32), np.array([[0, 0, -1.0]], np.float32))
    assert prim[0] == 0 and t[0] == np.float32(1.0)


@pytest.mark.parametrize("nt", [4, 5, 9, 33])
def test_insertion_passes_on_small_and_degenerate_scenes(product_lib, nt):
    """Trees of a handful of triangles, and a scene of repeated, zero-area and far-away
    triangles: after the insertion passes the tree is complete and conservative, and ray
    queries answer as on the tree as built."""
    rng = np.random.default_rng(nt)
    if nt == 33:
        tri = np.repeat(rng.uniform(-1, 1, (1, 3, 3)), 12, axis=0)            # 12 copies of one triangle
        flat = rng.uniform(-1, 1, (12, 1, 3)) * np.array([[[1.0], [0.5], [0.25]]])  # collinear: zero area
        far = rng.uniform(-1, 1, (9, 3, 3)) + np.array([1e4, 0, -3e3])         # far from the rest
        tri = np.concatenate([tri, flat, far]).astype(np.float32)
    else:
        tri = rng.uniform(-1, 1, (nt, 3, 3)).astype(np.float32)
    mesh = TriangleMesh()
    mesh.append(tri.reshape(-1, 3), np.arange(3 * nt, dtype=np.int32).reshape(-1, 3))
    o = rng.uniform(-2, 2, (4000, 3)).astype(np.float32)
    d = rng.normal(size=(4000, 3))
    d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    res = {}
    try:
        for passes in (0, 32):
            product_lib.hsr_set_bvh_optimize(passes)
            be = gb300.Backend(mesh, None)
            check_tree(be, mesh)
            res[passes] = be.intersect(o, d)
    finally:
        product_lib.hsr_set_bvh_optimize(32)
    for a, b in zip(res[0], res[32]):
        assert np.array_equal(np.asarray(a).view(np.uint8), np.asarray(b).view(np.uint8))
