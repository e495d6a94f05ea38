"""The device traversal code on the CPU: hussar_gb300/csrc/hsr_traverse.cuh compiled with
g++ through host definitions of the CUDA intrinsics (tests/native/host_shim.h), over a
binary tree in the kernels' node layout (leaves of one or several triangles); every
closest-hit and any-hit answer is compared
with brute force over all triangles (same triangle test and tie rule). Catches traversal
logic errors without a GPU."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from hussar_gb300 import scenes

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CUDA_INC = "/usr/local/cuda/include"


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    if not os.path.exists(os.path.join(CUDA_INC, "cuda_runtime.h")) or shutil.which("g++") is None:
        pytest.skip("needs g++ and the CUDA headers")
    exe = str(tmp_path_factory.mktemp("trav") / "bvh_traverse_check")
    subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-I", os.path.join(ROOT, "tests", "native"),
                    "-I", os.path.join(ROOT, "hussar_gb300", "csrc"), "-I", CUDA_INC, "-I",
                    os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "native", "bvh_traverse_check.cpp"),
                    "-o", exe], check=True)
    return exe


def run(checker, tmp_path, mesh, rays, seed, leaf=1):
    rng = np.random.default_rng(seed)
    v = np.asarray(mesh.vertexBuffer, np.float32)
    f = np.asarray(mesh.indexBuffer, np.int32)
    lo, hi = v.min(0), v.max(0)
    span = hi - lo
    o = rng.uniform(lo - 0.1 * span, hi + 0.1 * span, (rays, 3)).astype(np.float32)
    d = rng.normal(size=(rays, 3))
    # a third of the rays are parallel to one or two axes (exact zero components)
    third = rays // 3
    d[:third, 0] = 0.0
    d[third // 2:third, 2] = 0.0
    d[third:third + third // 4] = [[0, -1, 0]]
    d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    tf = rng.uniform(0, 2 * np.linalg.norm(span), rays).astype(np.float32)
    path = tmp_path / ("in%d.bin" % seed)
    with open(path, "wb") as fh:
        fh.write(np.array([len(v), len(f), rays], np.int64).tobytes())
        for a in (v, f, o, d, tf):
            fh.write(np.ascontiguousarray(a).tobytes())
    out = subprocess.run([checker, str(path), str(leaf)], check=True, capture_output=True,
                         text=True).stdout.split()
    res = {out[i]: float(out[i + 1]) for i in range(0, len(out), 2)}
    print(res)
    return res


@pytest.mark.parametrize("leaf", [1, 3, 8])
@pytest.mark.parametrize("name", ["dihedral", "sphere", "boxes"])
def test_traversal_matches_brute_force(checker, tmp_path, name, leaf):
    """Leaves of one triangle and of several (consecutive slots, the leaf reference's
    count in its low three bits)."""
    mesh = {"dihedral": lambda: scenes.dihedral_mesh(),
            "sphere": lambda: scenes.sphere_ground_workload(level=3).mesh,
            "boxes": lambda: scenes.boxes_mesh(seed=5, count=400, extent=30.0)}[name]()
    res = run(checker, tmp_path, mesh, 3000, seed=len(name), leaf=leaf)
    assert res["closest_mismatch"] == 0 and res["any_mismatch"] == 0
    assert res["stack_status"] == 0


def far_rays(checker, tmp_path, mesh, rays, seed, distance, offset=0.0):
    """Rays from a sphere of `distance` around the scene's centre aimed at random points of
    the scene (the far-field disk of the RCS runs): the quantised boxes' margin and the
    exit-distance slack must hold for origins far outside the grid."""
    rng = np.random.default_rng(seed)
    v = np.asarray(mesh.vertexBuffer, np.float32) + np.float32(offset)
    m = type(mesh)()
    m.append(v, np.asarray(mesh.indexBuffer, np.int32).reshape(-1, 3))
    lo, hi = v.min(0), v.max(0)
    c = 0.5 * (lo + hi)
    u = rng.normal(size=(rays, 3))
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    o = (c + distance * u).astype(np.float32)
    target = rng.uniform(lo, hi, (rays, 3))
    d = target - o
    d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    tf = np.full(rays, 2 * distance, np.float32)
    path = tmp_path / ("far%d.bin" % seed)
    with open(path, "wb") as fh:
        fh.write(np.array([len(v), len(m.indexBuffer), rays], np.int64).tobytes())
        for a in (v, np.asarray(m.indexBuffer, np.int32), o, d, tf):
            fh.write(np.ascontiguousarray(a).tobytes())
    out = subprocess.run([checker, str(path), "4"], check=True, capture_output=True, text=True).stdout.split()
    return {out[i]: float(out[i + 1]) for i in range(0, len(out), 2)}


@pytest.mark.parametrize("distance,offset", [(20.0, 0.0), (200.0, 0.0), (5.0, 1e4)])
@pytest.mark.parametrize("name", ["dihedral", "icosphere"])
def test_far_and_offset_rays_match_brute_force(checker, tmp_path, name, distance, offset):
    """A 10 cm dihedral and a 10 cm icosphere of 1280 triangles seen from 20 m and 200 m
    (200 and 2000 scene extents), and from 5 m with the scene 10 km from the coordinate
    origin."""
    if name == "dihedral":
        mesh = scenes.dihedral_mesh()
    else:
        from hussar_gb300 import TriangleMesh
        v, f = scenes.icosphere(3, radius=0.05)
        mesh = TriangleMesh()
        mesh.append(v, f)
    res = far_rays(checker, tmp_path, mesh, 4000, 11, distance, offset)
    print(res)
    assert res["closest_mismatch"] == 0 and res["any_mismatch"] == 0
