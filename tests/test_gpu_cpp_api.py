"""The C++ drop-in (include/hussar/gb300.h + gb300_types.h): the reference's example
flow compiled with g++ against libhsr_gb300.so gives the same frames as the Python
binding and the oracle, and so does the C++ serving wrapper with several client
threads submitting at once."""
import os
import subprocess

import numpy as np
import pytest

from hussar_gb300 import NFAntenna, PathTracer, gb300, scenes

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def compile_example(name, out_dir):
    out = str(out_dir / name)
    libdir = os.path.join(ROOT, "hussar_gb300")
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-pthread", "-I", os.path.join(ROOT, "include"),
                           os.path.join(ROOT, "tests", "cpp", name + ".cpp"), "-L", libdir, "-lhsr_gb300",
                           "-Wl,-rpath," + libdir, "-o", out])
    return out


@pytest.fixture(scope="module")
def example_bin(product_lib, tmp_path_factory):
    return compile_example("dihedral_example", tmp_path_factory.mktemp("cpp"))


@pytest.fixture(scope="module")
def serve_bin(product_lib, tmp_path_factory):
    return compile_example("serve_example", tmp_path_factory.mktemp("cpp"))


def test_cpp_example_matches_python_and_oracle(example_bin, tmp_path, oracle_lib):
    poses, samples = 7, 1 << 16
    sim = str(tmp_path / "dihedral.SIM")
    subprocess.check_call([example_bin, sim, str(poses), str(samples)])
    frames = np.fromfile(sim, np.complex64).reshape(poses, 256)
    pose = np.fromfile(sim + ".poses", np.float32).reshape(poses, 12)
    w = scenes.dihedral_workload(poses=poses, samples_per_pose=samples)
    # the exact antenna poses the C++ program used
    w.tx = [NFAntenna(p[:3], p[3:].reshape(3, 3)) for p in pose]
    w.rx = w.tx
    t = PathTracer()
    t.doGuiding = False
    t.maxDepth = 2
    be = gb300.Backend(w.mesh, None)
    rows = be.simulate_batch(w.rf, 256, t, w.tx, w.rx, w.budget)
    ora = oracle_lib.Scene(w.mesh)
    for k in range(poses):
        ref = ora.fetch_row(w.rf, 256, w.tx[k], w.rx[k], t, samples)
        if np.linalg.norm(ref) == 0:
            assert np.linalg.norm(frames[k]) == 0
            continue
        assert np.linalg.norm(frames[k] - ref) / np.linalg.norm(ref) <= 1e-4
        assert np.linalg.norm(frames[k] - rows[k]) / np.linalg.norm(rows[k]) <= 1e-5


def test_cpp_server_matches_batch_and_oracle(serve_bin, tmp_path, oracle_lib):
    poses, samples, threads = 24, 1 << 16, 4
    sim = str(tmp_path / "served.SIM")
    out = subprocess.check_output([serve_bin, sim, str(poses), str(samples), str(threads)], text=True)
    print(out)
    rows = np.fromfile(sim, np.complex64).reshape(poses, 256)
    pose = np.fromfile(sim + ".poses", np.float32).reshape(poses, 12)
    w = scenes.dihedral_workload(poses=poses, samples_per_pose=samples)
    w.tx = [NFAntenna(p[:3], p[3:].reshape(3, 3)) for p in pose]
    w.rx = w.tx
    t = PathTracer()
    t.doGuiding = False
    t.maxDepth = 2
    be = gb300.Backend(w.mesh, None)
    batch = be.simulate_batch(w.rf, 256, t, w.tx, w.rx, w.budget)
    ora = oracle_lib.Scene(w.mesh)
    for k in range(0, poses, 5):
        ref = ora.fetch_row(w.rf, 256, w.tx[k], w.rx[k], t, samples)
        if np.linalg.norm(ref) > 0:
            assert np.linalg.norm(rows[k] - ref) / np.linalg.norm(ref) <= 1e-4, k
    for k in range(poses):
        if np.linalg.norm(batch[k]) == 0:
            assert np.linalg.norm(rows[k]) == 0, k
        else:
            # the same Halton samples; only the FP64 summation order differs
            assert np.linalg.norm(rows[k] - batch[k]) / np.linalg.norm(batch[k]) <= 1e-5, k


@pytest.fixture(scope="module")
def guided_bin(product_lib, tmp_path_factory):
    return compile_example("guided_example", tmp_path_factory.mktemp("cpp"))


def test_cpp_guided_schedule(guided_bin, tmp_path):
    """doGuiding = true (the reference's default) through the C++ drop-in: the mirror
    PathTracer::run calls Backend::run per doubling iteration and the backend guides each
    with its device tree. The frames equal the C ABI's own guided schedule
    (hsr_path_tracer_run, the same samples and tree procedure) up to the order of the
    float training sums, and both sit near a converged plain result (the guided and plain
    estimators share the integrand)."""
    poses, samples = 5, 1 << 18
    sim = str(tmp_path / "guided.SIM")
    subprocess.check_call([guided_bin, sim, str(poses), str(samples)])
    frames = np.fromfile(sim, np.complex64).reshape(poses, 256).astype(np.complex128)
    w = scenes.dihedral_workload(poses=poses, samples_per_pose=samples)
    be = gb300.Backend(w.mesh, None)
    t = PathTracer()
    t.maxDepth = 2
    t.doGuiding = True
    guided = be.simulate_batch(w.rf, 256, t, w.tx, w.rx, w.budget).astype(np.complex128)
    t.doGuiding = False
    plain = be.simulate_batch(w.rf, 256, t, w.tx, w.rx, np.full(poses, 1 << 24, np.int64)).astype(np.complex128)
    for k in range(poses):
        if np.linalg.norm(plain[k]) == 0:
            continue
        e_abi = np.linalg.norm(frames[k] - guided[k]) / np.linalg.norm(guided[k])
        e_conv = np.linalg.norm(frames[k] - plain[k]) / np.linalg.norm(plain[k])
        print("pose %d: C++ guided vs C ABI guided %.3e, vs plain 2^24 %.3e" % (k, e_abi, e_conv))
        assert e_abi <= 0.05, k
        assert e_conv <= 0.08, k


@pytest.fixture(scope="module")
def obj_bin(product_lib, tmp_path_factory):
    return compile_example("obj_example", tmp_path_factory.mktemp("cpp"))


def test_cpp_obj_scene_matches_oracle(obj_bin, tmp_path, oracle_lib):
    """An OBJ scene (the sphere above ground, written out as 'v'/'f' lines with a comment,
    a smoothing line and slash-separated face tokens) read by the C++ WavefrontFile,
    traced through the C++ drop-in, against the oracle on the same mesh at 1e-4."""
    w = scenes.sphere_ground_workload(samples=1 << 16, level=4)
    v = np.asarray(w.mesh.vertexBuffer, np.float32)
    f = np.asarray(w.mesh.indexBuffer, np.int32)
    obj = tmp_path / "sphere.obj"
    with open(obj, "w") as fh:
        fh.write("# icosphere above a ground quad\ns off\n")
        for x in v:
            fh.write("v %r %r %r\n" % (float(x[0]), float(x[1]), float(x[2])))
        for i, t in enumerate(f):
            a, b, c = (int(k) + 1 for k in t)
            fh.write(("f %d/%d/%d %d/%d/%d %d/%d/%d\n" % (a, a, a, b, b, b, c, c, c)) if i % 2 else
                     ("f %d %d %d\n" % (a, b, c)))
    a = w.tx[0]
    pose = [str(float(x)) for x in list(a.position()) + list(np.asarray(a.rotation(), np.float32).ravel())]
    sim = str(tmp_path / "obj.SIM")
    subprocess.check_call([obj_bin, str(obj), sim, str(1 << 16), str(w.max_depth), str(w.frame.samplesPerChirp),
                           repr(float(w.rf.adcRate))] + pose)
    row = np.fromfile(sim, np.complex64)
    t = PathTracer()
    t.doGuiding = False
    t.maxDepth = w.max_depth
    ref = oracle_lib.Scene(w.mesh).fetch_row(w.rf, w.frame.samplesPerChirp, a, a, t, 1 << 16)
    assert np.linalg.norm(ref) > 0
    assert np.linalg.norm(row - ref) / np.linalg.norm(ref) <= 1e-4
