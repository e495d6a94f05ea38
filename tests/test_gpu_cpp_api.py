"""The C++ drop-in (include/hussar/gb300.h + gb300_types.h): the reference's example
flow compiled with g++ against libhsr_gb300.so gives the same frames as the Python
binding and the oracle."""
import os
import subprocess

import numpy as np
import pytest

from hussar_gb300 import NFAntenna, PathTracer, gb300, scenes

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def example_bin(product_lib, tmp_path_factory):
    out = str(tmp_path_factory.mktemp("cpp") / "dihedral_example")
    libdir = os.path.join(ROOT, "hussar_gb300")
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"),
                           os.path.join(ROOT, "tests", "cpp", "dihedral_example.cpp"), "-L", libdir, "-lhsr_gb300",
                           "-Wl,-rpath," + libdir, "-o", out])
    return out


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
