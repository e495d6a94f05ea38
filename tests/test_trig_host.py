"""The primary direction's sine and cosine on the CPU (tests/native/sincos_check.cpp,
compiled from the product's own header): the fast certified evaluation the reference-phase
kernels call gives the double-precision evaluation's bits on a sweep of the floats in
[-8, 8] (the angle 2 pi u lies in [0, 2 pi]), and its double-float results stay within the
relative error the rounding test assumes (2^-37, stated bound 2^-38.8)."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CUDA_INC = "/usr/local/cuda/include"


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    if not os.path.isdir(CUDA_INC):
        pytest.skip("CUDA headers not found")
    exe = str(tmp_path_factory.mktemp("trig") / "sincos_check")
    subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-I", os.path.join(ROOT, "hussar_gb300", "csrc"),
                    "-I", CUDA_INC, "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "native", "sincos_check.cpp"), "-o", exe, "-pthread"], check=True)
    return exe


def test_fast_sincos_matches_double_evaluation(checker):
    out = subprocess.run([checker, "61", str(min(8, os.cpu_count() or 1))], check=True, capture_output=True,
                         text=True).stdout.split()
    res = {out[i]: float(out[i + 1]) for i in range(0, len(out), 2)}
    print(res)
    assert res["checked"] > 3.5e7
    assert res["mismatches"] == 0
    assert res["max_log2_rel_err"] < -38.8
