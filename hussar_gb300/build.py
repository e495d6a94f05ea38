"""Builds libhsr_gb300.so in-tree with nvcc for sm_103a (no torch involved).

The trace kernels are compiled with -fmad=false so that their float expressions round
exactly like the CPU restatement used by the tests, except the wavefront kernel's
split-phase instantiations (hsr_wave_split.cu): that form is bounded against the FP64
oracle rather than matched to the reference's FP32 rounding, and is compiled with fused
multiply-adds and the approximate single-precision divide and square root (within 2 ulp;
1.1x on the guided dihedral). The other translation units use the default contraction.
"""
import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libhsr_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O3",
          "--expt-relaxed-constexpr", "-I", os.path.join(ROOT, "include")]
UNITS = {
    "hsr_api.cu": [],
    "hsr_bvh.cu": [],
    "hsr_guide.cu": [],
    "hsr_synth.cu": [],
    "hsr_noalloc.cu": [],
    "hsr_serve.cu": [],
    "hsr_trace.cu": ["-fmad=false"],
    "hsr_wave.cu": ["-fmad=false"],
    "hsr_wave_split.cu": ["-prec-div=false", "-prec-sqrt=false"],
    "hsr_io.cpp": [],
}


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _compile(unit, extra, verbose):
    src = os.path.join(CSRC, unit)
    obj = os.path.join(BUILD, os.path.splitext(unit)[0] + ".o")
    cmd = [nvcc()] + ARCH + COMMON + extra + (["-Xptxas", "-v"] if verbose else []) + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (unit, " ".join(cmd), r.stderr))
    return obj, r.stderr


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    for f in os.listdir(CSRC):
        if os.path.getmtime(os.path.join(CSRC, f)) > t:
            return True
    if os.path.getmtime(os.path.join(ROOT, "include", "hsr_gb300.h")) > t:
        return True
    return os.path.getmtime(__file__) > t


def build(force=False, verbose=False):
    """Compiles every translation unit in parallel and links the shared library."""
    if not force and not _stale():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    with concurrent.futures.ThreadPoolExecutor(len(UNITS)) as ex:
        futs = [ex.submit(_compile, u, e, verbose) for u, e in UNITS.items()]
        results = [f.result() for f in futs]
    if verbose:
        for _, log in results:
            sys.stderr.write(log)
    objs = [o for o, _ in results]
    tmp = LIB + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcuda"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
