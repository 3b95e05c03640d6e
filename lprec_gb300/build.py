"""Build liblprec_gb300.so in-tree with nvcc for sm_103a (GB300).

    python -m lprec_gb300.build          # or: python lprec_gb300/build.py

Each translation unit compiles in parallel to lprec_gb300/_build/, then one
shared library is linked next to this file.  Host code is compiled with
-ffp-contract=off so the float32 steps of the precompute round exactly like
the reference's NumPy/CuPy precompute on both x86_64 and aarch64 hosts.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "liblprec_gb300.so")
SOURCES = ["lp_kernels.cu", "lp_kernels_mr.cu", "lp_kernels_mr2.cu", "lp_kernels_mr3.cu", "lp_kernels_mr4.cu",
           "lp_kernels_mr5.cu", "lp_handle.cu", "lp_solver.cu", "precompute.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _deps():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [
        os.path.join(HERE, "..", "include", "lprec_gb300.h"), __file__]


def build(force=False, verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    nv = nvcc()
    deps = _deps()
    common = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off,-O2", "-I", CSRC]
    jobs = []
    objs = []
    for src in SOURCES:
        obj = os.path.join(BUILD, src + ".o")
        objs.append(obj)
        if force or _newer(obj, deps):
            if src.endswith(".cu"):
                cmd = [nv] + ARCH + ["-lineinfo", "-Xptxas", "-v" if verbose else "-O3"] + common
            else:
                cmd = [nv, "-x", "c++"] + common
            jobs.append(cmd + ["-c", os.path.join(CSRC, src), "-o", obj])
    with cf.ThreadPoolExecutor(max(1, len(jobs))) as ex:
        results = list(ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), jobs))
    for cmd, r in zip(jobs, results):
        if verbose or r.returncode != 0:
            sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s" % cmd[-3])
    if force or jobs or not os.path.exists(LIB):
        cmd = [nv] + ARCH + ["-shared", "-o", LIB] + objs + ["-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("link failed")
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
