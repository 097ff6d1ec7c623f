"""Builds libsphgpu.so in-tree from opensph_gb300/csrc with nvcc for sm_103a (GB300).

    python -m opensph_gb300.build [--jobs N] [--verbose]

Each translation unit is compiled in parallel; the FP64 units are compiled without FMA contraction
(-fmad=false) so that their per-pair terms are the IEEE-identical expressions of the reference, the
mixed-precision units and the FP64 gravity evaluation (walk64.cu, whose terms differ from the reference's in
the last bits only) with contraction. Host code is compiled with -ffp-contract=off for the same reason
(the LUT tables built on the host must match the reference's bit for bit on both x86 and Arm hosts).
"""
import argparse
import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
TARGET = os.path.join(HERE, "libsphgpu.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off", "-Xptxas", "-v",
          "--expt-relaxed-constexpr", "-I", os.path.join(HERE, "..", "include")]
UNITS = {
    "abi.cu": ["-fmad=false"],
    "grid.cu": ["-fmad=false"],
    "sph64.cu": ["-fmad=false"],
    "gravity.cu": ["-fmad=false"],
    "treebuild.cu": ["-fmad=false"],
    "sph32.cu": [],
    "gravity32.cu": [],
    "walk64.cu": [],
    "noalloc.cu": [],
    "peak.cu": [],
    "adjoint.cu": ["-fmad=false"],
    "nbody.cu": ["-fmad=false"],
}


def nvcc():
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found")
    return path


def _compile(unit, extra, verbose):
    src = os.path.join(CSRC, unit)
    obj = os.path.join(BUILD, unit + ".o")
    cmd = [nvcc()] + ARCH + COMMON + extra + ["-c", src, "-o", obj]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {unit}:\n{res.stderr}")
    return obj, res.stderr if verbose else ""


def build(jobs=None, verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    jobs = jobs or min(len(UNITS), os.cpu_count() or 4)
    with concurrent.futures.ThreadPoolExecutor(max_workers=jobs) as ex:
        futs = [ex.submit(_compile, u, f, verbose) for u, f in UNITS.items()]
        objs = []
        for f in futs:
            obj, log = f.result()
            objs.append(obj)
            if log:
                sys.stderr.write(log)
    tmp = TARGET + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-Xlinker", "-z,defs"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stderr}")
    os.replace(tmp, TARGET)
    return TARGET


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--jobs", type=int, default=None)
    ap.add_argument("--verbose", action="store_true")
    a = ap.parse_args()
    print(build(a.jobs, a.verbose))
