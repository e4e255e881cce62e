"""Builds the in-tree shared library libdes_gb300.so (CUDA for sm_103a + host C++).

nvcc compiles the device code with -fmad=false (no fused multiply-add, so the
FP64 arithmetic follows the reference's operation order exactly) and the host
code with -ffp-contract=off (aarch64 compilers fuse by default).
"""
import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parents[1]          # dynearthsol-old_gb300/
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
INCLUDE = ROOT / "include"
LIB = BUILD / "libdes_gb300.so"

ARCH = "-gencode=arch=compute_103a,code=sm_103a"
NVCC_FLAGS = ["-O3", "-std=c++17", ARCH, "-lineinfo", "-fmad=false", "--extended-lambda",
              "-Xcompiler=-fPIC,-ffp-contract=off", f"-I{INCLUDE}", f"-I{CSRC}"]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-fopenmp", "-ffp-contract=off", f"-I{INCLUDE}"]

CU_SOURCES = ["des_gpu.cu", "des_noalloc.cu", "des_mlp.cu"]
CXX_SOURCES = ["topology.cpp", "workload.cpp", "save.cpp"]


def _nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found")
    return cand


def _newer(target, deps):
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(map(str, cmd)) + "\n" + r.stdout + r.stderr)
    return r


def build(force=False, verbose=False):
    BUILD.mkdir(exist_ok=True)
    headers = list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + list(INCLUDE.glob("*.h"))
    jobs = []
    objs = []
    nvcc = _nvcc()
    for s in CU_SOURCES:
        src, obj = CSRC / s, BUILD / (s + ".o")
        objs.append(obj)
        if force or _newer(obj, [src] + headers):
            jobs.append([nvcc] + NVCC_FLAGS + ["-c", str(src), "-o", str(obj)])
    for s in CXX_SOURCES:
        src, obj = CSRC / s, BUILD / (s + ".o")
        objs.append(obj)
        if force or _newer(obj, [src] + headers):
            jobs.append(["g++"] + CXX_FLAGS + ["-c", str(src), "-o", str(obj)])
    with ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        for r in ex.map(_run, jobs):
            if verbose and r.stderr:
                print(r.stderr)
    if force or jobs or _newer(LIB, objs):
        _run([nvcc, "-shared", ARCH, "-o", str(LIB)] + [str(o) for o in objs] +
             ["-Xcompiler=-fopenmp", "-lgomp"])
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))
