"""Build the native library and the ``rad`` command for sm_103a.

Outputs (git-ignored, rebuilt on each machine):
    hw-radiosity_gb300/lib/librad_gb300.so   C ABI (include/rad_gb300.h)
    hw-radiosity_gb300/bin/rad               drop-in command line

Host sources are compiled by g++ and the CUDA source by nvcc, in parallel;
every translation unit gets no floating-point contraction (``-ffp-contract=off``
for host code, ``-fmad=false`` for device code) because the solver reproduces
the reference's arithmetic operation by operation.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REPO = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INC = os.path.join(REPO, "include")
OBJ = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "lib", "librad_gb300.so")
BIN = os.path.join(PKG, "bin", "rad")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
HOST_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-Wno-unused-function", f"-I{INC}"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "--prec-div=true", "--prec-sqrt=true",
                     "-Xcompiler", "-fPIC,-ffp-contract=off", f"-I{INC}", "-Xptxas", "-v"]

HOST_SRC = ["scene.cpp", "octree.cpp", "capi.cpp"]
CUDA_SRC = ["rad_dev.cu", "rad_batch.cu", "rad_adapt.cu", "rad_raster.cu", "rad_octree_dev.cu", "rad_scene_dev.cu"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd, log):
    r = subprocess.run(cmd, capture_output=True, text=True)
    log.append((cmd, r.returncode, r.stdout + r.stderr))
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r


def _stale(out: str, deps) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> dict:
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    os.makedirs(os.path.dirname(BIN), exist_ok=True)
    headers = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".h", ".cuh"))] + \
        [os.path.join(INC, "rad_gb300.h")]
    nvcc = _nvcc()
    log: list = []
    jobs = []
    objs = []
    for src in HOST_SRC:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append(["g++"] + HOST_FLAGS + ["-c", s, "-o", o])
    for src in CUDA_SRC:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([nvcc] + NVCC_FLAGS + ["-c", s, "-o", o])
    with ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        for f in [ex.submit(_run, j, log) for j in jobs]:
            f.result()
    if force or _stale(LIB, objs):
        _run([nvcc] + ARCH + ["-shared", "-o", LIB] + objs + ["-lpthread"], log)
    main = os.path.join(CSRC, "rad_main.cpp")
    if force or _stale(BIN, [main, LIB] + headers):
        _run(["g++", "-O2", "-std=c++17", f"-I{INC}", main, "-o", BIN, f"-L{os.path.dirname(LIB)}", "-lrad_gb300",
              "-Wl,-rpath,$ORIGIN/../lib"], log)
    if verbose:
        for cmd, rc, out in log:
            print(" ".join(cmd))
            if out.strip():
                print(out)
    ptxas = "\n".join(out for cmd, rc, out in log if "ptxas" in out)
    return {"lib": LIB, "bin": BIN, "ptxas": ptxas}


if __name__ == "__main__":
    info = build(verbose="-v" in sys.argv, force="-f" in sys.argv)
    print(info["lib"])
    print(info["bin"])
