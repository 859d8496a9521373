"""The host thread pool of the packing passes, compiled and stressed on the CPU."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "hw-radiosity_gb300", "csrc")
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")


def test_host_pool_passes_visit_every_index_once(tmp_path):
    if not shutil.which("g++") or not os.path.exists(os.path.join(CUDA, "include", "cuda_runtime.h")):
        pytest.skip("g++ or the CUDA headers are missing")
    exe = str(tmp_path / "pool_check")
    subprocess.run(["g++", "-O2", "-std=c++17", "-pthread", "-I", CSRC, "-I", os.path.join(CUDA, "include"),
                    os.path.join(HERE, "host_pool_check.cpp"), "-o", exe, "-L", os.path.join(CUDA, "lib64"),
                    "-lcudart"], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and "bad 0" in r.stdout, r.stdout + r.stderr
