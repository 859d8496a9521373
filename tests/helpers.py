"""Shared helpers for the test suite."""
import hashlib
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def golden_index():
    with open(os.path.join(GOLDEN, "index.json")) as fh:
        return json.load(fh)


def golden(name):
    return dict(np.load(os.path.join(GOLDEN, f"{name}.npz")))


def bits(a):
    return np.ascontiguousarray(a).view(np.uint8)


def same_bits(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return a.shape == b.shape and a.dtype == b.dtype and np.array_equal(bits(a), bits(b))


def sha256_file(path):
    with open(path, "rb") as fh:
        return hashlib.sha256(fh.read()).hexdigest()


def write_case(name, workdir):
    """Regenerate a golden case's scene; returns (tri_path, argv, index entry)."""
    from golden_cases import CASES, make_scene
    case = CASES[name]
    sc = make_scene(case)
    tri = sc.write(os.path.join(workdir, f"{name}.tri"))
    idx = golden_index()[name]
    return tri, idx["argv"], idx


def rel_l2(a, b):
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    den = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / den) if den > 0 else float(np.linalg.norm(a - b))


def build_fp_forms_check(workdir):
    """Compile tests/fp_forms_check.cu (host and device checks of the FP32
    forms of the reference's double expressions) with the solver's flags."""
    import shutil
    import subprocess
    here = os.path.dirname(os.path.abspath(__file__))
    repo = os.path.dirname(here)
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    exe = os.path.join(workdir, "fp_forms_check")
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-std=c++17", "-fmad=false",
                    "--prec-div=true", "--prec-sqrt=true", "-Xcompiler", "-ffp-contract=off,-O2",
                    "-I", os.path.join(repo, "hw-radiosity_gb300", "csrc"), "-I", os.path.join(repo, "include"),
                    "-o", exe, os.path.join(here, "fp_forms_check.cu")], check=True, capture_output=True)
    return exe


EDGE_SCENES = ["empty", "dark", "one", "two"]


def write_edge_scene(name, workdir):
    """Small edge inputs: an empty file, a room with no emitter, one emitting
    triangle, and an emitting triangle with one receiver.  Returns
    (tri_path, argv)."""
    from hwrad import scenes
    path = os.path.join(workdir, f"edge_{name}.tri")
    if name == "empty":
        open(path, "w").close()
        return path, []
    if name == "dark":
        s = scenes.room(4, emitter=(0.0, 0.0), name="dark")
    elif name == "one":
        s = scenes.Scene(vtx=np.array([[[0, 0, 0], [1, 0, 0], [0, 1, 0]]], np.float32),
                         frgb=np.array([[100, 100, 100]]), brgb=np.array([[255, 255, 255]]),
                         options={"-light": "0.05"}, name="one")
    elif name == "two":
        s = scenes.Scene(vtx=np.array([[[0, 0, 0], [0, 1, 0], [1, 0, 0]], [[0, 0, 2], [1, 0, 2], [0, 1, 2]]],
                                      np.float32),
                         frgb=np.array([[100, 100, 100], [200, 150, 100]]),
                         brgb=np.array([[255, 255, 255], [0, 0, 0]]), options={"-light": "0.05"}, name="two")
    else:
        raise ValueError(name)
    return s.write(path), s.argv()
