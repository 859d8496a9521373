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
