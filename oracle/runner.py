"""Run the checkers: the C restatement (``_build/radoracle``) and, where it was
built from the reference's own sources, the reference binary (``_ref/``).

ORACLE / TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke()
and bench.py's CPU-baseline leg, never by the product.
"""
from __future__ import annotations

import os
import subprocess
import tempfile
from typing import Dict, List, Optional, Sequence

import numpy as np

from raddump import read_dump, read_trace  # noqa: E402  (oracle/ is on sys.path)

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE32 = os.path.join(HERE, "_build", "radoracle")
ORACLE64 = os.path.join(HERE, "_build", "radoracle64")
REF32 = os.path.join(HERE, "_ref", "rad_ref32")
REF32C = os.path.join(HERE, "_ref", "rad_ref32c")
REF64 = os.path.join(HERE, "_ref", "rad_ref64")
REF32A = os.path.join(HERE, "_ref", "rad_ref32a")
# the reference's own build flags (FP contraction on): timed, never compared
REF_SHIPPED = os.path.join(HERE, "_ref", "rad_ref_shipped")
REF_SHIPPED_FLAGS = "-O2 -fopenmp -std=c++11 -march=native (reference Makefile:7) + -include vector"


def build_oracle() -> None:
    subprocess.run(["make", "-s", "-C", HERE, "oracle"], check=True)


def reference_dir() -> Optional[str]:
    """The reference tree (morris821028/hw-radiosity) to stage from, or None:
    $RAD_REFERENCE_DIR, else baseline/_ref, else /root/reference -- the first
    that holds a src/ directory.  On a machine without any of them the staged
    copy under oracle/_ref is built as it is."""
    repo = os.path.dirname(HERE)
    for cand in (os.environ.get("RAD_REFERENCE_DIR"), os.path.join(repo, "baseline", "_ref"), "/root/reference"):
        if cand and os.path.isdir(os.path.join(cand, "src")):
            return cand
    return None


def build_ref(ref_root: Optional[str] = None) -> bool:
    """Stage (when the reference tree is present) and build the reference binaries.
    Returns True when oracle/_ref binaries exist afterwards."""
    ref_root = ref_root or reference_dir()
    if ref_root and os.path.isdir(os.path.join(ref_root, "src")):
        subprocess.run(["python3", os.path.join(HERE, "stage_ref.py"), "--ref", ref_root], check=True,
                       capture_output=True)
    if os.path.isdir(os.path.join(HERE, "_ref", "src", "src")):
        subprocess.run(["make", "-s", "-C", HERE, "ref"], check=True)
    return have_ref()


def have_ref() -> bool:
    return all(os.path.exists(p) for p in (REF32, REF64))


def run(binary: str, tri: str, args: Sequence[str], steps: Optional[int] = None, env: Optional[Dict] = None,
        workdir: Optional[str] = None, timeout: float = 600) -> Dict[str, object]:
    """Run one checker binary; returns dump, trace, .fin bytes and stderr."""
    wd = workdir or tempfile.mkdtemp(prefix="radora_")
    e = dict(os.environ)
    e.update({"RAD_DUMP": os.path.join(wd, "out.dump"), "RAD_TRACE": os.path.join(wd, "out.trace")})
    if steps is not None:
        e["RAD_MAX_STEPS"] = str(int(steps))
    if env:
        e.update(env)
    cmd = [binary, tri] + list(args) + ["-write_cycle", "1000000000", "-o", os.path.join(wd, "out")]
    r = subprocess.run(cmd, env=e, capture_output=True, text=True, timeout=timeout)
    if r.returncode != 0:
        raise RuntimeError(f"{binary} failed ({r.returncode}): {r.stderr[-2000:]}")
    with open(os.path.join(wd, "out.fin"), "rb") as fh:
        fin = fh.read()
    return {"dump": read_dump(os.path.join(wd, "out.dump")), "trace": read_trace(os.path.join(wd, "out.trace")),
            "fin": fin, "stderr": r.stderr, "stdout": r.stdout, "dir": wd}


def oracle(tri: str, args: Sequence[str], steps: Optional[int] = None, fp64: bool = False, adaptive: bool = False,
           **kw):
    """The C restatement; adaptive=True runs the adaptive split variant."""
    return run(ORACLE64 if fp64 else ORACLE32, tri, list(args) + (["-adaptive"] if adaptive else []), steps, **kw)


def rays(tri: str, args: Sequence[str], p: np.ndarray, v: np.ndarray, ban: np.ndarray, fp64: bool = False) -> np.ndarray:
    """RayHitted for each (p, v, ban) after init + pre-partition."""
    ft = np.float64 if fp64 else np.float32
    wd = tempfile.mkdtemp(prefix="radray_")
    path = os.path.join(wd, "rays.bin")
    rec = np.zeros(len(p), dtype=[("pv", ft, 6), ("ban", np.int32)])
    rec["pv"][:, :3] = p
    rec["pv"][:, 3:] = v
    rec["ban"] = ban
    rec.tofile(path)
    run(ORACLE64 if fp64 else ORACLE32, tri, args, steps=0, env={"RAD_RAYS": path}, workdir=wd)
    return np.fromfile(path + ".out", np.int32)


def form_factors(tri: str, args: Sequence[str], src: int, rcv: np.ndarray, fp64: bool = False) -> np.ndarray:
    ft = np.float64 if fp64 else np.float32
    wd = tempfile.mkdtemp(prefix="radff_")
    path = os.path.join(wd, "ff.bin")
    np.concatenate([np.array([src, len(rcv)], np.int32), np.asarray(rcv, np.int32)]).tofile(path)
    run(ORACLE64 if fp64 else ORACLE32, tri, args, steps=0, env={"RAD_FF": path}, workdir=wd)
    return np.fromfile(path + ".out", ft).reshape(-1, 3)


def counters(stderr: str) -> Dict[str, int]:
    for line in stderr.splitlines():
        if line.startswith("[COUNT]"):
            w = line.split()
            return {w[i]: int(w[i + 1]) for i in range(1, len(w) - 1, 2)}
    return {}


def trace_array(trace: List[List[int]], P: int = 1) -> np.ndarray:
    """Shooter lists of the executed steps, padded with -1 to P columns."""
    steps = [t for t in trace if t]
    out = np.full((len(steps), P), -1, np.int32)
    for i, t in enumerate(steps):
        out[i, :len(t)] = t
    return out
