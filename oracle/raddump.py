"""Reader for RADDUMP1 per-slot state dumps.

ORACLE / TEST INFRASTRUCTURE ONLY.  Both checkers (the reference build with
oracle/ref_hooks.cpp and the C restatement oracle/radoracle.c) write this
format: "RADDUMP1", int32 n_slots, int32 element size (4 or 8), int32 steps,
then field-major arrays over slots 0..n-1: parent i32, p f[9], accB f[9],
deltaB f[3], area f, n f[3], c f[3], Frgb i32[3], neighbor i32[3].
"""
import numpy as np


def read_dump(path):
    with open(path, "rb") as fh:
        buf = fh.read()
    assert buf[:8] == b"RADDUMP1", path
    n, esz, steps = np.frombuffer(buf, np.int32, 3, 8)
    ft = np.float32 if esz == 4 else np.float64
    off = 20
    out = {"n": int(n), "steps": int(steps)}

    def take(name, dt, cols):
        nonlocal off
        cnt = int(n) * cols
        a = np.frombuffer(buf, dt, cnt, off)
        off += cnt * np.dtype(dt).itemsize
        out[name] = a.reshape(int(n), cols) if cols > 1 else a

    take("parent", np.int32, 1)
    take("p", ft, 9)
    take("accB", ft, 9)
    take("deltaB", ft, 3)
    take("area", ft, 1)
    take("n_", ft, 3)
    take("c", ft, 3)
    take("Frgb", np.int32, 3)
    take("nb", np.int32, 3)
    assert off == len(buf), (off, len(buf))
    return out


def read_trace(path):
    """List of shooter lists, one per step (the final empty list included)."""
    steps = []
    with open(path) as fh:
        for line in fh:
            parts = line.split()
            if not parts:
                continue
            k = int(parts[0])
            steps.append([int(x) for x in parts[1:1 + k]])
    return steps
