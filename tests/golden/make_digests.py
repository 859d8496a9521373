#!/usr/bin/env python3
"""Digests of the reference's own CPU solver on the benchmark-size scenes.

The per-slot fixtures of make_golden.py would be tens of megabytes at these
sizes, so this script keeps, per case, the shooter trace and the SHA-256 of
the bit patterns of each per-slot array (parent, vertices, accB, deltaB) after
a bounded number of steps, plus a few raw values for diagnosis.  The GPU tests
compare the solver's arrays with these digests bit for bit.

Cases (the scenes are regenerated from hwrad.scenes, seeded):
  hall         the 40x20x100 hall, 422,429 slots after pre-partition, 12 steps
  batch256     the 256 rooms of the batched benchmark (batch_rooms(256, 4000)),
               100 steps each: the iterations the benchmark times

Some batch rooms have walks the reference never finishes: its TreeNodeNum
returns a leaf that does not contain the point and RayHitted cycles forever
(scene 27 has tens of thousands per step).  A scene whose reference run does
not end within the per-scene limit is recorded as such, with no digest; the
tests pin those scenes to the C restatement, which stops a walk whose state
repeats.

The reference binary is oracle/_ref/rad_ref32 (staged from the reference's
sources by oracle/stage_ref.py, no FP contraction; its arithmetic is the
same on x86-64 and aarch64).  Its O(N^2) neighbour scan makes the hall take
about ten minutes on eight cores, which is why these are fixtures and not
live runs.

    python3 tests/golden/make_digests.py [--ref DIR] [--only hall|batch256] [--jobs N]
"""
import argparse
import hashlib
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "oracle"))
sys.path.insert(0, os.path.join(REPO, "hw-radiosity_gb300"))

import runner  # noqa: E402
from hwrad import scenes  # noqa: E402

DIGEST_FIELDS = ("parent", "p", "accB", "deltaB")


def digest(a) -> str:
    a = np.ascontiguousarray(a)
    return hashlib.sha256(a.view(np.uint8).tobytes()).hexdigest()


def summarize(dump, trace):
    tr = np.ascontiguousarray(trace[:, 0], np.int32)
    out = {"n_slots": int(dump["n"]), "steps": int(dump["steps"]), "trace_len": int(len(tr)),
           "trace_sha256": digest(tr), "trace_head": [int(x) for x in tr[:16]]}
    for k in DIGEST_FIELDS:
        out[f"{k}_sha256"] = digest(dump[k])
    # a few raw values, to tell a near miss from garbage when a digest differs
    out["accB_head"] = [float(x) for x in dump["accB"][:4].ravel()]
    out["deltaB_sum"] = float(np.asarray(dump["deltaB"], np.float64).sum())
    return out


def run_case(sc, steps, jobs, wd, timeout=24 * 3600):
    tri = sc.write(os.path.join(wd, "scene.tri"))
    argv = sc.argv()
    try:
        out = runner.run(runner.REF32, tri, argv + ["-jobs", str(jobs)], steps=steps, workdir=wd, timeout=timeout)
    except subprocess.TimeoutExpired:
        return {"argv": argv, "reference_ends": False,
                "note": f"the reference run did not end within {timeout} s (a walk that cycles forever)"}
    tr = runner.trace_array(out["trace"])
    res = summarize(out["dump"], tr)
    res["argv"] = argv
    res["reference_ends"] = True
    res["tri_sha256"] = hashlib.sha256(open(tri, "rb").read()).hexdigest()
    return res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=None, help="reference tree (default: RAD_REFERENCE_DIR or the staged copy)")
    ap.add_argument("--only", default=None)
    ap.add_argument("--jobs", type=int, default=os.cpu_count() or 1)
    args = ap.parse_args()
    if not runner.build_ref(args.ref):
        sys.exit("reference binaries could not be built")
    path = os.path.join(HERE, "digests.json")
    index = json.load(open(path)) if os.path.exists(path) else {}
    src = "reference src/ (staged by oracle/stage_ref.py), oracle/_ref/rad_ref32"
    if args.only in (None, "hall"):
        t0 = time.time()
        wd = tempfile.mkdtemp(prefix="digest_hall_")
        res = run_case(scenes.hall(), 12, args.jobs, wd)
        res["source"] = src
        index["hall"] = res
        print(f"hall: {res['n_slots']} slots, {res['steps']} steps, {time.time() - t0:.0f} s", flush=True)
        json.dump(index, open(path, "w"), indent=1, sort_keys=True)
    if args.only in (None, "batch256"):
        t0 = time.time()
        rooms = scenes.batch_rooms(256, seed=4000)
        per = []
        for k, sc in enumerate(rooms):
            wd = tempfile.mkdtemp(prefix=f"digest_b{k}_")
            per.append(run_case(sc, 100, args.jobs, wd, timeout=300))
            if k % 16 == 0:
                print(f"batch256: scene {k}, {time.time() - t0:.0f} s", flush=True)
        index["batch256"] = {"scenes": per, "steps": 100, "seed": 4000, "source": src}
        print(f"batch256: {len(per)} scenes, {time.time() - t0:.0f} s", flush=True)
        json.dump(index, open(path, "w"), indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
