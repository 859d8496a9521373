#!/usr/bin/env python3
"""Generate the golden fixtures from the reference's own CPU solver.

Run in a container that has the reference tree (it stages and builds
``oracle/_ref/rad_ref32`` and ``rad_ref64`` from the reference's sources, see
oracle/stage_ref.py).  For every case it writes the seeded scene (generated
by hwrad.scenes), runs the reference binary to convergence, and stores:
the shooter trace, per-slot parent / vertices / accB / deltaB / neighbours,
the SHA-256 of the ``.fin`` output and of the ``.tri`` input text.

    python3 tests/golden/make_golden.py [--ref /path/to/reference]
"""
import argparse
import hashlib
import json
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "oracle"))
sys.path.insert(0, os.path.join(REPO, "hw-radiosity_gb300"))

import runner  # noqa: E402
from golden_cases import CASES, make_scene  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=None, help="reference tree (default: runner.reference_dir())")
    args = ap.parse_args()
    if not runner.build_ref(args.ref):
        sys.exit("reference binaries could not be built")
    index = {}
    for name, case in CASES.items():
        sc = make_scene(case)
        wd = tempfile.mkdtemp(prefix=f"golden_{name}_")
        tri = sc.write(os.path.join(wd, "scene.tri"))
        argv = sc.argv(case.get("extra"))
        binary = runner.REF64 if case.get("fp64") else (runner.REF32A if case.get("adaptive") else runner.REF32)
        # the adaptive variant is the reference's serial loop: one job
        out = runner.run(binary, tri, argv + ["-jobs", "1" if case.get("adaptive") else "4"], workdir=wd)
        d = out["dump"]
        P = int(dict(zip(argv[::2], argv[1::2])).get("-parallel_src", 1)) if "-parallel_src" in argv else 1
        tr = runner.trace_array(out["trace"], P)
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), trace=tr, parent=d["parent"], p=d["p"],
                            accB=d["accB"], deltaB=d["deltaB"], nb=d["nb"])
        index[name] = {
            "argv": argv, "fp64": bool(case.get("fp64")), "adaptive": bool(case.get("adaptive")), "P": P,
            "n_slots": d["n"], "steps": d["steps"],
            "fin_sha256": hashlib.sha256(out["fin"]).hexdigest(),
            "tri_sha256": hashlib.sha256(open(tri, "rb").read()).hexdigest(),
            "source": "reference src/ (staged by oracle/stage_ref.py), built by oracle/Makefile",
        }
        print(f"{name}: {d['n']} slots, {d['steps']} steps")
    with open(os.path.join(HERE, "index.json"), "w") as fh:
        json.dump(index, fh, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
