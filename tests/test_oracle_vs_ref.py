"""The oracle against the reference binary itself, where it was built from the
reference's sources (oracle/_ref).  Covers the reference's own model files
when the reference tree is mounted; skipped otherwise."""
import os

import numpy as np
import pytest

import runner
from helpers import EDGE_SCENES, same_bits, write_edge_scene
from hwrad import scenes

REF_MODELS = os.path.join(runner.reference_dir() or "", "model")


def _cases(workdir):
    out = []
    s = scenes.room_with_boxes(10, 5, 2, seed=3, size=25.0)
    out.append((s.write(os.path.join(workdir, "vr_boxes.tri")), s.argv({"-triangle": "3000"})))
    if os.path.isdir(REF_MODELS):
        for m in ("box", "model1", "model2s", "room", "sbox", "blocks", "hall"):
            out.append((os.path.join(REF_MODELS, f"{m}.tri"), ["-triangle", "2500"]))
    return out


@pytest.mark.skipif(not runner.have_ref(), reason="reference binary not built here")
@pytest.mark.parametrize("fp64", [False, True])
def test_oracle_equals_reference_binary(built, workdir, fp64):
    for tri, argv in _cases(workdir):
        a = runner.run(runner.REF64 if fp64 else runner.REF32, tri, argv + ["-jobs", "2"])
        b = runner.oracle(tri, argv, fp64=fp64)
        assert a["trace"] == b["trace"], tri
        for k in ("parent", "p", "accB", "deltaB", "nb", "n_", "c", "area", "Frgb"):
            assert same_bits(a["dump"][k], b["dump"][k]), (tri, k)
        assert a["fin"] == b["fin"], tri


@pytest.mark.skipif(not os.path.exists(runner.REF32C), reason="reference counter build not here")
def test_oracle_counters_equal_reference(built, workdir):
    s = scenes.room(8)
    tri = s.write(os.path.join(workdir, "cnt_room8.tri"))
    a = runner.run(runner.REF32C, tri, s.argv() + ["-jobs", "2"], steps=40)
    b = runner.oracle(tri, s.argv(), steps=40)
    ca, cb = runner.counters(a["stderr"]), runner.counters(b["stderr"])
    assert cb.pop("loops") == 0          # no walk of this scene repeats a state
    assert ca == cb


@pytest.mark.skipif(not runner.have_ref(), reason="reference binary not built here")
@pytest.mark.parametrize("name", EDGE_SCENES)
@pytest.mark.parametrize("fp64", [False, True])
@pytest.mark.parametrize("P", [1, 2])
def test_oracle_equals_reference_on_edge_scenes(built, workdir, name, fp64, P):
    tri, argv = write_edge_scene(name, workdir)
    argv = argv + ["-parallel_src", str(P)]
    a = runner.run(runner.REF64 if fp64 else runner.REF32, tri, argv + ["-jobs", "2"])
    b = runner.oracle(tri, argv, fp64=fp64)
    assert a["trace"] == b["trace"]
    for k in ("parent", "p", "accB", "deltaB"):
        assert same_bits(a["dump"][k], b["dump"][k]), k
    assert a["fin"] == b["fin"]
