"""Host half of the product (scene input, neighbour links, pre-partition,
octree build, .fin writer) against the oracle, bit for bit.  No GPU."""
import os
import re

import numpy as np
import pytest

import runner
from helpers import same_bits
from hwrad import capi, scenes

FIELDS = ("parent", "p", "accB", "deltaB", "area", "n_", "c", "Frgb", "nb")


def _scene_cases(workdir):
    c = []
    s = scenes.room(8)
    c.append(("room8", s.write(os.path.join(workdir, "h_room8.tri")), s.argv()))
    s = scenes.room(8, size=100.0)
    c.append(("big", s.write(os.path.join(workdir, "h_big.tri")), s.argv({"-triangle": "2500"})))
    s = scenes.room_with_boxes(12, 6, 2, seed=7, size=30.0)
    c.append(("boxes", s.write(os.path.join(workdir, "h_boxes.tri")), s.argv({"-triangle": "4000"})))
    s = scenes.room(3, size=40.0, emitter=(0.3, 0.7))
    c.append(("coarse", s.write(os.path.join(workdir, "h_coarse.tri")), s.argv({"-triangle": "900"})))
    if os.path.isdir("/root/reference/model"):
        for m in ("box", "model2s", "room", "blocks", "church"):
            c.append((m, f"/root/reference/model/{m}.tri", ["-triangle", "3000"]))
    return c


@pytest.mark.parametrize("fp64", [False, True])
def test_host_state_equals_oracle(built, workdir, fp64):
    for name, tri, argv in _scene_cases(workdir):
        ref = runner.oracle(tri, argv, steps=0, fp64=fp64)
        o = capi.options_from_argv(argv, precision=64 if fp64 else 32)
        sc = capi.Scene.load(tri, o)
        tree = capi.Octree(sc, 4)
        sc.init()
        sc.prepartition()
        v = sc.view()
        assert v["n"] == ref["dump"]["n"], name
        for k in FIELDS:
            assert same_bits(v[k], ref["dump"][k]), (name, k)
        m = re.search(r"#TreeNode = (\d+), #Trilist = (\d+)", ref["stderr"])
        info = tree.info()
        assert (info["ref_nodes"], info["ref_list"]) == (int(m.group(1)), int(m.group(2))), name
        prefix = os.path.join(workdir, f"h_{name}_{int(fp64)}")
        sc.write_fin(prefix, 0)
        with open(prefix + ".fin", "rb") as fh:
            assert fh.read() == ref["fin"], name


def test_octree_build_threads_agree(built, workdir):
    s = scenes.room_with_boxes(16, 8, 2, seed=5)
    tri = s.write(os.path.join(workdir, "h_thr.tri"))
    o = capi.options_from_argv(s.argv())
    a = capi.Octree(capi.Scene.load(tri, o), 1).info()
    b = capi.Octree(capi.Scene.load(tri, o), 8).info()
    assert a == b


def test_scene_from_arrays_equals_text(built, workdir):
    s = scenes.room_with_boxes(6, 3, 1, seed=9)
    tri = s.write(os.path.join(workdir, "h_arr.tri"))
    o = capi.options_from_argv(s.argv())
    a = capi.Scene.load(tri, o)
    b = capi.Scene.from_arrays(s.vtx, s.frgb, s.brgb, o)
    for sc in (a, b):
        sc.init()
        sc.prepartition()
    va, vb = a.view(), b.view()
    for k in FIELDS:
        assert same_bits(va[k], vb[k]), k


def test_malformed_input_is_an_error(built, workdir):
    bad = os.path.join(workdir, "bad.tri")
    with open(bad, "w") as fh:
        fh.write("Triangle\n1 2 3 0 0 0\n0 0 0\n1 0 oops\n0 1 0\n")
    with pytest.raises(capi.RadError) as e:
        capi.Scene.load(bad, capi.options())
    assert e.value.code == capi.RAD_ERR_PARSE
    with pytest.raises(capi.RadError) as e:
        capi.Scene.load(os.path.join(workdir, "missing.tri"), capi.options())
    assert e.value.code == capi.RAD_ERR_IO


def test_empty_scene(built, workdir):
    empty = os.path.join(workdir, "empty.tri")
    open(empty, "w").close()
    sc = capi.Scene.load(empty, capi.options())
    tree = capi.Octree(sc, 2)
    sc.init()
    sc.prepartition()
    assert sc.view()["n"] == 0
    assert tree.info()["leaves"] == 1


def test_trailing_token_without_newline(built, workdir):
    # a keyword that runs into end of file ends the scan (fscanf + feof)
    s = scenes.room(2, emitter=(0.0, 1.0))
    text = s.to_tri() + "Triangle"
    p = os.path.join(workdir, "trail.tri")
    with open(p, "w") as fh:
        fh.write(text)
    assert capi.Scene.load(p, capi.options()).view()["n"] == s.n
