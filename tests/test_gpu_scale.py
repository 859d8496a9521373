"""Parity at benchmark scale, against the reference binary itself.

- The config-2 room (64x64-quad walls + 16 boxes, 61,440 slots): 600 shooter
  steps, compared bit for bit with oracle/_ref/rad_ref32 built on this machine
  from the reference's sources and run live.
- The config-3 hall (422,429 slots): 12 steps, against the digests of the
  same binary's run (tests/golden/digests.json; the reference's O(N^2)
  neighbour scan takes about ten minutes there, so it is not run live).
- The 256-room benchmark batch: 100 steps of every scene in the batched form,
  against the digests of the binary's run of each scene.  Scenes whose
  reference run never ends (walks that cycle forever) are compared with the
  C restatement instead, which stops such walks.

Bitwise equality of the shooter trace and of every per-slot array is the bar.
"""
import hashlib
import json
import os

import numpy as np
import pytest

import runner
from helpers import GOLDEN, same_bits
from hwrad import capi, scenes

pytestmark = pytest.mark.gpu


def _digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).view(np.uint8).tobytes()).hexdigest()


def _digests():
    with open(os.path.join(GOLDEN, "digests.json")) as fh:
        return json.load(fh)


@pytest.fixture(scope="module")
def ref_built():
    assert runner.build_ref(), "the reference binary could not be built from the staged sources"
    return True


def _prepare(o, gen_or_tri, device_prep=True):
    sc = capi.Scene.load(gen_or_tri, o) if isinstance(gen_or_tri, str) else \
        capi.Scene.from_arrays(gen_or_tri.vtx, gen_or_tri.frgb, gen_or_tri.brgb, o)
    if device_prep:
        tree = capi.Octree(sc, device=0)
        sc.init(device=0)
    else:
        tree = capi.Octree(sc, 8)
        sc.init()
    sc.prepartition()
    return sc, tree


def _check_digest(v, trace, want, what):
    assert v["n"] == want["n_slots"], what
    tr = np.ascontiguousarray(trace[:, 0], np.int32)
    assert len(tr) == want["trace_len"], what
    assert list(tr[:16]) == want["trace_head"], what
    assert _digest(tr) == want["trace_sha256"], what
    for k in ("parent", "p", "accB", "deltaB"):
        assert _digest(v[k]) == want[f"{k}_sha256"], (what, k)


def test_config2_600_steps_equal_reference_binary(built, ref_built, workdir):
    s = scenes.config2()
    tri = s.write(os.path.join(workdir, "config2_ref.tri"))
    argv = s.argv()
    steps = 600
    o = capi.options_from_argv(argv)
    sc, tree = _prepare(o, tri)
    dv = capi.Device(sc, tree, o)
    n, conv, _ = dv.run(steps)
    assert n == steps and not conv
    dv.download(sc)
    ref = runner.run(runner.REF32, tri, argv + ["-jobs", str(os.cpu_count() or 1)], steps=steps, timeout=1800)
    assert ref["dump"]["steps"] == steps
    assert np.array_equal(dv.trace(), runner.trace_array(ref["trace"]))
    v = sc.view()
    for k in ("parent", "p", "accB", "deltaB"):
        assert same_bits(v[k], ref["dump"][k]), k


@pytest.mark.parametrize("layout", [1, 2])
def test_hall_12_steps_equal_reference_digest(built, layout):
    """Both kernel forms (the hall's chosen form 2 and form 1)."""
    want = _digests()["hall"]
    gen = scenes.hall()
    assert gen.argv() == want["argv"]
    o = capi.options_from_argv(gen.argv())
    sc, tree = _prepare(o, gen)
    dv = capi.Device(sc, tree, o)
    dv.set_layout(layout)
    n, conv, _ = dv.run(want["steps"])
    assert n == want["steps"]
    dv.download(sc)
    _check_digest(sc.view(), dv.trace(), want, f"hall, form {layout}")
    dv.close()


def test_benchmark_batch_100_steps_equal_reference(built, workdir):
    """The 256 rooms of the batched benchmark, shot together as the bench
    shoots them (form chosen by the autotuner, then fixed chunks)."""
    want = _digests()["batch256"]
    gens = scenes.batch_rooms(256, seed=want["seed"])
    preps = []
    for g in gens:
        o = capi.options_from_argv(g.argv())
        preps.append((o,) + _prepare(o, g))
    b = capi.Batch([p[1] for p in preps], [p[2] for p in preps], [p[0] for p in preps])
    b.autotune(4, 1)      # ordinary iterations in both forms
    for k in (1, 7, 32):
        b.run(k)
    steps = [b.scene_stats(i)[0] for i in range(len(gens))]
    b.run(want["steps"] - max(steps))
    unpinned = []
    for i, (g, w) in enumerate(zip(gens, want["scenes"])):
        sc = preps[i][1]
        b.download(i, sc)
        st, _ = b.scene_stats(i)
        if w["reference_ends"]:
            assert st == w["steps"], i
            _check_digest(sc.view(), b.trace(i), w, f"batch scene {i}")
        else:
            unpinned.append(i)
            tri = g.write(os.path.join(workdir, f"b256_{i}.tri"))
            ref = runner.oracle(tri, g.argv(), steps=want["steps"], timeout=1800)
            assert np.array_equal(b.trace(i), runner.trace_array(ref["trace"])), i
            v = sc.view()
            for k in ("accB", "deltaB"):
                assert same_bits(v[k], ref["dump"][k]), (i, k)
    assert len(unpinned) < 8, unpinned
    b.close()
