"""Batched form: every scene's result equals the single-scene solver's, bit for bit."""
import os

import numpy as np
import pytest

import runner
from helpers import same_bits
from hwrad import capi, scenes

pytestmark = pytest.mark.gpu


def _prep(sc, workdir, name, extra=None, **kw):
    tri = sc.write(os.path.join(workdir, f"{name}.tri"))
    argv = sc.argv(extra)
    o = capi.options_from_argv(argv, **kw)
    s = capi.Scene.load(tri, o)
    t = capi.Octree(s, 2)
    s.init()
    s.prepartition()
    return tri, argv, o, s, t


def _scenes():
    out = [scenes.room(4, emitter=(0.25, 0.75)), scenes.room(8), scenes.room(8, size=100.0),
           scenes.room_with_boxes(6, 3, 1, seed=3, size=20.0), scenes.room(12, size=10.0),
           scenes.room_with_boxes(10, 8, 1, seed=9)]
    out += scenes.batch_rooms(6, seed=77, lo=500, hi=4000)
    extras = [None, None, {"-triangle": "1500"}, {"-triangle": "1200"}, None, None] + [None] * 6
    return out, extras


def test_batch_equals_single_scene(built, workdir):
    scs, extras = _scenes()
    preps = [_prep(sc, workdir, f"b{i}", extras[i]) for i, sc in enumerate(scs)]
    batch = capi.Batch([p[3] for p in preps], [p[4] for p in preps], [p[2] for p in preps])
    total, n_active, _ = batch.run()
    assert n_active == 0
    steps = []
    for i, (tri, argv, o, s, t) in enumerate(preps):
        # the same scene through the single-scene solver, from a fresh host copy
        s2 = capi.Scene.load(tri, o)
        t2 = capi.Octree(s2, 2)
        s2.init()
        s2.prepartition()
        dv = capi.Device(s2, t2, o)
        n, conv, _ = dv.run()
        assert conv
        dv.download(s2)
        st, cv = batch.scene_stats(i)
        assert cv and st == n, i
        assert np.array_equal(batch.trace(i), dv.trace()), i
        batch.download(i, s)
        a, b = s.view(), s2.view()
        for k in ("accB", "deltaB"):
            assert same_bits(a[k], b[k]), (i, k)
        steps.append(n)
    assert len(set(steps)) > 3          # scenes converge at different iterations
    assert total == max(steps) + 1      # the last iteration finds every scene converged


def test_batch_chunks_and_oracle(built, workdir):
    scs = scenes.batch_rooms(4, seed=5, lo=500, hi=3000)
    preps = [_prep(sc, workdir, f"bc{i}") for i, sc in enumerate(scs)]
    batch = capi.Batch([p[3] for p in preps], [p[4] for p in preps], [p[2] for p in preps])
    for k in (1, 3, 29, 64):
        batch.run(k)
    batch.run()
    for i, (tri, argv, o, s, t) in enumerate(preps):
        ref = runner.oracle(tri, argv)
        assert np.array_equal(batch.trace(i), runner.trace_array(ref["trace"])), i
        batch.download(i, s)
        v = s.view()
        for k in ("accB", "deltaB"):
            assert same_bits(v[k], ref["dump"][k]), (i, k)


def _single(tri, o):
    """The single-scene solver on a fresh host copy of a scene, to convergence."""
    s2 = capi.Scene.load(tri, o)
    t2 = capi.Octree(s2, 2)
    s2.init()
    s2.prepartition()
    dv = capi.Device(s2, t2, o)
    n, conv, _ = dv.run()
    assert conv
    dv.download(s2)
    return s2, dv, n


def _check_batch_against_single(batch, preps):
    for i, (tri, argv, o, s, t) in enumerate(preps):
        s2, dv, n = _single(tri, o)
        st, cv = batch.scene_stats(i)
        assert cv and st == n, i
        assert np.array_equal(batch.trace(i), dv.trace()), i
        batch.download(i, s)
        a, b = s.view(), s2.view()
        for k in ("accB", "deltaB"):
            assert same_bits(a[k], b[k]), (i, k)
        dv.close()


def _mode_scenes():
    return scenes.batch_rooms(4, seed=91, lo=500, hi=2500) + [scenes.room_with_boxes(6, 3, 1, seed=3, size=20.0),
                                                             scenes.room(8, size=100.0)]


@pytest.mark.parametrize("P", [2, 5])
def test_batch_parallel_shooters_equal_single_scene(built, workdir, P):
    """-parallel_src P > 1 in the batched form: listCanditate's top n per scene
    (a selection kernel with one CTA per scene), every scene bit-equal to the
    single-scene solver with the same P, trace P entries per step."""
    scs = _mode_scenes()
    preps = [_prep(sc, workdir, f"bp{P}_{i}", {"-triangle": "1500", "-parallel_src": str(P)})
             for i, sc in enumerate(scs)]
    batch = capi.Batch([p[3] for p in preps], [p[4] for p in preps], [p[2] for p in preps])
    _, n_active, _ = batch.run()
    assert n_active == 0
    assert batch.trace(0).shape[1] == P
    _check_batch_against_single(batch, preps)


@pytest.mark.parametrize("P", [1, 3])
def test_batch_fp64_equals_single_scene(built, workdir, P):
    """The all-FP64 form batched: every scene bit-equal to the single-scene
    FP64 solver (which is bit-equal to the reference's float->double build)."""
    scs = _mode_scenes()
    preps = [_prep(sc, workdir, f"b64_{P}_{i}", {"-triangle": "1500", "-parallel_src": str(P)}, precision=64)
             for i, sc in enumerate(scs)]
    batch = capi.Batch([p[3] for p in preps], [p[4] for p in preps], [p[2] for p in preps])
    assert batch.form == 2
    _, n_active, _ = batch.run()
    assert n_active == 0
    _check_batch_against_single(batch, preps)


def test_batch_fp64_against_fp64_oracle(built, workdir):
    scs = scenes.batch_rooms(3, seed=17, lo=500, hi=2000)
    preps = [_prep(sc, workdir, f"b64o_{i}", precision=64) for i, sc in enumerate(scs)]
    batch = capi.Batch([p[3] for p in preps], [p[4] for p in preps], [p[2] for p in preps])
    batch.run()
    for i, (tri, argv, o, s, t) in enumerate(preps):
        ref = runner.oracle(tri, argv, fp64=True)
        assert np.array_equal(batch.trace(i), runner.trace_array(ref["trace"])), i
        batch.download(i, s)
        for k in ("accB", "deltaB"):
            assert same_bits(s.view()[k], ref["dump"][k]), (i, k)


def test_batch_forms_and_autotune_do_not_change_results(built, workdir):
    """Both shooting-kernel forms (4 and 3 CTAs per SM), switched between
    chunks and chosen by the autotuner, give the same bits."""
    scs = scenes.batch_rooms(5, seed=33, lo=500, hi=3000)
    preps = [_prep(sc, workdir, f"bf{i}") for i, sc in enumerate(scs)]
    batch = capi.Batch([p[3] for p in preps], [p[4] for p in preps], [p[2] for p in preps])
    assert batch.form == 1
    chosen = batch.autotune(2, 2)
    assert chosen in (1, 2) and batch.form == chosen
    for k, form in enumerate((2, 1, 2, 1)):
        batch.set_form(form)
        batch.run(3 + k)
    batch.run()
    _check_batch_against_single(batch, preps)


def test_batch_rejects_mixed_modes(built, workdir):
    sc = scenes.room(4, emitter=(0.25, 0.75))
    tri = sc.write(os.path.join(workdir, "brej.tri"))
    o1 = capi.options_from_argv(sc.argv())
    o2 = capi.options_from_argv(sc.argv(), parallel_src=2)
    s = capi.Scene.load(tri, o1)
    t = capi.Octree(s, 2)
    s.init()
    with pytest.raises(capi.RadError):
        capi.Batch([s, s], [t, t], [o1, o2])
    o64 = capi.options_from_argv(sc.argv(), precision=64)
    with pytest.raises(capi.RadError):
        capi.Batch([s], [t], [o64])


def test_walks_the_reference_never_finishes(built, workdir):
    """Scene 27 of the 256-room batch: the reference's TreeNodeNum returns leaves
    that do not contain the point (GridNum truncates to 63), and tens of
    thousands of walks cycle forever in the reference.  The solver and the
    oracle both stop a walk whose (t, prev) state repeats and treat the ray as
    blocked; they must agree bit for bit."""
    g = scenes.batch_rooms(28, seed=4000)[27]
    tri, argv, o, s, t = _prep(g, workdir, "loop27")
    dv = capi.Device(s, t, o)
    n, conv, _ = dv.run(6)
    assert n == 6
    dv.download(s)
    assert dv.stats()["walk_loops"] > 1000
    ref = runner.oracle(tri, argv, steps=6)
    assert runner.counters(ref["stderr"])["loops"] > 1000
    assert np.array_equal(dv.trace(), runner.trace_array(ref["trace"]))
    v = s.view()
    for k in ("accB", "deltaB"):
        assert same_bits(v[k], ref["dump"][k]), k
