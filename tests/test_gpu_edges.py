"""Edge cases of the device solver against the oracle: an empty scene, a room
without an emitter, a lone emitting triangle and two triangles, in FP32 and
FP64, with one and two shooters per step, alone and inside a batch.  The
oracle itself is held to the reference build on the same inputs in
test_oracle_vs_ref.py."""
import os

import numpy as np
import pytest

import runner
from helpers import EDGE_SCENES, same_bits, write_edge_scene
from hwrad import capi, scenes

pytestmark = pytest.mark.gpu


def _load(tri, argv, fp64=False):
    o = capi.options_from_argv(argv, precision=64 if fp64 else 32)
    sc = capi.Scene.load(tri, o)
    tree = capi.Octree(sc, 2)
    sc.init()
    sc.prepartition()
    return sc, tree, o


@pytest.mark.parametrize("name", EDGE_SCENES)
@pytest.mark.parametrize("fp64", [False, True])
@pytest.mark.parametrize("P", [1, 2])
def test_edge_scene_equals_oracle(built, workdir, name, fp64, P):
    tri, argv = write_edge_scene(name, workdir)
    argv = argv + ["-parallel_src", str(P)]
    sc, tree, o = _load(tri, argv, fp64)
    dv = capi.Device(sc, tree, o)
    n, conv, _ = dv.run()
    assert conv
    dv.download(sc)
    ref = runner.oracle(tri, argv, fp64=fp64)
    want = runner.trace_array(ref["trace"], P)
    assert np.array_equal(dv.trace(), want)
    assert n == len(want)
    v = sc.view()
    assert v["n"] == ref["dump"]["n"]
    for k in ("accB", "deltaB"):
        assert same_bits(v[k], ref["dump"][k]), k
    if n == 0:
        assert dv.stats()["unshot_power"] == 0.0
    prefix = os.path.join(workdir, f"edge_{name}_{int(fp64)}_{P}")
    sc.write_fin(prefix, 0)
    with open(prefix + ".fin", "rb") as fh:
        assert fh.read() == ref["fin"]
    dv.close()


def test_edge_scenes_in_a_batch(built, workdir):
    """Empty, dark and one-triangle scenes among ordinary rooms: each scene of
    the batch equals the oracle, and the batch still converges."""
    preps = []
    for nm in EDGE_SCENES:
        tri, argv = write_edge_scene(nm, workdir)
        preps.append((tri, argv) + _load(tri, argv))
    for i, g in enumerate(scenes.batch_rooms(2, seed=77, lo=500, hi=1500)):
        tri = g.write(os.path.join(workdir, f"edge_room{i}.tri"))
        preps.append((tri, g.argv()) + _load(tri, g.argv()))
    batch = capi.Batch([p[2] for p in preps], [p[3] for p in preps], [p[4] for p in preps])
    _, n_active, _ = batch.run()
    assert n_active == 0
    for i, (tri, argv, s, t, o) in enumerate(preps):
        ref = runner.oracle(tri, argv)
        assert np.array_equal(batch.trace(i), runner.trace_array(ref["trace"])), i
        batch.download(i, s)
        v = s.view()
        for k in ("accB", "deltaB"):
            assert same_bits(v[k], ref["dump"][k]), (i, k)
