"""InitRadiosity with the neighbour links found on the device: the links, and
everything the pre-partition then builds from them, equal the host form bit
for bit; the solver's results with it equal the reference fixtures."""
import os

import numpy as np
import pytest

from helpers import EDGE_SCENES, golden, same_bits, write_case, write_edge_scene
from hwrad import capi, scenes

pytestmark = pytest.mark.gpu

FIELDS = ("parent", "p", "accB", "deltaB", "area", "n_", "c", "Frgb", "nb")


def _both(tri, o):
    a = capi.Scene.load(tri, o)
    b = capi.Scene.load(tri, o)
    a.init()
    b.init(device=0)
    return a, b


@pytest.mark.parametrize("fp64", [False, True])
@pytest.mark.parametrize("which", ["room8", "boxes", "config2", "precision", "batch3", "hall"])
def test_device_links_equal_host_links(built, workdir, which, fp64):
    gen = {"room8": lambda: scenes.room(8), "boxes": lambda: scenes.room_with_boxes(16, 10, 2, seed=5),
           "config2": scenes.config2, "precision": scenes.precision_stress,
           "batch3": lambda: scenes.batch_rooms(4, seed=4000)[3], "hall": scenes.hall}[which]()
    if which == "hall" and fp64:
        pytest.skip("the FP32 hall covers the large case")
    tri = gen.write(os.path.join(workdir, f"init_{which}.tri"))
    o = capi.options_from_argv(gen.argv(), precision=64 if fp64 else 32)
    a, b = _both(tri, o)
    va, vb = a.view(), b.view()
    assert (va["nb"] >= 0).any()
    for k in FIELDS:
        assert same_bits(va[k], vb[k]), k
    assert a.log(1) == b.log(1) and a.log(2) == b.log(2)
    a.prepartition()
    b.prepartition()
    va, vb = a.view(), b.view()
    assert va["n"] == vb["n"]
    for k in FIELDS:
        assert same_bits(va[k], vb[k]), k


@pytest.mark.parametrize("name", EDGE_SCENES)
def test_device_links_on_edge_scenes(built, workdir, name):
    tri, argv = write_edge_scene(name, workdir)
    a, b = _both(tri, capi.options_from_argv(argv))
    assert same_bits(a.view()["nb"], b.view()["nb"])


@pytest.mark.parametrize("name", ["room8", "boxes", "room8_fp64"])
def test_solver_with_device_init_matches_fixture(built, workdir, name):
    tri, argv, idx = write_case(name, workdir)
    o = capi.options_from_argv(argv, precision=64 if idx["fp64"] else 32)
    sc = capi.Scene.load(tri, o)
    tree = capi.Octree(sc, device=0)
    sc.init(device=0)
    sc.prepartition()
    dv = capi.Device(sc, tree, o)
    n, conv, _ = dv.run()
    assert conv and n == idx["steps"]
    dv.download(sc)
    g = golden(name)
    assert np.array_equal(dv.trace(), g["trace"])
    v = sc.view()
    for k in ("parent", "p", "accB", "deltaB", "nb"):
        assert same_bits(v[k], g[k]), k
