"""The octree built with its overlap tests on the device against the host
build: the same leaves (box and list, bit for bit), the same cell-to-leaf map
up to leaf numbering, the same reference counts, and solver results that
equal the reference fixtures when the device-built tree is used."""
import hashlib
import os
import subprocess

import numpy as np
import pytest

from helpers import golden, same_bits, write_case
from hwrad import build, capi, scenes

pytestmark = pytest.mark.gpu


def _leaf_keys(t):
    """Canonical key per leaf: box bytes + list bytes."""
    box, rng, ent = t["leaf_box"], t["leaf_range"], t["entry_tri"]
    return [box[l].tobytes() + ent[rng[l, 0]:rng[l, 1]].tobytes() for l in range(len(box))]


def _assert_same_tree(a, b):
    ia, ib = a.info(), b.info()
    assert ia == ib
    ta, tb = a.tables(), b.tables()
    # the cell map agrees up to a renumbering of the leaves
    ha, hb = ta["cell_leaf"], tb["cell_leaf"]
    m = np.full(ia["leaves"], -1, np.int64)
    m[ha] = hb
    assert np.array_equal(m[ha], hb)
    inv = np.full(ib["leaves"], -1, np.int64)
    inv[hb] = ha
    assert np.array_equal(inv[hb], ha)
    # the leaves (box and list) agree as sets, and pair up through the cell map
    ka, kb = _leaf_keys(ta), _leaf_keys(tb)
    assert sorted(ka) == sorted(kb)
    used = np.unique(ha)
    assert all(ka[l] == kb[m[l]] for l in used)


@pytest.mark.parametrize("fp64", [False, True])
@pytest.mark.parametrize("which", ["room8", "boxes", "config2", "precision"])
def test_device_octree_equals_host_octree(built, workdir, which, fp64):
    gen = {"room8": lambda: scenes.room(8), "boxes": lambda: scenes.room_with_boxes(16, 10, 2, seed=5),
           "config2": scenes.config2, "precision": scenes.precision_stress}[which]()
    tri = gen.write(os.path.join(workdir, f"oct_{which}.tri"))
    o = capi.options_from_argv(gen.argv(), precision=64 if fp64 else 32)
    sc = capi.Scene.load(tri, o)
    _assert_same_tree(capi.Octree(sc, 4), capi.Octree(sc, device=0))


def test_device_octree_hall(built, workdir):
    gen = scenes.hall()
    tri = gen.write(os.path.join(workdir, "oct_hall.tri"))
    o = capi.options_from_argv(gen.argv())
    sc = capi.Scene.load(tri, o)
    _assert_same_tree(capi.Octree(sc, 8), capi.Octree(sc, device=0))


@pytest.mark.parametrize("name", ["room8", "bigroom", "room8_fp64"])
def test_solver_with_device_octree_matches_fixture(built, workdir, name):
    tri, argv, idx = write_case(name, workdir)
    o = capi.options_from_argv(argv, precision=64 if idx["fp64"] else 32)
    sc = capi.Scene.load(tri, o)
    tree = capi.Octree(sc, device=0)
    sc.init()
    sc.prepartition()
    dv = capi.Device(sc, tree, o)
    n, conv, _ = dv.run()
    assert conv and n == idx["steps"]
    dv.download(sc)
    g = golden(name)
    assert np.array_equal(dv.trace(), g["trace"])
    v = sc.view()
    for k in ("accB", "deltaB"):
        assert same_bits(v[k], g[k]), k


@pytest.mark.parametrize("flags", [["-octree_host"], ["-init_host"], ["-octree_host", "-init_host"]])
def test_cli_host_preparation(built, workdir, flags):
    """./rad builds the octree and the neighbour links on the GPU by default;
    -octree_host and -init_host give the host forms, with the same output."""
    tri, argv, idx = write_case("room8", workdir)
    prefix = os.path.join(workdir, "cli_" + "_".join(f.strip("-") for f in flags))
    r = subprocess.run([build.BIN, tri] + argv + flags + ["-o", prefix], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stderr
    with open(prefix + ".fin", "rb") as fh:
        assert hashlib.sha256(fh.read()).hexdigest() == idx["fin_sha256"]


def test_preparation_on_many_host_threads(built):
    """Octrees and neighbour links of 24 batch rooms built on the device from
    8 host threads at once (each thread with its own stream and device
    scratch, kept between its calls) equal the host builds."""
    from concurrent.futures import ThreadPoolExecutor
    gens = scenes.batch_rooms(24, seed=61, lo=500, hi=8000)

    def dev(g):
        o = capi.options_from_argv(g.argv())
        sc = capi.Scene.from_arrays(g.vtx, g.frgb, g.brgb, o)
        t = capi.Octree(sc, device=0)
        sc.init(device=0)
        return sc, t

    with ThreadPoolExecutor(8) as ex:
        got = list(ex.map(dev, gens))
    for g, (sc, t) in zip(gens, got):
        o = capi.options_from_argv(g.argv())
        sh = capi.Scene.from_arrays(g.vtx, g.frgb, g.brgb, o)
        th = capi.Octree(sh, 2)
        sh.init()
        _assert_same_tree(t, th)
        assert same_bits(sc.view()["nb"], sh.view()["nb"])
