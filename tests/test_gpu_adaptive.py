"""Adaptive split variant (the reference built with ADAPT + ROLLBACK only):
the device computes each step's corner and centre form factors, the delta-FF
test of every receiver and (speculatively) the form factors of its rand()
sample points; the host runs the receiver loop and the splits.  Results must
equal the reference's adaptive build bit for bit: shooter sequence, split
topology, per-vertex radiosity, .fin bytes."""
import hashlib
import os
import subprocess

import numpy as np
import pytest

import runner
from helpers import golden, golden_index, same_bits, write_case
from hwrad import build, capi, scenes

pytestmark = pytest.mark.gpu

CASES = sorted(k for k, v in golden_index().items() if v.get("adaptive"))


def _adapt(tri, argv, fp64=False, chunks=None):
    o = capi.options_from_argv(argv, precision=64 if fp64 else 32)
    sc = capi.Scene.load(tri, o)
    tree = capi.Octree(sc, 4)
    sc.init()
    ad = capi.Adaptive(sc, tree, o)
    total = 0
    for c in (chunks or []):
        n, conv, _ = ad.run(c)
        total += n
    n, conv, _ = ad.run()
    return sc, ad, total + n, conv


@pytest.mark.parametrize("name", CASES)
def test_adaptive_matches_reference_fixture(built, workdir, name):
    tri, argv, idx = write_case(name, workdir)
    sc, ad, steps, conv = _adapt(tri, argv, chunks=[3, 17])
    g = golden(name)
    assert conv and steps == idx["steps"]
    assert np.array_equal(ad.trace(), g["trace"])
    v = sc.view()
    assert v["n"] == idx["n_slots"]
    for k in ("parent", "p", "accB", "deltaB", "nb"):
        assert same_bits(v[k], g[k]), k
    prefix = os.path.join(workdir, f"ad_{name}")
    sc.write_fin(prefix, 0)
    with open(prefix + ".fin", "rb") as fh:
        assert hashlib.sha256(fh.read()).hexdigest() == idx["fin_sha256"]
    st = ad.stats()
    assert st["splits"] > 0 and st["rays"] > 0


@pytest.mark.parametrize("wait", [False, True])
def test_adaptive_device_sample_points_bench_room(built, workdir, wait):
    """The bench's adaptive workload (100^3 room, 4 boxes, splitting toward
    40,000 slots), 30 steps, in both speculation modes: equal to the oracle
    bit for bit, with sample points taken from the device's speculation.
    Racing (the default), the host takes the points the device has written
    by the time it reads them and evaluates the rest, so the device's share
    depends on how far the kernel runs ahead (about two thirds on a GB300);
    waiting, the host takes every point a speculation covers."""
    s = scenes.room_with_boxes(8, 4, 1, seed=5, size=100.0)
    tri = s.write(os.path.join(workdir, "ad_bench.tri"))
    argv = s.argv({"-triangle": "40000", "-converge": "5"})
    o = capi.options_from_argv(argv)
    sc = capi.Scene.load(tri, o)
    tree = capi.Octree(sc, 4)
    sc.init()
    ad = capi.Adaptive(sc, tree, o)
    ad.set_speculation(wait)
    for c in (1, 9, 20):
        ad.run(c)
    ref = runner.oracle(tri, argv, steps=30, adaptive=True)
    assert np.array_equal(ad.trace(), runner.trace_array(ref["trace"]))
    v = sc.view()
    for k in ("parent", "p", "accB", "deltaB", "nb"):
        assert same_bits(v[k], ref["dump"][k]), k
    st = ad.stats()
    assert st["samples"] > 1000
    assert st["device_points"] > (0.7 if wait else 0.2) * st["samples"]
    assert st["speculations"] >= 30


def test_adaptive_fp64_equals_oracle(built, workdir):
    s = scenes.room_with_boxes(6, 2, 1, seed=12, size=30.0)
    tri = s.write(os.path.join(workdir, "ad64.tri"))
    argv = s.argv({"-triangle": "900", "-converge": "30"})
    sc, ad, steps, conv = _adapt(tri, argv, fp64=True)
    ref = runner.oracle(tri, argv, fp64=True, adaptive=True)
    assert np.array_equal(ad.trace(), runner.trace_array(ref["trace"]))
    v = sc.view()
    for k in ("parent", "p", "accB", "deltaB", "nb"):
        assert same_bits(v[k], ref["dump"][k]), k


def test_adaptive_cli(built, workdir):
    tri, argv, idx = write_case("adapt_room", workdir)
    prefix = os.path.join(workdir, "cli_adapt")
    r = subprocess.run([build.BIN, tri] + argv + ["-adaptive", "-write_cycle", "1000000", "-o", prefix],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    with open(prefix + ".fin", "rb") as fh:
        assert hashlib.sha256(fh.read()).hexdigest() == idx["fin_sha256"]
