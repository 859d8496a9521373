"""GPU solver parity through the C ABI.

Bar: the FP32 solver reproduces the reference's FP32 build bit for bit
(shooter sequence, per-slot accB/deltaB, .fin bytes); the FP64 form
reproduces the reference's float->double build bit for bit.  Where bitwise
equality is not the claim, the tolerance is written in the test.
"""
import hashlib
import os
import subprocess

import numpy as np
import pytest

import runner
from helpers import golden, golden_index, rel_l2, same_bits, write_case
from hwrad import build, capi, scenes

pytestmark = pytest.mark.gpu

CASES = sorted(k for k, v in golden_index().items() if not v.get("adaptive"))


def _solve(tri, argv, fp64=False, chunks=None, schedule=None, layout=None, **kw):
    o = capi.options_from_argv(argv, precision=64 if fp64 else 32, **kw)
    sc = capi.Scene.load(tri, o)
    tree = capi.Octree(sc, 4)
    sc.init()
    sc.prepartition()
    dv = capi.Device(sc, tree, o)
    if schedule is not None:
        dv.set_schedule(*schedule)
    if layout is not None:
        dv.set_layout(layout)
    if chunks:
        total = 0
        for c in chunks:
            n, conv, _ = dv.run(c)
            total += n
            if conv:
                break
        n, conv, _ = dv.run()
        total += n
    else:
        total, conv, _ = dv.run()
    dv.download(sc)
    return sc, dv, total, conv


@pytest.mark.parametrize("name", CASES)
def test_solver_matches_reference_fixture(built, workdir, name):
    tri, argv, idx = write_case(name, workdir)
    sc, dv, steps, conv = _solve(tri, argv, fp64=idx["fp64"])
    g = golden(name)
    assert conv
    assert steps == idx["steps"]
    assert np.array_equal(dv.trace(), g["trace"])
    v = sc.view()
    for k in ("parent", "p", "accB", "deltaB", "nb"):
        assert same_bits(v[k], g[k]), k
    prefix = os.path.join(workdir, f"gpu_{name}")
    sc.write_fin(prefix, 0)
    with open(prefix + ".fin", "rb") as fh:
        assert hashlib.sha256(fh.read()).hexdigest() == idx["fin_sha256"]


def test_chunked_runs_equal_one_run(built, workdir):
    tri, argv, idx = write_case("boxes", workdir)
    sc, dv, steps, conv = _solve(tri, argv, chunks=[1, 7, 33, 100, 2])
    g = golden("boxes")
    assert conv and steps == idx["steps"]
    assert np.array_equal(dv.trace(), g["trace"])
    assert same_bits(sc.view()["accB"], g["accB"])


def test_work_on_the_handle_stream_runs_before_the_next_steps(built, workdir):
    """rad_dev_stream: a caller's kernel enqueued on the handle's stream (here
    an L2-sized write, as the bench's flush) runs before the next steps, with
    no host synchronisation between; the results equal the reference
    fixture's."""
    torch = pytest.importorskip("torch")
    tri, argv, idx = write_case("boxes", workdir)
    o = capi.options_from_argv(argv)
    sc = capi.Scene.load(tri, o)
    tree = capi.Octree(sc, 4)
    sc.init()
    sc.prepartition()
    dv = capi.Device(sc, tree, o)
    ptr = dv.stream()
    assert ptr != 0
    buf = torch.zeros(64 << 20, dtype=torch.float32, device="cuda")
    ext = torch.cuda.ExternalStream(ptr)
    total, conv = 0, False
    for k in range(1, 1 << 20):
        with torch.cuda.stream(ext):
            buf.add_(1.0)
        n, conv, _ = dv.run_timed(1)
        total += n
        if conv:
            break
    torch.cuda.synchronize()
    assert float(buf[0]) == float(k) and float(buf[-1]) == float(k)
    dv.download(sc)
    g = golden("boxes")
    assert conv and total == idx["steps"]
    assert np.array_equal(dv.trace(), g["trace"])
    assert same_bits(sc.view()["accB"], g["accB"])


@pytest.mark.parametrize("P", [2, 5])
def test_parallel_shooters_equal_oracle(built, workdir, P):
    s = scenes.room_with_boxes(8, 4, 1, seed=21, size=20.0)
    tri = s.write(os.path.join(workdir, f"p{P}.tri"))
    argv = s.argv({"-triangle": "1800", "-parallel_src": str(P)})
    sc, dv, steps, conv = _solve(tri, argv)
    ref = runner.oracle(tri, argv)
    assert np.array_equal(dv.trace(), runner.trace_array(ref["trace"], P))
    v = sc.view()
    for k in ("accB", "deltaB"):
        assert same_bits(v[k], ref["dump"][k]), k


def test_large_room_bounded_steps_equal_oracle(built, workdir):
    """The benchmark-size room (64x64-quad walls + 16 boxes, 61,440 triangles)
    for a bounded number of steps."""
    s = scenes.config2()
    tri = s.write(os.path.join(workdir, "config2.tri"))
    argv = s.argv()
    steps = 12
    o = capi.options_from_argv(argv)
    sc = capi.Scene.load(tri, o)
    tree = capi.Octree(sc, 8)
    sc.init()
    sc.prepartition()
    dv = capi.Device(sc, tree, o)
    n, conv, _ = dv.run(steps)
    assert n == steps and not conv
    dv.download(sc)
    ref = runner.oracle(tri, argv, steps=steps)
    assert np.array_equal(dv.trace(), runner.trace_array(ref["trace"]))
    v = sc.view()
    for k in ("accB", "deltaB"):
        assert same_bits(v[k], ref["dump"][k]), k


def test_counters_equal_oracle(built, workdir):
    """Cell, triangle-test and edge-test counts of the walk equal the oracle's
    where no source is split (64x64-quad walls: every edge^2 < 0.1)."""
    s = scenes.room(64)
    tri = s.write(os.path.join(workdir, "cnt64.tri"))
    argv = s.argv()
    o = capi.options_from_argv(argv)
    sc = capi.Scene.load(tri, o)
    tree = capi.Octree(sc, 8)
    sc.init()
    sc.prepartition()
    dv = capi.Device(sc, tree, o)
    dv.set_counting(True)
    dv.run(4)
    st = dv.stats()
    ref = runner.counters(runner.oracle(tri, argv, steps=4)["stderr"])
    assert st["rays"] == ref["rays"] == st["rays_ref"]
    assert (st["cells"], st["tri_tests"], st["se_tests"], st["prec_steps"]) == \
        (ref["cells"], ref["tri_tests"], ref["se_tests"], ref["prec"])


def _ray_set(scene_view, rng, n):
    G0, G1 = scene_view["G0"].astype(np.float64), scene_view["G1"].astype(np.float64)
    P = scene_view["p"].reshape(-1, 3, 3)
    C = scene_view["c"]
    nslot = len(P)
    k = rng.integers(0, nslot, n)
    corner = rng.integers(0, 3, n)
    origin = P[k, corner]
    tgt = C[rng.integers(0, nslot, n)]
    v = (tgt - origin).astype(np.float32)
    ban = scene_view["parent"][k]
    # adversarial: axis-parallel, tiny components, zero components, points on cell planes
    m = n // 4
    v[:m, 1:] = 0
    v[m:2 * m, 0] = np.float32(1e-7)
    v[2 * m:3 * m] = rng.normal(size=(m, 3)).astype(np.float32) * np.float32(1e-3)
    lo, hi = G0 + 1e-3, G1 - 1e-3
    origin[3 * m:] = rng.uniform(lo, hi, size=(n - 3 * m, 3)).astype(np.float32)
    return origin.astype(np.float32), v, ban.astype(np.int32)


@pytest.mark.parametrize("fp64", [False, True])
def test_ray_walk_equals_oracle(built, workdir, fp64):
    s = scenes.room_with_boxes(16, 10, 2, seed=5)
    tri = s.write(os.path.join(workdir, "rays.tri"))
    argv = s.argv()
    o = capi.options_from_argv(argv, precision=64 if fp64 else 32)
    sc = capi.Scene.load(tri, o)
    tree = capi.Octree(sc, 4)
    sc.init()
    sc.prepartition()
    dv = capi.Device(sc, tree, o)
    rng = np.random.default_rng(1234)
    p, v, ban = _ray_set(sc.view(), rng, 20000)
    ft = np.float64 if fp64 else np.float32
    got = dv.ray_hit(p.astype(ft), v.astype(ft), ban, dtype=ft)
    want = runner.rays(tri, argv, p.astype(ft), v.astype(ft), ban, fp64=fp64)
    assert np.array_equal(got, want)
    assert (got >= 0).mean() > 0.2      # the set exercises hits and misses
    assert (got < 0).mean() > 0.01


def test_form_factors_equal_oracle(built, workdir):
    s = scenes.room_with_boxes(12, 6, 2, seed=8, size=15.0)
    tri = s.write(os.path.join(workdir, "ff.tri"))
    argv = s.argv()
    o = capi.options_from_argv(argv)
    sc = capi.Scene.load(tri, o)
    tree = capi.Octree(sc, 4)
    sc.init()
    sc.prepartition()
    dv = capi.Device(sc, tree, o)
    v = sc.view()
    rcv = np.arange(v["n"], dtype=np.int32)
    # a large (split) source and a small (unsplit) box face
    sizes = np.array([((p[3:6] - p[0:3]) ** 2).sum() for p in v["p"]])
    for src in (int(np.argmax(sizes)), int(np.argmin(sizes))):
        got = dv.form_factors(src, rcv)
        want = runner.form_factors(tri, argv, src, rcv)
        assert same_bits(got, want), src
        assert (got > 0).any()


def test_walk_cap_reports_error(built, workdir):
    s = scenes.room(8)
    tri = s.write(os.path.join(workdir, "cap.tri"))
    o = capi.options_from_argv(s.argv(), walk_cap=2)
    sc = capi.Scene.load(tri, o)
    tree = capi.Octree(sc, 2)
    sc.init()
    sc.prepartition()
    dv = capi.Device(sc, tree, o)
    n, conv, rc = dv.run(3)
    assert rc == capi.RAD_ERR_WALK
    assert dv.stats()["walk_cap_hits"] > 0


@pytest.mark.parametrize("autotune", [False, True])
def test_cli_outputs_equal_oracle(built, workdir, autotune):
    tri, argv, idx = write_case("room8", workdir)
    prefix = os.path.join(workdir, f"cli_room8_{int(autotune)}")
    r = subprocess.run([build.BIN, tri] + argv + ["-write_cycle", "250", "-o", prefix] + (["-autotune"] if autotune else []),
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    if autotune:
        assert "autotuned over 64 loops" in r.stderr
    assert "Complete in #Iterations 744" in r.stderr
    with open(prefix + ".fin", "rb") as fh:
        assert hashlib.sha256(fh.read()).hexdigest() == idx["fin_sha256"]
    # intermediate outputs every 250 loops equal the oracle's
    od = os.path.join(workdir, "cli_oracle")
    os.makedirs(od, exist_ok=True)
    subprocess.run([runner.ORACLE32, tri] + argv + ["-write_cycle", "250", "-o", os.path.join(od, "o")],
                   check=True, capture_output=True)
    for loop in (250, 500):
        with open(f"{prefix}.{loop}", "rb") as a, open(os.path.join(od, f"o.{loop}"), "rb") as b:
            assert a.read() == b.read(), loop
    assert not os.path.exists(f"{prefix}.750")


def test_fp32_form_error_against_fp64_oracle(built, workdir):
    """Reported, not a parity claim: the FP32 solver against the FP64 oracle
    on the 768-triangle room, next to the reference-vs-reference gap."""
    tri, argv, idx = write_case("room8", workdir)
    sc32, _, _, _ = _solve(tri, argv)
    g64 = golden("room8_fp64")
    e_gpu = rel_l2(sc32.view()["accB"], g64["accB"])
    e_ref = rel_l2(golden("room8")["accB"], g64["accB"])
    assert e_gpu == pytest.approx(e_ref, rel=0, abs=0)   # identical, as the FP32 solver equals the FP32 build


@pytest.mark.parametrize("fp64", [False, True])
def test_unshot_power_monitor(built, workdir, fp64):
    """rad_stats.unshot_power: the FP64 total of (dB_r + dB_g + dB_b) * area over
    live slots, reduced on the device in a fixed order.  Equal to the same sum
    over the downloaded slots (to summation-order rounding), the same on
    repeated calls, and non-increasing from step to step (each step zeroes the
    shooter's unshot energy and passes on at most a reflectance < 1 of it)."""
    sc = scenes.room_with_boxes(12, 6, 2, seed=7, size=30.0)
    tri = sc.write(os.path.join(workdir, f"unshot{int(fp64)}.tri"))
    o = capi.options_from_argv(sc.argv({"-triangle": "4000"}), precision=64 if fp64 else 32)
    scene = capi.Scene.load(tri, o)
    tree = capi.Octree(scene, 2)
    scene.init()
    scene.prepartition()
    dv = capi.Device(scene, tree, o)
    prev = None
    for _ in range(6):
        dv.run(7)
        a = dv.stats()["unshot_power"]
        assert dv.stats()["unshot_power"] == a
        dv.download(scene)
        v = scene.view()
        live = v["parent"] >= 0
        db = v["deltaB"].astype(np.float64)
        want = float(np.sum((db[:, 0] + db[:, 1] + db[:, 2])[live] * v["area"].astype(np.float64)[live]))
        assert abs(a - want) <= 1e-12 * abs(want)
        if prev is not None:
            assert a <= prev
        prev = a
    dv.close()



SPLIT_ALWAYS = (0.0, 0.0, 0.0, 0.0)   # every group shot as 2-slot items, 4 lanes per corner, from step 2 on
SPLIT_NEVER = (1e9, 1e9, 1e9, 1e9)


@pytest.mark.parametrize("name", [c for c in CASES if not golden_index()[c].get("P", 1) > 1])
@pytest.mark.parametrize("schedule", [SPLIT_ALWAYS, SPLIT_NEVER], ids=["split_always", "split_never"])
@pytest.mark.parametrize("layout", [1, 2])
def test_schedule_does_not_change_results(built, workdir, name, schedule, layout):
    """The schedule (which groups are split, which start early) and the
    kernel form change only timing.  Form 1 splits a group into 2-slot items
    with 4 lanes per corner, form 2 into 3-slot items on one lane.  With every
    group split from the second step on (in form 1 the 4-lane walk and its NaN
    fallback everywhere, FP32 and FP64) and with nothing split, the results
    equal the reference fixture bit for bit."""
    tri, argv, idx = write_case(name, workdir)
    if layout == 2 and idx["fp64"]:
        pytest.skip("the FP64 solver has only form 1")
    sc, dv, steps, conv = _solve(tri, argv, fp64=idx["fp64"], schedule=schedule, layout=layout)
    assert dv.layout == layout
    g = golden(name)
    assert conv
    assert steps == idx["steps"]
    assert np.array_equal(dv.trace(), g["trace"])
    v = sc.view()
    for k in ("parent", "p", "accB", "deltaB", "nb"):
        assert same_bits(v[k], g[k]), k


def test_split_schedule_on_hall_steps(built, workdir):
    """The 422k-triangle hall, 40 steps, in both kernel forms with every group
    split and with nothing split: all four runs equal (the first steps of the
    automatic choice are held to the oracle by
    test_hall_bounded_steps_equal_oracle)."""
    sc_gen = scenes.hall()
    tri = sc_gen.write(os.path.join(workdir, "hall_split.tri"))
    out = []
    for layout, sched in ((1, SPLIT_ALWAYS), (1, SPLIT_NEVER), (2, SPLIT_ALWAYS), (2, SPLIT_NEVER), (0, None)):
        o = capi.options_from_argv(sc_gen.argv())
        sc = capi.Scene.load(tri, o)
        tree = capi.Octree(sc, 8)
        sc.init()
        sc.prepartition()
        dv = capi.Device(sc, tree, o)
        if layout:
            dv.set_schedule(*sched)
            dv.set_layout(layout)
            assert dv.layout == layout
            dv.run(40)
        else:   # both forms timed on the scene's own steps, then the faster kept
            n, conv, form = dv.autotune(8, 40)
            assert n == 40 and not conv and form in (1, 2)
        dv.download(sc)
        v = sc.view()
        out.append((dv.trace().copy(), v["accB"].copy(), v["deltaB"].copy()))
        dv.close()
    for o in out[1:]:
        assert np.array_equal(out[0][0], o[0])
        assert same_bits(out[0][1], o[1])
        assert same_bits(out[0][2], o[2])


def test_layout_choice(built, workdir):
    """The automatic form: 1 for a scene with few groups per resident warp,
    2 above 4 (FP32, one shooter per step); several shooters per step and FP64
    stay in form 1 whatever is asked."""
    tri, argv, idx = write_case("room8", workdir)
    o = capi.options_from_argv(argv)
    sc = capi.Scene.load(tri, o)
    tree = capi.Octree(sc, 4)
    sc.init()
    sc.prepartition()
    dv = capi.Device(sc, tree, o)
    assert dv.layout == 1
    dv.set_layout(2)
    assert dv.layout == 2
    dv.set_layout(0)
    assert dv.layout == 1
    with pytest.raises(capi.RadError):
        dv.set_layout(3)
    dv.close()
    for name in ("room8_p3", "room8_fp64"):
        tri, argv, idx = write_case(name, workdir)
        o = capi.options_from_argv(argv, precision=64 if idx["fp64"] else 32)
        sc = capi.Scene.load(tri, o)
        tree = capi.Octree(sc, 4)
        sc.init()
        sc.prepartition()
        dv = capi.Device(sc, tree, o)
        dv.set_layout(2)
        assert dv.layout == 1, name
        dv.close()


@pytest.mark.parametrize("name", ["room8", "bigroom", "room8_fp64", "room8_p3"])
def test_autotune_does_not_change_results(built, workdir, name):
    """rad_dev_autotune shoots ordinary steps in both forms and keeps the
    faster; the solution equals the reference fixture bit for bit.  FP64 and
    several shooters per step have one form: the steps just run."""
    tri, argv, idx = write_case(name, workdir)
    o = capi.options_from_argv(argv, precision=64 if idx["fp64"] else 32)
    sc = capi.Scene.load(tri, o)
    tree = capi.Octree(sc, 4)
    sc.init()
    sc.prepartition()
    dv = capi.Device(sc, tree, o)
    n, conv, form = dv.autotune(4, 50)
    assert n == 50 and not conv
    assert form == dv.layout
    if idx["fp64"] or idx.get("P", 1) > 1:
        assert form == 1
    else:
        assert form in (1, 2)
    m, conv, _ = dv.run()
    assert conv and n + m == idx["steps"]
    dv.download(sc)
    g = golden(name)
    assert np.array_equal(dv.trace(), g["trace"])
    v = sc.view()
    for k in ("parent", "p", "accB", "deltaB", "nb"):
        assert same_bits(v[k], g[k]), k
    with pytest.raises(capi.RadError):
        dv.autotune(0, 10)
