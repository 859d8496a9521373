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
    ref = runner.reference_dir()
    if ref and os.path.isdir(os.path.join(ref, "model")):
        for m in ("box", "model2s", "room", "blocks", "church"):
            c.append((m, os.path.join(ref, "model", f"{m}.tri"), ["-triangle", "3000"]))
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


@pytest.mark.parametrize("fp64", [False, True])
def test_cell_thresholds_equal_reference_expression(built, workdir, fp64):
    """The device finds (int)(((double)q - G0) / MinGridLen) from per-axis
    thresholds; on the host the same search must agree with the expression for
    every q in [G0, G1], including values next to each threshold."""
    ft = np.float64 if fp64 else np.float32
    for q_, size in ((8, 10.0), (64, 10.0), (3, 40.0)):
        s = scenes.room_with_boxes(q_, 4, 1, seed=q_, size=size)
        tri = s.write(os.path.join(workdir, f"thr{q_}.tri"))
        sc = capi.Scene.load(tri, capi.options(precision=64 if fp64 else 32))
        tree = capi.Octree(sc, 2)
        v = sc.view()
        rng = np.random.default_rng(q_)
        for axis in range(3):
            g0, g1 = ft(v["G0"][axis]), ft(v["G1"][axis])
            if fp64:   # the view reports corners as float; use the scene's own bounds
                g0, g1 = ft(np.nextafter(g0, np.inf)), ft(np.nextafter(g1, -np.inf))
            q = rng.uniform(g0, g1, 200000).astype(ft)
            ref, fast = tree.cell_coords(axis, q, ft)
            # neighbours of every cell boundary the sample found
            edges = q[np.nonzero(np.diff(ref[np.argsort(q)]))[0]]
            near = np.concatenate([np.nextafter(edges, -np.inf), edges, np.nextafter(edges, np.inf),
                                   np.nextafter(np.nextafter(edges, np.inf), np.inf)]).astype(ft)
            near = near[(near >= g0) & (near <= g1)]
            r2, f2 = tree.cell_coords(axis, near, ft)
            assert np.array_equal(ref, fast)
            assert np.array_equal(r2, f2)
            assert ref.min() >= 0 and ref.max() <= tree.info()["dims"][axis] - 1


def test_oracle_terminates_on_cycling_walks(built, workdir):
    """The reference loops forever on some walks of batch scene 27; the oracle
    (and the solver) stop them by detecting a repeated walk state."""
    g = scenes.batch_rooms(28, seed=4000)[27]
    tri = g.write(os.path.join(workdir, "cyc27.tri"))
    r = runner.oracle(tri, g.argv(), steps=3, timeout=120)
    assert runner.counters(r["stderr"])["loops"] > 0


def test_rand_restatement_equals_libc(built, workdir):
    """The oracle's glibc rand() restatement (used by the adaptive variant's
    sample points, shade.cpp:49-68) against the C library, seed 1."""
    import ctypes
    import subprocess
    libc = ctypes.CDLL(None)
    libc.srand(1)
    want = [libc.rand() for _ in range(2000)]
    src = os.path.join(workdir, "rnd.c")
    with open(src, "w") as fh:
        fh.write('#define main oracle_main\n#include "%s"\n#undef main\n'
                 'int main(void){for(int i=0;i<2000;i++)printf("%%d\\n",glibc_rand());return 0;}\n'
                 % os.path.join(runner.HERE, "radoracle.c"))
    exe = os.path.join(workdir, "rnd")
    subprocess.run(["gcc", "-O2", "-std=c11", "-o", exe, src, "-lm"], check=True, capture_output=True)
    got = [int(x) for x in subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()]
    assert got == want


def test_fp32_forms_equal_double_expressions(workdir):
    """The walk's overshoot (float)((double)t + 0.1) and CalFF's scale
    (float)((double)ff * ((double)a / ((double)d2 * PI))) have FP32 forms
    (add_tenth, ff_scale) that fall back to the double expression only near
    a rounding midpoint.  add_tenth: every float bit pattern; ff_scale: 20 M
    triples, one in eight placed next to a rounding midpoint."""
    import subprocess
    from helpers import build_fp_forms_check
    exe = build_fp_forms_check(workdir)
    r = subprocess.run([exe, "cpu", "1", "20000000"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.split() == ["ok", str(1 << 32), "20000000"]


def test_octree_tables(built, workdir):
    """rad_octree_tables: every cell names a leaf, leaf ranges tile the entry
    list in order, each list is ascending (the reference's order), and every
    entry's triangle meets its leaf's box region (bounds overlap)."""
    s = scenes.room_with_boxes(16, 6, 2, seed=9)
    tri = s.write(os.path.join(workdir, "tables.tri"))
    sc = capi.Scene.load(tri, capi.options())
    t = capi.Octree(sc, 2)
    i, tb = t.info(), t.tables()
    assert len(tb["cell_leaf"]) == int(np.prod(i["dims"]))
    assert tb["cell_leaf"].min() >= 0 and tb["cell_leaf"].max() < i["leaves"]
    rng = tb["leaf_range"]
    assert rng[0, 0] == 0 and rng[-1, 1] == i["entries"]
    assert np.array_equal(rng[1:, 0], rng[:-1, 1])
    ent = tb["entry_tri"]
    for b, e in rng:
        assert np.all(np.diff(ent[b:e]) > 0)
    assert i["ref_list"] == i["entries"] + i["leaves"]
    box = tb["leaf_box"]
    v = sc.view()["p"].reshape(-1, 3, 3)[:sc.view()["n"]]
    lo, hi = v.min(axis=1), v.max(axis=1)
    leaf_of_entry = np.repeat(np.arange(len(rng)), rng[:, 1] - rng[:, 0])
    assert np.all(lo[ent] <= box[leaf_of_entry, 4:7]) and np.all(hi[ent] >= box[leaf_of_entry, 0:3])
