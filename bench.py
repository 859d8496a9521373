#!/usr/bin/env python3
"""Benchmark: shooter steps per second of the progressive-refinement loop.

Workload: the 64x64-quad room with 16 seeded boxes (61,440 triangles,
-converge at 1e-4 of an emitter's key, -adapt_area 5 -delta_ff 5e-6
-triangle 200000), FP32 solver.  A step is one shooter step: select the
shooter and shoot it to every receiver (the reference's parallelRadiosity).

Our arm (default): the scene is resident in HBM; W warm-up steps, then K
timed steps, each timed on the device with CUDA events on the solver's own
stream; L2 is flushed (a 512 MB write) before every timed step because the
scene is smaller than L2.  Also reported:
  roofline      the shooting kernel's algorithmic bytes per launch (176 B per
                slot streamed + 8 B per walk cell, 24 B per triangle test,
                48 B per edge test, counts taken exactly from a counting pass
                over the same steps) over its event-timed duration, against
                the measured HBM copy bandwidth;
  e2e           the same steps through the C ABI from host buffers: device
                upload of the scene, K steps, download of the results;
  cpu_baseline  the reference's own CPU solver (built from its sources, when
                available; else the C restatement) on the machine's host cores.
  hall          the config-3 hall (422,429 slots) in the solver's chosen form
                and the other one, L2 flushed before each timed step.
--impl reference times the reference's CPU solver alone on the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(REPO, "hw-radiosity_gb300"))

WORKLOAD = "room64x64_boxes16 (61,440 triangles, config 2), FP32, plain single-scene form"
L2_NOTE = ("GPU arm: flushed (512 MB write, enqueued on the solver's stream) before every timed step; "
           "CPU arm: not applicable")
# the k_shoot sources whose ncu capture gave the committed DRAM traffic figure
KERNEL_SOURCES = ("hw-radiosity_gb300/csrc/rad_dev.cu", "hw-radiosity_gb300/csrc/rad_kernels.cuh")
TRAFFIC_FILE = "profiles/k_shoot_room64_boxes16.traffic.txt"


def kernel_source_sha():
    import hashlib
    h = hashlib.sha256()
    for f in KERNEL_SOURCES:
        with open(os.path.join(REPO, f), "rb") as fh:
            h.update(fh.read())
    return h.hexdigest()[:16]


def committed_traffic():
    """DRAM bytes per k_shoot launch from the committed ncu capture, and whether
    it was captured from the kernel sources as they are now."""
    path = os.path.join(REPO, TRAFFIC_FILE)
    if not os.path.exists(path):
        return None, None
    vals = {}
    for line in open(path):
        if ":" in line and not line.startswith("#"):
            k, v = line.split(":", 1)
            vals[k.strip()] = v.strip()
    traffic = int(vals["dram_bytes_per_launch"]) if "dram_bytes_per_launch" in vals else None
    src = vals.get("kernel_sources_sha256_16")
    return traffic, {"captured_from_sources": src, "current_sources": kernel_source_sha(),
                     "matches": src == kernel_source_sha()}
BYTES_PER_SLOT = 176       # selection key 16 + receiver read 112 + receiver write 48
BYTES_PER_CELL = 8
BYTES_PER_TRI_TEST = 24
BYTES_PER_SE_TEST = 48


_T0 = time.time()


def log(msg):
    """Progress on stderr (the JSON line is the only stdout output)."""
    print(f"[bench {time.time() - _T0:8.1f}s] {msg}", file=sys.stderr, flush=True)


def _peaks():
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled while the GPU works."""

    def __init__(self, index: int):
        self.index = index
        self.samples = []
        self.proc = None
        self.thread = None

    def start(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, FileNotFoundError):
            self.proc = None
            return

        def reader():
            for line in self.proc.stdout:
                f = [x.strip() for x in line.split(",")]
                if len(f) >= 9:
                    self.samples.append(f)

        self.thread = threading.Thread(target=reader, daemon=True)
        self.thread.start()

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        if self.thread:
            self.thread.join(timeout=5)

    def summary(self):
        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        sm = [num(s[1]) for s in self.samples if num(s[1]) is not None]
        mx = [num(s[2]) for s in self.samples if num(s[2]) is not None]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for s in self.samples:
            for k, name in enumerate(names):
                if s[5 + k].lower().startswith("active"):
                    reasons.add(name)
        loaded = [x for x in sm if mx and x >= 0.5 * max(mx)] or sm
        return {"sm_mhz": statistics.median(loaded) if loaded else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.samples)}


def _nproc():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def _scene_file(tmp):
    from hwrad import scenes
    sc = scenes.config2()
    return sc, sc.write(os.path.join(tmp, "config2.tri"))


def cpu_reference(tri, argv, warmup, steps, jobs=None):
    """Time the reference's CPU solver, built from its sources with its own
    Makefile flags (oracle/_ref/rad_ref_shipped), over steps [warmup,
    warmup+steps) from its per-step timestamps.  There is no fallback: without
    the reference build this raises."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import runner
    cores = _nproc()
    if not os.path.exists(runner.REF_SHIPPED):
        runner.build_ref()
    if not os.path.exists(runner.REF_SHIPPED):
        raise RuntimeError("the reference CPU solver (oracle/_ref/rad_ref_shipped) is not built: "
                           "no reference sources were staged under oracle/_ref")
    jobs = jobs or cores
    wd = tempfile.mkdtemp(prefix="radcpu_")
    times = os.path.join(wd, "times.txt")
    t0 = time.time()
    out = runner.run(runner.REF_SHIPPED, tri, list(argv) + ["-jobs", str(jobs)], steps=warmup + steps,
                     env={"RAD_TIMES": times}, workdir=wd, timeout=3600)
    wall = time.time() - t0
    stamps = [float(x) for x in open(times).read().split()]
    # stamp k = start of step k (0-based); the last stamp is the call that stopped the loop
    a, b = stamps[warmup], stamps[min(warmup + steps, len(stamps) - 1)]
    n = min(warmup + steps, len(stamps) - 1) - warmup
    return {"value": n / (b - a) if b > a else None, "unit": "shots/s", "cores": jobs, "kind": "reference",
            "build": runner.REF_SHIPPED_FLAGS,
            "sample": f"steps {warmup}..{warmup + n} of the workload ({n} shooter steps after {warmup} "
                      f"warm-up steps; {wall:.1f} s wall including the solver's own init)",
            "seconds": b - a, "slots": int(out["dump"]["n"])}


SIZE_BANDS = ((0, 2000, "<2k"), (2000, 10000, "2k-10k"), (10000, 1 << 40, ">10k"))


def prepare_scenes(capi, gens, device, threads=None):
    """Scenes from the generator's arrays; octree and InitRadiosity's
    neighbour links on the device, pre-partition on the host.  Scenes are
    prepared on several host threads at once (each with its own stream and
    device scratch in the library); the calls release the GIL."""
    from concurrent.futures import ThreadPoolExecutor

    def one(g):
        o = capi.options_from_argv(g.argv(), jobs=_nproc())
        sc = capi.Scene.from_arrays(g.vtx, g.frgb, g.brgb, o)
        tr = capi.Octree(sc, device=device)
        sc.init(device=device)
        sc.prepartition()
        return sc, tr, o
    with ThreadPoolExecutor(max_workers=threads or min(16, _nproc())) as ex:
        return list(ex.map(one, gens))


def _batch(capi, preps, device, form=None):
    b = capi.Batch([p[0] for p in preps], [p[1] for p in preps], [p[2] for p in preps], device)
    if form:
        b.set_form(form)
    return b


def measure_batched(capi, n_scenes, warmup, iters, device, world=1, rank=0, ranks=None):
    """Config 4: n_scenes seeded rooms (triangles log-uniform in [500, 50000],
    0-32 boxes), each converging at 1e-4 of its emitter key.  Batched: every
    running scene does one shooter step per iteration, all in one launch, in
    the kernel form the autotuner picks.  Plain: the single-scene solver on
    each scene in turn, over the same steps.  Device time from CUDA events on
    each solver's stream.  Each scene's batched trace and accB/deltaB are
    compared with its plain run bit for bit; no ratio is given if any differs.
    With several ranks, each takes a share of the scenes balanced by triangle
    count (no exchange of data) and the totals are summed over ranks."""
    import numpy as np
    from hwrad import scenes as S, shard
    gens_all = S.batch_rooms(n_scenes, seed=4000)
    share = shard.partition_scenes([len(g.vtx) for g in gens_all], world)[rank]
    gens = [gens_all[i] for i in share]
    # first use of the preparation kernels (module load) on a small room
    prepare_scenes(capi, [S.room(2)], device)
    t0 = time.perf_counter()
    preps = prepare_scenes(capi, gens, device)
    prep_s = time.perf_counter() - t0
    log(f"batch: {len(gens)} scenes prepared (device octree and links) in {prep_s:.2f} s")
    tris = [p[0].view()["n"] for p in preps]
    t0 = time.perf_counter()
    b = _batch(capi, preps, device)
    create_s = time.perf_counter() - t0
    form = b.autotune(4, 2)
    b.run(warmup)
    s0 = [b.scene_stats(i)[0] for i in range(len(preps))]
    K = max(s0)                      # iterations before the timed window
    it, active, ms = b.run_timed(iters)
    s1 = [b.scene_stats(i)[0] for i in range(len(preps))]
    shots = sum(s1) - sum(s0)
    dev_bytes = b.stats()["device_bytes"]
    log(f"batch: form {form}, {it} iterations, {shots} shots in {ms:.1f} ms")
    # exact walk counts over the same iterations (counting pass on a fresh batch)
    bc = _batch(capi, preps, device, form)
    bc.run(K)
    bc.set_counting(True)
    c0 = bc.stats()
    bc.run(iters)
    c1 = bc.stats()
    bc.close()
    cnt = {k: c1[k] - c0[k] for k in ("rays", "cells", "tri_tests", "se_tests")}
    slot_steps = sum(n * (s1[i] - s0[i]) for i, n in enumerate(tris))
    alg = slot_steps * BYTES_PER_SLOT + cnt["cells"] * BYTES_PER_CELL + cnt["tri_tests"] * BYTES_PER_TRI_TEST + \
        cnt["se_tests"] * BYTES_PER_SE_TEST
    # the same window per scene-size band, each band batched on its own
    bands = {}
    for lo, hi, name in SIZE_BANDS:
        idx = [i for i, n in enumerate(tris) if lo <= n < hi]
        if not idx:
            continue
        bb = _batch(capi, [preps[i] for i in idx], device, form)
        bb.run(K)
        s0b = sum(bb.scene_stats(j)[0] for j in range(len(idx)))
        _, _, msb = bb.run_timed(iters)
        s1b = sum(bb.scene_stats(j)[0] for j in range(len(idx)))
        bb.close()
        bands[name] = {"scenes": len(idx), "triangles": int(sum(tris[i] for i in idx)), "shots": s1b - s0b,
                       "batched_ms": msb, "idx": idx}
    # plain: the single-scene solver scene by scene over the same steps, and parity
    plain_ms = 0.0
    plain_shots = 0
    per_plain = []
    bad = []
    for k, (sc, tr, o) in enumerate(preps):
        d = capi.Device(sc, tr, o, device)
        if s0[k]:
            d.run(s0[k])
        n, conv, m = d.run_timed(iters)
        plain_ms += m
        plain_shots += n
        per_plain.append((n, m))
        same = n == s1[k] - s0[k] and np.array_equal(d.trace(), b.trace(k))
        d.download(sc)
        v = sc.view()
        acc, db = v["accB"].copy(), v["deltaB"].copy()
        d.close()
        b.download(k, sc)
        v = sc.view()
        same = same and np.array_equal(acc.view(np.uint32), v["accB"].view(np.uint32)) and \
            np.array_equal(db.view(np.uint32), v["deltaB"].view(np.uint32))
        if not same:
            bad.append(share[k])
    b.close()
    log(f"plain: {plain_shots} shots in {plain_ms:.1f} ms; scenes differing: {bad}")
    for name, v in bands.items():
        ps = sum(per_plain[i][0] for i in v["idx"])
        pm = sum(per_plain[i][1] for i in v["idx"])
        bs = v["shots"] / (v["batched_ms"] / 1000.0) if v["batched_ms"] > 0 else None
        pl = ps / (pm / 1000.0) if pm > 0 else None
        v.update({"batched_shots_per_s": bs, "plain_shots_per_s": pl,
                  "batched_over_plain": bs / pl if bs and pl and not bad else None})
        del v["idx"]
    # end to end through the C ABI: fresh scenes from the generator's arrays,
    # device preparation, upload, the same iterations, download of every scene
    t0 = time.perf_counter()
    ep = prepare_scenes(capi, gens, device)
    be = _batch(capi, ep, device, form)
    be.run(K + iters)
    e_shots = sum(be.scene_stats(i)[0] for i in range(len(ep)))
    for i, (sc, _, _) in enumerate(ep):
        be.download(i, sc)
    e2e_s = time.perf_counter() - t0
    est = be.stats()
    be.close()
    # totals over ranks (scenes are sharded; each rank reports its share)
    red_sum = ranks.sum if ranks else (lambda x: x)
    red_max = ranks.max if ranks else (lambda x: x)
    shots_t, plain_shots_t = red_sum(shots), red_sum(plain_shots)
    ms_t, plain_ms_t, e2e_t = red_max(ms), red_sum(plain_ms), red_max(e2e_s)
    n_bad = int(red_sum(len(bad)))
    batched = shots_t / (ms_t / 1000.0) if ms_t > 0 else None
    plain = plain_shots_t / (plain_ms_t / 1000.0) if plain_ms_t > 0 else None
    achieved = alg / (ms / 1000.0) / 1e9 if ms > 0 else None
    peak, peak_kind = _peaks()
    all_tris = [len(g.vtx) for g in gens_all]
    return {"workload": f"{n_scenes} rooms (config 4), {sum(all_tris):,} input triangles, "
                        f"{min(all_tris)}-{max(all_tris)} per scene",
            "ranks": world, "scenes_this_rank": len(gens), "slots_this_rank": int(sum(tris)),
            "form": form, "iterations": it, "shots": shots_t, "active_scenes_end": active,
            "parity": "bit-identical" if n_bad == 0 else f"DIFFERS in {n_bad} scenes (first: {bad[:8]})",
            "batched_shots_per_s": batched, "plain_shots_per_s": plain,
            "batched_over_plain": batched / plain if batched and plain and n_bad == 0 else None,
            "rays_per_s": cnt["rays"] / (ms / 1000.0) if ms > 0 else None,
            "batched_ms_per_iter": ms / max(it, 1), "plain_shots": plain_shots_t,
            "bands": bands,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak if achieved else None, "kernel": "k_batch_shoot",
                         "peak_kind": f"{peak_kind} hbm_gbs", "alg_bytes_per_iter": alg / max(it, 1),
                         "counts_per_iter": {k: v / max(it, 1) for k, v in cnt.items()}},
            "e2e": {"value": e_shots * world / e2e_t if e2e_t > 0 else None, "unit": "shots/s",
                    "seconds": e2e_t, "h2d_bytes": est["h2d_bytes"],
                    "note": "generator arrays -> device octree + links, host pre-partition, rad_batch_create "
                            "(upload), warm-up and timed iterations, download of every scene"},
            "device_bytes": dev_bytes, "prep_s": round(prep_s, 3), "create_s": round(create_s, 3),
            "l2": "batch inputs exceed L2; plain timed without flush (graph chunks)"}


def measure_adaptive(capi, steps, device, with_reference=True):
    """The adaptive split variant (ADAPT + ROLLBACK build of the reference) on
    a 100x100x100 room with 4 boxes that splits from 960 triangles toward the
    40,000 cap: wall-clock steps/s of the GPU + host solver, next to the
    reference's own adaptive build (serial by construction) on the same steps.
    Both speculation modes run; their results must be bit-identical."""
    import numpy as np
    from hwrad import scenes as S
    sc_gen = S.room_with_boxes(8, 4, 1, seed=5, size=100.0)
    argv = sc_gen.argv({"-triangle": "40000", "-converge": "5"})
    tmp = tempfile.mkdtemp(prefix="radadapt_")
    tri = sc_gen.write(os.path.join(tmp, "adapt.tri"))
    o = capi.options_from_argv(argv)

    def one(wait):
        sc = capi.Scene.load(tri, o)
        tree = capi.Octree(sc, _nproc())
        sc.init()
        ad = capi.Adaptive(sc, tree, o, device)
        ad.set_speculation(wait)
        t0 = time.perf_counter()
        n, conv, _ = ad.run(steps)
        dt = time.perf_counter() - t0
        st = ad.stats()
        trace = ad.trace()
        ad.close()
        v = sc.view()
        res = {"steps": n, "steps_per_s": n / dt if dt > 0 else None, "host_form_factors": st["host_points"],
               "device_sample_points": st["device_points"], "speculations": st["speculations"]}
        return res, st, (trace, v["accB"].copy(), v["deltaB"].copy(), v["parent"].copy())

    race, st, r_state = one(False)
    wait, _, w_state = one(True)
    same = all(np.array_equal(a, b) for a, b in zip(r_state, w_state))
    out = {"workload": "room 100^3, 4 boxes, 960 triangles splitting toward the 40,000 cap, -converge 5",
           "steps": race["steps"], "slots_end": st["n_slots"], "steps_per_s": race["steps_per_s"],
           "rays": st["rays"], "splits": st["splits"], "host_form_factors": race["host_form_factors"],
           "sample_points": st["samples"], "device_sample_points": race["device_sample_points"],
           "speculations": race["speculations"], "split_candidates": st["split_candidates"],
           "speculation": "raced by the host (default)",
           "waiting_speculation": {k: wait[k] for k in ("steps_per_s", "host_form_factors",
                                                        "device_sample_points", "speculations")},
           "modes_bit_identical": bool(same)}
    if with_reference:
        sys.path.insert(0, os.path.join(REPO, "oracle"))
        import runner
        if os.path.exists(runner.REF32A):
            times = os.path.join(tmp, "times.txt")
            runner.run(runner.REF32A, tri, argv + ["-jobs", "1"], steps=steps, env={"RAD_TIMES": times},
                       workdir=tmp, timeout=1800)
            stamps = [float(x) for x in open(times).read().split()]
            if len(stamps) > steps:
                ref = steps / (stamps[steps] - stamps[0])
                out["reference_steps_per_s"] = ref
                out["over_reference"] = out["steps_per_s"] / ref if out["steps_per_s"] else None
    return out


def measure_hall(capi, device, steps, warmup, flush_l2):
    """The config-3 hall (40x20x100, 406,684 wall/floor triangles + 300
    pillars, pre-partitioned to 422,429 slots): shots/s of the single-scene
    solver in the form it chooses for this scene (form 2: 4 CTAs per SM) and
    in the other form, L2 flushed before each timed step as in the headline,
    plus the chosen form's steady state.  The octree and the neighbour links
    are built on the device."""
    from hwrad import scenes as S
    gen = S.hall()
    tmp = tempfile.mkdtemp(prefix="radhall_")
    tri = gen.write(os.path.join(tmp, "hall.tri"))
    o = capi.options_from_argv(gen.argv())
    # first use of the preparation kernels (module load) on a small room
    wtri = S.room(2).write(os.path.join(tmp, "warm.tri"))
    ws = capi.Scene.load(wtri, o)
    capi.Octree(ws, device=device).close()
    ws.init(device=device)
    ws.close()
    t0 = time.time()
    sc = capi.Scene.load(tri, o)
    t1 = time.perf_counter()
    tree = capi.Octree(sc, device=device)
    t2 = time.perf_counter()
    sc.init(device=device)
    t3 = time.perf_counter()
    sc.prepartition()
    out = {"workload": "hall 40x20x100, 406,684 triangles + 300 pillars (config 3), FP32",
           "slots": int(sc.view()["n"]), "host_prep_s": round(time.time() - t0, 2), "steps": steps,
           "l2": "flushed (512 MB write, enqueued on the solver's stream) before every timed step"}
    # the same preparation in its host forms, for comparison (octree on all
    # host cores; InitRadiosity's neighbour links by the host hash)
    sh = capi.Scene.load(tri, o)
    t4 = time.perf_counter()
    th = capi.Octree(sh, _nproc())
    t5 = time.perf_counter()
    sh.init()
    t6 = time.perf_counter()
    out["preparation_ms"] = {"octree_device": round(1e3 * (t2 - t1), 1), "octree_host": round(1e3 * (t5 - t4), 1),
                             "host_cores": _nproc(), "init_device": round(1e3 * (t3 - t2), 1),
                             "init_host": round(1e3 * (t6 - t5), 1)}
    th.close()
    sh.close()
    for which in ("chosen", "other"):
        dv = capi.Device(sc, tree, o, device)
        if which == "chosen":
            out["form"] = dv.layout
        else:
            dv.set_layout(3 - out["form"])
            out["other_form"] = dv.layout
        dv.run(warmup)
        tot, n_done = 0.0, 0
        for _ in range(steps):
            flush_l2(dv)
            n, conv, ms = dv.run_timed(1)
            tot += ms
            n_done += n
            if conv:
                break
        out[f"{which}_flushed_shots_per_s"] = 1000.0 * n_done / tot if tot > 0 else None
        if which == "chosen":
            n, _, ms = dv.run_timed(steps * 4)
            out["chosen_steady_shots_per_s"] = 1000.0 * n / ms if ms > 0 else None
        dv.close()
    return out


def measure_render(capi, scene, device, reps, with_oracle=True):
    """Headless render of the config-2 result as the viewer shows it (1024x768,
    flat and Gouraud): end-to-end images/s of rad_render_scene and of
    rad_render_fin (converter restatement on the host, upload, CUDA raster,
    download), next to the C++ restatement (oracle/raster_oracle, one core)
    on the same .fin."""
    tmp = tempfile.mkdtemp(prefix="radrender_")
    prefix = os.path.join(tmp, "result")
    scene.write_fin(prefix)
    fin = prefix + ".fin"
    out = {"workload": "config-2 result, 1024x768, the viewer's initial view", "reps": reps}
    for shading in ("flat", "gouraud"):
        capi.render_scene(scene, device, shading=shading)     # warm-up
        t0 = time.perf_counter()
        for _ in range(reps):
            capi.render_scene(scene, device, shading=shading)
        out[f"{shading}_scene_images_per_s"] = reps / (time.perf_counter() - t0)
        t0 = time.perf_counter()
        for _ in range(reps):
            capi.render_fin(fin, device, shading=shading)
        out[f"{shading}_fin_images_per_s"] = reps / (time.perf_counter() - t0)
        if with_oracle:
            sys.path.insert(0, os.path.join(REPO, "oracle"))
            import runner
            exe = os.path.join(runner.HERE, "_build", "raster_oracle")
            if os.path.exists(exe):
                t0 = time.perf_counter()
                subprocess.run([exe, fin, os.path.join(tmp, "o.rgba"), "1024", "768",
                                "0" if shading == "flat" else "1", "0", "0"], check=True)
                out[f"{shading}_restatement_cpu_images_per_s"] = 1.0 / (time.perf_counter() - t0)
    return out


def rank_env():
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


class Ranks:
    """Replicas only: one solver per GPU, no data exchange.  The only
    collectives are the contract's barrier around the timed region and the
    maximum of the ranks' times (the whole job ends with the slowest rank)."""

    def __init__(self, world, backend):
        import torch
        self.torch = torch
        self.dist = None
        self.cuda = backend == "nccl"
        if world > 1:
            import torch.distributed as dist
            dist.init_process_group(backend)
            self.dist = dist

    def sync(self):
        if self.cuda:
            self.torch.cuda.synchronize()

    def barrier(self):
        self.sync()
        if self.dist:
            self.dist.barrier()
        self.sync()

    def _reduce(self, x, op):
        if not self.dist:
            return x
        t = self.torch.tensor([x], dtype=self.torch.float64, device="cuda" if self.cuda else "cpu")
        self.dist.all_reduce(t, op=op)
        return float(t.item())

    def max(self, x):
        return self._reduce(x, self.dist.ReduceOp.MAX if self.dist else None)

    def sum(self, x):
        return self._reduce(x, self.dist.ReduceOp.SUM if self.dist else None)

    def close(self):
        if self.dist:
            self.dist.destroy_process_group()


def replica_value(world, steps_per_rank, worst_ms):
    """Whole-job shots/s: every rank shoots its own replica."""
    return world * steps_per_rank / (worst_ms / 1000.0) if worst_ms > 0 else None


def bench_config(slots, world):
    """The workload keys both arms report (the reference arm and ours)."""
    return {"workload": WORKLOAD, "slots": int(slots), "l2": L2_NOTE, "parallelism": f"replicas x{world}"}


def run_reference_arm(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    with tempfile.TemporaryDirectory() as tmp:
        sc, tri = _scene_file(tmp)
        try:
            res = cpu_reference(tri, sc.argv(), args.warmup, args.steps)
        except Exception as exc:
            print(json.dumps({"impl": "reference", "unavailable": f"{exc}".splitlines()[0]}))
            return 0
    line = {"metric": "shots/s", "value": res["value"], "unit": "shots/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000.0 / res["value"] if res["value"] else None,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded generator, hwrad.scenes.config2)", "impl": "reference",
            "config": bench_config(res["slots"], args.gpus),
            "cpu_baseline": {"value": res["value"], "unit": "shots/s", "cores": res["cores"], "kind": res["kind"],
                             "build": res["build"], "sample": res["sample"]},
            "e2e": {"value": res["value"], "unit": "shots/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=500)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--batch-scenes", type=int, default=256, help="0 skips the batched measurement")
    ap.add_argument("--batch-iters", type=int, default=100)
    ap.add_argument("--adaptive-steps", type=int, default=100, help="0 skips the adaptive-variant measurement")
    ap.add_argument("--render-reps", type=int, default=5, help="0 skips the headless-render measurement")
    ap.add_argument("--hall-steps", type=int, default=30, help="0 skips the config-3 hall measurement")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference_arm(args)

    import numpy as np
    import torch
    from hwrad import capi

    world, rank, local = rank_env()
    torch.cuda.set_device(local)
    ranks = Ranks(world, "nccl")
    barrier, max_over_ranks = ranks.barrier, ranks.max
    dist = ranks.dist

    log("config-2 scene: host preparation")
    tmp = tempfile.mkdtemp(prefix="radbench_")
    sc_gen, tri = _scene_file(tmp)
    argv = sc_gen.argv()
    opts = capi.options_from_argv(argv, jobs=_nproc())
    t0 = time.time()
    scene = capi.Scene.load(tri, opts)
    tree = capi.Octree(scene, _nproc())
    scene.init()
    scene.prepartition()
    host_prep_s = time.time() - t0
    n_slots = scene.view()["n"]

    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def flush_l2(dev=None):
        """Write 512 MB (4x L2) before a timed step.  With a solver handle the
        write is enqueued on the handle's own stream, so the step's launch is
        already queued when it ends and the step's events see device time
        only; the host's launch latency stays outside, as in a run of steps
        back to back."""
        if dev is None:
            flush.add_(1.0)
            torch.cuda.synchronize()
            return
        with torch.cuda.stream(torch.cuda.ExternalStream(dev.stream())):
            flush.add_(1.0)

    clocks = ClockSampler(local)
    clocks.start()
    # ---- timed region: W warm-up steps, K timed steps, L2 flushed before each
    dev = capi.Device(scene, tree, opts, local)
    dev.run(args.warmup)
    unshot_start = dev.stats()["unshot_power"]
    barrier()
    total_ms = 0.0
    done = 0
    for _ in range(args.steps):
        flush_l2(dev)
        n, conv, ms = dev.run_timed(1)
        total_ms += ms
        done += n
        if conv:
            break
    barrier()
    worst_ms = max_over_ranks(total_ms)
    # steady state without the flush (graph chunks of 32 steps)
    unshot_end = dev.stats()["unshot_power"]
    n_ss, _, ms_ss = dev.run_timed(args.steps)
    st_main = dev.stats()
    dev.close()

    log(f"timed {done} steps: {total_ms:.2f} ms; steady state {n_ss} steps {ms_ss:.2f} ms")
    # ---- per-kernel durations over the same steps (fresh instance, one launch at a time)
    dprof = capi.Device(scene, tree, opts, local)
    dprof.run(args.warmup)
    setup_ms = shoot_ms = 0.0
    for _ in range(done):
        flush_l2(dprof)
        _, _, a, b = dprof.run_profiled(1)
        setup_ms += a
        shoot_ms += b
    dprof.close()

    log(f"profiled pass: setup {setup_ms:.2f} ms, shoot {shoot_ms:.2f} ms")
    # ---- exact walk counts over the same steps (deterministic solver)
    dcnt = capi.Device(scene, tree, opts, local)
    dcnt.set_counting(True)
    dcnt.run(args.warmup)
    c0 = dcnt.stats()
    dcnt.run(done)
    c1 = dcnt.stats()
    dcnt.close()

    log("counting pass done")
    # ---- e2e: C ABI with host buffers (upload, K steps, download)
    barrier()
    te0 = time.perf_counter()
    dev2 = capi.Device(scene, tree, opts, local)
    n_e2e, _, _ = dev2.run(args.warmup + done)
    dev2.download(scene)
    torch.cuda.synchronize()
    te1 = time.perf_counter()
    e2e_s = max_over_ranks(te1 - te0)
    h2d_bytes = dev2.stats()["h2d_bytes"]
    dev2.close()
    clocks.stop()

    d = {k: c1[k] - c0[k] for k in ("rays", "rays_ref", "cells", "tri_tests", "se_tests", "prec_steps")}
    alg_bytes = n_slots * BYTES_PER_SLOT * done + d["cells"] * BYTES_PER_CELL + \
        d["tri_tests"] * BYTES_PER_TRI_TEST + d["se_tests"] * BYTES_PER_SE_TEST
    per_launch = alg_bytes / max(done, 1)
    avg_shoot_s = shoot_ms / 1000.0 / max(done, 1)
    peak, peak_kind = _peaks()
    achieved = per_launch / avg_shoot_s / 1e9 if avg_shoot_s > 0 else None
    traffic, traffic_src = committed_traffic()

    value = replica_value(world, done, worst_ms)
    # bytes rad_dev_create copied to the device (counted by the library), and
    # the download of accB + deltaB (4 records of 16 B per slot), per step
    h2d = h2d_bytes / max(args.warmup + done, 1)
    d2h = n_slots * 16 * 4 / max(args.warmup + done, 1)

    log(f"e2e {e2e_s:.3f} s")
    batched = None
    if args.batch_scenes > 0:
        batched = measure_batched(capi, args.batch_scenes, args.warmup, args.batch_iters, local, world, rank, ranks)

    adaptive = None
    if args.adaptive_steps > 0:
        log("adaptive variant")
        adaptive = measure_adaptive(capi, args.adaptive_steps, local, with_reference=not args.no_cpu_baseline)

    hall = None
    if args.hall_steps > 0 and rank == 0:
        log("config-3 hall")
        hall = measure_hall(capi, local, args.hall_steps, args.warmup, flush_l2)

    render = None
    if args.render_reps > 0 and rank == 0:
        log("headless render")
        render = measure_render(capi, scene, local, args.render_reps, with_oracle=not args.no_cpu_baseline)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        log("cpu baseline")
        try:
            cpu = cpu_reference(tri, argv, 2, 60)
        except Exception as exc:
            cpu = {"value": None, "unit": "shots/s", "cores": _nproc(), "kind": "reference",
                   "sample": f"failed: {exc}"}
        cpu = {k: cpu.get(k) for k in ("value", "unit", "cores", "kind", "build", "sample")}
        if cpu["value"] is not None and cpu["cores"] > 1:
            try:
                one = cpu_reference(tri, argv, 2, 12, jobs=1)
                cpu["one_thread"] = {k: one[k] for k in ("value", "cores", "sample")}
            except Exception as exc:
                cpu["one_thread"] = {"value": None, "sample": f"failed: {exc}"}

    line = {
        "metric": "shots/s", "value": value, "unit": "shots/s", "n_gpus": world, "steps": done,
        "warmup": args.warmup, "ms_per_step": worst_ms / max(done, 1), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded generator, hwrad.scenes.config2)",
        "config": bench_config(n_slots, world),
        "host_prep_s": round(host_prep_s, 3),
        "rays_per_s": d["rays"] / (worst_ms / 1000.0) if worst_ms > 0 else None,
        "rays_per_step": d["rays"] / max(done, 1),
        "unshot_power": {"after_warmup": unshot_start, "after_timed_steps": unshot_end,
                         "note": "FP64 total of (dB_r+dB_g+dB_b)*area over live slots (convergence monitor)"},
        "steady_state": {"value": n_ss / (ms_ss / 1000.0) if ms_ss > 0 else None, "unit": "shots/s",
                         "note": "graph chunks of 32 steps, no L2 flush", "steps": n_ss},
        "kernels_ms_per_step": {"k_setup": setup_ms / max(done, 1), "k_shoot": shoot_ms / max(done, 1)},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak if achieved else None, "traffic": traffic,
                     "traffic_capture": traffic_src,
                     "kernel": "k_shoot", "peak_kind": f"{peak_kind} hbm_gbs (burst)",
                     "alg_bytes_per_launch": per_launch,
                     "counts_per_launch": {k: v / max(done, 1) for k, v in d.items()}},
        "e2e": {"value": world * n_e2e / e2e_s, "unit": "shots/s", "steps": n_e2e,
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "note": "rad_dev_create (upload) + run + rad_dev_download over the warm-up + timed steps from "
                        "the same initial state, the steps back to back in graph chunks: no L2 flush between "
                        "them, unlike `value`, which flushes L2 before every step (so e2e can exceed it)"},
        "batched": batched,
        "adaptive": adaptive,
        "render": render,
        "hall": hall,
        "gpu_launches": done if opts.parallel_src <= 1 else 2 * done,
        "clocks": clocks.summary(),
        "cpu_baseline": cpu,
    }
    if rank == 0:
        print(json.dumps(line))
    ranks.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
