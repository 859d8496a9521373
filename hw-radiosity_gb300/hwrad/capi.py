"""ctypes binding of the C ABI in ``include/rad_gb300.h``.

The Python side is a thin mirror of the reference's flow (``src/rad.cpp``
``main`` -> ``InitModelFromFile`` -> ``DoRadiosity``): load a ``.tri`` scene,
build the visibility structure, initialise, pre-partition, run the shooting
loop on the device, read the results back.  The library must have been built
(``hwrad.build.build()``); there is no fallback path.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Dict, Optional, Sequence

import numpy as np

from . import build as _build

RAD_OK = 0
RAD_ERR_ARG, RAD_ERR_IO, RAD_ERR_PARSE, RAD_ERR_CAPACITY, RAD_ERR_CUDA, RAD_ERR_WALK, RAD_ERR_NODEV = range(1, 8)

EXPORTS = [
    "rad_options_default", "rad_last_error", "rad_version",
    "rad_scene_load", "rad_scene_from_arrays", "rad_scene_init", "rad_scene_init_device", "rad_scene_prepartition",
    "rad_scene_view_get", "rad_scene_write_fin", "rad_scene_log", "rad_scene_free",
    "rad_octree_build", "rad_octree_build_device", "rad_octree_tables", "rad_octree_info", "rad_octree_cell_coords", "rad_octree_free",
    "rad_dev_create", "rad_dev_run", "rad_dev_stream", "rad_dev_run_timed", "rad_dev_run_profiled", "rad_dev_download", "rad_dev_trace", "rad_dev_stats",
    "rad_dev_set_counting", "rad_dev_set_schedule", "rad_dev_set_layout", "rad_dev_layout", "rad_dev_autotune", "rad_dev_ray_hit", "rad_dev_form_factors", "rad_dev_form_factors_noalloc",
    "rad_dev_destroy",
    "rad_batch_create", "rad_batch_run", "rad_batch_run_timed", "rad_batch_scene_stats", "rad_batch_download",
    "rad_batch_trace", "rad_batch_stats", "rad_batch_set_counting", "rad_batch_destroy",
    "rad_adapt_create", "rad_adapt_run", "rad_adapt_trace", "rad_adapt_stats", "rad_adapt_set_speculation", "rad_adapt_destroy",
    "rad_render_options_default", "rad_render_fin", "rad_render_scene",
]


class Options(C.Structure):
    _fields_ = [("debug", C.c_int32), ("adapt_area", C.c_float), ("sample_area", C.c_float),
                ("converge", C.c_float), ("delta_ff", C.c_float), ("write_cycle", C.c_int32),
                ("zip", C.c_int32), ("triangle_limit", C.c_int32), ("light_scale", C.c_float),
                ("interactive", C.c_int32), ("jobs", C.c_int32), ("parallel_src", C.c_int32),
                ("precision", C.c_int32), ("walk_cap", C.c_int32)]


class SceneView(C.Structure):
    _fields_ = [("n", C.c_int32), ("n_orig", C.c_int32), ("elem_size", C.c_int32),
                ("p", C.c_void_p), ("accB", C.c_void_p), ("deltaB", C.c_void_p), ("area", C.c_void_p),
                ("nrm", C.c_void_p), ("ctr", C.c_void_p), ("parent", C.c_void_p), ("frgb", C.c_void_p),
                ("brgb", C.c_void_p), ("nb", C.c_void_p), ("G0", C.c_float * 3), ("G1", C.c_float * 3),
                ("sample_area", C.c_float), ("min_area", C.c_float), ("max_area", C.c_float)]


class Stats(C.Structure):
    _fields_ = [("steps", C.c_int64), ("shots", C.c_int64), ("rays", C.c_int64), ("rays_ref", C.c_int64),
                ("cells", C.c_int64), ("tri_tests", C.c_int64), ("se_tests", C.c_int64),
                ("prec_steps", C.c_int64), ("walk_cap_hits", C.c_int64), ("converged", C.c_int32),
                ("n_slots", C.c_int32), ("device_bytes", C.c_int64), ("walk_loops", C.c_int64),
                ("unshot_power", C.c_double), ("h2d_bytes", C.c_int64)]


class RadError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code


_lib: Optional[C.CDLL] = None


def lib_path() -> str:
    return _build.LIB


def load(path: Optional[str] = None) -> C.CDLL:
    """Load the native library (it must exist: there is no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    p = path or _build.LIB
    if not os.path.exists(p):
        raise RuntimeError(f"native library {p} missing; run hwrad.build.build() first")
    L = C.CDLL(p)
    vp, i32, i64, f = C.c_void_p, C.c_int32, C.c_int64, C.c_float
    P = C.POINTER
    sig = {
        "rad_options_default": (None, [P(Options)]),
        "rad_last_error": (C.c_char_p, []),
        "rad_version": (C.c_char_p, []),
        "rad_scene_load": (C.c_int, [C.c_char_p, P(Options), P(vp)]),
        "rad_scene_from_arrays": (C.c_int, [vp, vp, vp, i32, P(Options), P(vp)]),
        "rad_scene_init": (C.c_int, [vp]),
        "rad_scene_init_device": (C.c_int, [vp, i32]),
        "rad_scene_prepartition": (C.c_int, [vp]),
        "rad_scene_view_get": (C.c_int, [vp, P(SceneView)]),
        "rad_scene_write_fin": (C.c_int, [vp, C.c_char_p, i32]),
        "rad_scene_log": (C.c_char_p, [vp, i32]),
        "rad_scene_free": (None, [vp]),
        "rad_octree_build": (C.c_int, [vp, i32, P(vp)]),
        "rad_octree_build_device": (C.c_int, [vp, i32, P(vp)]),
        "rad_octree_tables": (C.c_int, [vp, vp, vp, vp, vp]),
        "rad_octree_info": (C.c_int, [vp, P(i64), P(i64), P(i32), P(i64), P(i32)]),
        "rad_octree_cell_coords": (C.c_int, [vp, i32, vp, i32, vp, vp]),
        "rad_octree_free": (None, [vp]),
        "rad_dev_create": (C.c_int, [vp, vp, P(Options), i32, P(vp)]),
        "rad_dev_run": (C.c_int, [vp, i64, P(i64), P(i32)]),
        "rad_dev_stream": (C.c_int, [vp, P(vp)]),
        "rad_dev_run_timed": (C.c_int, [vp, i64, P(i64), P(i32), P(C.c_double)]),
        "rad_dev_run_profiled": (C.c_int, [vp, i64, P(i64), P(i32), P(C.c_double), P(C.c_double)]),
        "rad_dev_download": (C.c_int, [vp, vp]),
        "rad_dev_trace": (C.c_int, [vp, vp, i64, P(i64)]),
        "rad_dev_stats": (C.c_int, [vp, P(Stats)]),
        "rad_dev_set_counting": (C.c_int, [vp, i32]),
        "rad_dev_set_layout": (C.c_int, [vp, i32]),
        "rad_dev_layout": (C.c_int, [vp]),
        "rad_dev_autotune": (C.c_int, [vp, i32, i64, C.POINTER(i64), C.POINTER(i32), C.POINTER(i32)]),
        "rad_dev_ray_hit": (C.c_int, [vp, vp, vp, vp, i32, vp]),
        "rad_dev_form_factors": (C.c_int, [vp, i32, vp, i32, vp]),
        "rad_dev_form_factors_noalloc": (C.c_int, [vp, vp, i32, vp, i32, vp, vp]),
        "rad_dev_set_schedule": (C.c_int, [vp, C.c_double, C.c_double, C.c_double, C.c_double]),
        "rad_dev_destroy": (None, [vp]),
        "rad_batch_create": (C.c_int, [vp, vp, vp, i32, i32, i32, P(vp)]),
        "rad_batch_run": (C.c_int, [vp, i64, P(i64), P(i32)]),
        "rad_batch_run_timed": (C.c_int, [vp, i64, P(i64), P(i32), P(C.c_double)]),
        "rad_batch_scene_stats": (C.c_int, [vp, i32, P(i64), P(i32)]),
        "rad_batch_download": (C.c_int, [vp, i32, vp]),
        "rad_batch_trace": (C.c_int, [vp, i32, vp, i64, P(i64)]),
        "rad_batch_stats": (C.c_int, [vp, P(Stats)]),
        "rad_batch_set_counting": (C.c_int, [vp, i32]),
        "rad_batch_set_form": (C.c_int, [vp, i32]),
        "rad_batch_form": (C.c_int, [vp]),
        "rad_batch_autotune": (C.c_int, [vp, i32, i32, P(i32)]),
        "rad_batch_destroy": (None, [vp]),
        "rad_adapt_create": (C.c_int, [vp, vp, P(Options), i32, P(vp)]),
        "rad_adapt_device_stats": (C.c_int, [vp, P(i64), P(i64), P(i64)]),
        "rad_adapt_run": (C.c_int, [vp, i64, P(i64), P(i32)]),
        "rad_adapt_trace": (C.c_int, [vp, vp, i64, P(i64)]),
        "rad_adapt_stats": (C.c_int, [vp, P(Stats), P(i64), P(i64), P(i64)]),
        "rad_adapt_set_speculation": (C.c_int, [vp, i32]),
        "rad_adapt_destroy": (None, [vp]),
        "rad_render_options_default": (None, [P(RenderOptions)]),
        "rad_render_fin": (C.c_int, [C.c_char_p, P(RenderOptions), i32, vp]),
        "rad_render_scene": (C.c_int, [vp, P(RenderOptions), i32, vp]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def _check(rc: int, allow=()):
    if rc != RAD_OK and rc not in allow:
        raise RadError(rc, load().rad_last_error().decode(errors="replace"))
    return rc


def options(**kw) -> Options:
    o = Options()
    load().rad_options_default(C.byref(o))
    for k, v in kw.items():
        setattr(o, k, v)
    return o


def options_from_argv(args: Sequence[str], **kw) -> Options:
    """Reference CLI options (e.g. ["-converge", "4.5", "-light", "0.0588"])."""
    m = {"-debug": ("debug", int), "-adapt_area": ("adapt_area", float), "-sample_area": ("sample_area", float),
         "-converge": ("converge", float), "-delta_ff": ("delta_ff", float), "-write_cycle": ("write_cycle", int),
         "-triangle": ("triangle_limit", int), "-light": ("light_scale", float), "-jobs": ("jobs", int),
         "-parallel_src": ("parallel_src", int)}
    o = options(**kw)
    a = list(args)
    i = 0
    while i < len(a):
        if a[i] in m:
            name, ty = m[a[i]]
            setattr(o, name, ty(a[i + 1]))
            i += 2
        elif a[i] == "-zip":
            o.zip = 1
            i += 1
        elif a[i] == "-interactive":
            o.interactive = 1
            i += 1
        else:
            i += 1
    return o


class Scene:
    """Host scene store (``rad_scene``)."""

    def __init__(self, handle, opts: Options):
        self.h = C.c_void_p(handle)
        self.opts = opts

    @classmethod
    def load(cls, path: str, opts: Options) -> "Scene":
        h = C.c_void_p()
        _check(load().rad_scene_load(path.encode(), C.byref(opts), C.byref(h)))
        return cls(h.value, opts)

    @classmethod
    def from_arrays(cls, vtx: np.ndarray, frgb: np.ndarray, brgb: np.ndarray, opts: Options) -> "Scene":
        vtx = np.ascontiguousarray(vtx, np.float32).reshape(-1, 9)
        frgb = np.ascontiguousarray(frgb, np.int32).reshape(-1, 3)
        brgb = np.ascontiguousarray(brgb, np.int32).reshape(-1, 3)
        h = C.c_void_p()
        _check(load().rad_scene_from_arrays(vtx.ctypes.data, frgb.ctypes.data, brgb.ctypes.data, len(vtx),
                                            C.byref(opts), C.byref(h)))
        return cls(h.value, opts)

    def init(self, device: Optional[int] = None):
        """InitRadiosity; device=k finds the neighbour links on that GPU
        (rad_scene_init_device), with the same result."""
        if device is None:
            _check(load().rad_scene_init(self.h))
        else:
            _check(load().rad_scene_init_device(self.h, int(device)))

    def prepartition(self):
        _check(load().rad_scene_prepartition(self.h))

    def log(self, stream: int = 2) -> str:
        return load().rad_scene_log(self.h, stream).decode(errors="replace")

    def view(self) -> Dict[str, np.ndarray]:
        v = SceneView()
        _check(load().rad_scene_view_get(self.h, C.byref(v)))
        n = v.n
        ft = np.float32 if v.elem_size == 4 else np.float64

        def arr(ptr, dt, cols):
            if n == 0:
                return np.zeros((0, cols) if cols > 1 else (0,), dt)
            a = np.ctypeslib.as_array(C.cast(ptr, C.POINTER(np.ctypeslib.as_ctypes_type(dt))), (n * cols,)).copy()
            return a.reshape(n, cols) if cols > 1 else a

        return {"n": n, "n_orig": v.n_orig, "p": arr(v.p, ft, 9), "accB": arr(v.accB, ft, 9),
                "deltaB": arr(v.deltaB, ft, 3), "area": arr(v.area, ft, 1), "n_": arr(v.nrm, ft, 3),
                "c": arr(v.ctr, ft, 3), "parent": arr(v.parent, np.int32, 1), "Frgb": arr(v.frgb, np.int32, 3),
                "Brgb": arr(v.brgb, np.int32, 3), "nb": arr(v.nb, np.int32, 3),
                "G0": np.array(v.G0[:], np.float32), "G1": np.array(v.G1[:], np.float32),
                "sample_area": v.sample_area}

    def write_fin(self, prefix: str, loop: int = 0):
        _check(load().rad_scene_write_fin(self.h, prefix.encode(), loop))

    def close(self):
        if self.h:
            load().rad_scene_free(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Octree:
    def __init__(self, scene: Scene, threads: int = 0, device: Optional[int] = None):
        """BuildTree on the host (threads), or with the overlap tests on a CUDA
        device (device=k, rad_octree_build_device)."""
        self.h = C.c_void_p()
        self.precision = scene.opts.precision
        if device is None:
            _check(load().rad_octree_build(scene.h, threads, C.byref(self.h)))
        else:
            _check(load().rad_octree_build_device(scene.h, int(device), C.byref(self.h)))

    def tables(self) -> Dict[str, np.ndarray]:
        """cell_leaf, leaf_box (n_leaves x 8), leaf_range (n_leaves x 2), entry_tri."""
        i = self.info()
        n_cell = int(np.prod(i["dims"]))
        ft = np.float64 if self.precision == 64 else np.float32
        out = {"cell_leaf": np.zeros(n_cell, np.int32), "leaf_box": np.zeros((i["leaves"], 8), ft),
               "leaf_range": np.zeros((i["leaves"], 2), np.int32), "entry_tri": np.zeros(i["entries"], np.int32)}
        _check(load().rad_octree_tables(self.h, out["cell_leaf"].ctypes.data, out["leaf_box"].ctypes.data,
                                        out["leaf_range"].ctypes.data, out["entry_tri"].ctypes.data))
        return out

    def info(self) -> Dict[str, object]:
        a, b, e = C.c_int64(), C.c_int64(), C.c_int64()
        nl = C.c_int32()
        dims = (C.c_int32 * 3)()
        _check(load().rad_octree_info(self.h, C.byref(a), C.byref(b), C.byref(nl), C.byref(e), dims))
        return {"ref_nodes": a.value, "ref_list": b.value, "leaves": nl.value, "entries": e.value,
                "dims": list(dims)}

    def cell_coords(self, axis: int, q: np.ndarray, dtype=np.float32):
        """(reference expression, device threshold method) cell coordinates of q."""
        q = np.ascontiguousarray(q, dtype)
        a = np.zeros(len(q), np.int32)
        b = np.zeros(len(q), np.int32)
        _check(load().rad_octree_cell_coords(self.h, axis, q.ctypes.data, len(q), a.ctypes.data, b.ctypes.data))
        return a, b

    def close(self):
        if self.h:
            load().rad_octree_free(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Device:
    """Device-resident solver (``rad_dev``)."""

    def __init__(self, scene: Scene, tree: Octree, opts: Options, device: int = 0):
        self.h = C.c_void_p()
        self.P = max(1, opts.parallel_src)
        _check(load().rad_dev_create(scene.h, tree.h, C.byref(opts), device, C.byref(self.h)))

    def run(self, max_steps: int = 1 << 62):
        sd = C.c_int64()
        cv = C.c_int32()
        rc = _check(load().rad_dev_run(self.h, max_steps, C.byref(sd), C.byref(cv)), allow=(RAD_ERR_WALK,))
        return sd.value, bool(cv.value), rc

    def stream(self) -> int:
        """The handle's CUDA stream (a cudaStream_t, as an integer)."""
        p = C.c_void_p()
        _check(load().rad_dev_stream(self.h, C.byref(p)))
        return p.value or 0

    def run_timed(self, max_steps: int):
        """(steps, converged, device milliseconds) for up to max_steps steps."""
        sd, cv, ms = C.c_int64(), C.c_int32(), C.c_double()
        _check(load().rad_dev_run_timed(self.h, max_steps, C.byref(sd), C.byref(cv), C.byref(ms)),
               allow=(RAD_ERR_WALK,))
        return sd.value, bool(cv.value), ms.value

    def run_profiled(self, max_steps: int):
        """(steps, converged, setup-kernel ms, shoot-kernel ms), one launch at a time."""
        sd, cv, a, b = C.c_int64(), C.c_int32(), C.c_double(), C.c_double()
        _check(load().rad_dev_run_profiled(self.h, max_steps, C.byref(sd), C.byref(cv), C.byref(a), C.byref(b)),
               allow=(RAD_ERR_WALK,))
        return sd.value, bool(cv.value), a.value, b.value

    def download(self, scene: Scene):
        _check(load().rad_dev_download(self.h, scene.h))

    def trace(self) -> np.ndarray:
        n = C.c_int64()
        _check(load().rad_dev_trace(self.h, None, 0, C.byref(n)))
        out = np.zeros(n.value, np.int32)
        if n.value:
            _check(load().rad_dev_trace(self.h, out.ctypes.data, n.value, C.byref(n)))
        return out.reshape(-1, self.P)

    def stats(self) -> Dict[str, int]:
        s = Stats()
        _check(load().rad_dev_stats(self.h, C.byref(s)))
        return {k: getattr(s, k) for k, _ in Stats._fields_}

    def set_counting(self, on: bool):
        _check(load().rad_dev_set_counting(self.h, 1 if on else 0))

    def set_schedule(self, split_frac=0.55, split_frac_split=0.27, split_mean_mult=3.0, early_mean_mult=1.5):
        """Limits of the single-shooter schedule (rad_dev_set_schedule); all 0
        splits every group after the first step."""
        _check(load().rad_dev_set_schedule(self.h, split_frac, split_frac_split, split_mean_mult, early_mean_mult))

    def set_layout(self, layout: int = 0):
        """k_shoot form (rad_dev_set_layout): 0 auto, 1 tail-bound, 2 throughput."""
        _check(load().rad_dev_set_layout(self.h, int(layout)))

    @property
    def layout(self) -> int:
        return int(load().rad_dev_layout(self.h))

    def autotune(self, steps_per_trial: int = 8, max_steps: int = 64):
        """Time both k_shoot forms on this scene's own steps and keep the
        faster (rad_dev_autotune); returns (steps shot, converged, form)."""
        n, cv, ch = C.c_int64(), C.c_int32(), C.c_int32()
        _check(load().rad_dev_autotune(self.h, int(steps_per_trial), int(max_steps), C.byref(n), C.byref(cv),
                                       C.byref(ch)), allow=(RAD_ERR_WALK,))
        return int(n.value), bool(cv.value), int(ch.value)

    def ray_hit(self, p: np.ndarray, v: np.ndarray, ban: np.ndarray, dtype=np.float32) -> np.ndarray:
        p = np.ascontiguousarray(p, dtype).reshape(-1, 3)
        v = np.ascontiguousarray(v, dtype).reshape(-1, 3)
        ban = np.ascontiguousarray(ban, np.int32).reshape(-1)
        out = np.zeros(len(p), np.int32)
        _check(load().rad_dev_ray_hit(self.h, p.ctypes.data, v.ctypes.data, ban.ctypes.data, len(p),
                                      out.ctypes.data))
        return out

    def form_factors(self, src: int, rcv: np.ndarray, dtype=np.float32) -> np.ndarray:
        rcv = np.ascontiguousarray(rcv, np.int32).reshape(-1)
        out = np.zeros((len(rcv), 3), dtype)
        _check(load().rad_dev_form_factors(self.h, int(src), rcv.ctypes.data, len(rcv), out.ctypes.data))
        return out

    def form_factors_noalloc(self, src, d_rcv: int, n_rcv: int, d_ff: int, stream: int = 0) -> int:
        """Enqueue the allocation-free form factors on device buffers (raw
        device pointers d_rcv, d_ff); returns the status code."""
        src = np.ascontiguousarray(src, np.int32).reshape(-1)
        return load().rad_dev_form_factors_noalloc(self.h, src.ctypes.data, len(src), C.c_void_p(d_rcv), n_rcv,
                                                   C.c_void_p(d_ff), C.c_void_p(stream))

    def close(self):
        if self.h:
            load().rad_dev_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """Batched form (``rad_batch``): independent scenes, one launch per iteration."""

    def __init__(self, scenes, trees, opts, device: int = 0, trace_cap: int = 0):
        n = len(scenes)
        self._keep = (list(scenes), list(trees), list(opts))
        self.P = max(1, int(opts[0].parallel_src)) if n else 1
        sp = (C.c_void_p * n)(*[s.h.value for s in scenes])
        tp = (C.c_void_p * n)(*[t.h.value for t in trees])
        op = (Options * n)(*opts)
        self._opts = op
        self.n = n
        self.h = C.c_void_p()
        _check(load().rad_batch_create(C.cast(sp, C.c_void_p), C.cast(tp, C.c_void_p), C.cast(op, C.c_void_p),
                                       n, trace_cap, device, C.byref(self.h)))

    def run(self, max_iters: int = 1 << 62):
        it, na = C.c_int64(), C.c_int32()
        rc = _check(load().rad_batch_run(self.h, max_iters, C.byref(it), C.byref(na)), allow=(RAD_ERR_WALK,))
        return it.value, na.value, rc

    def run_timed(self, max_iters: int):
        it, na, ms = C.c_int64(), C.c_int32(), C.c_double()
        _check(load().rad_batch_run_timed(self.h, max_iters, C.byref(it), C.byref(na), C.byref(ms)),
               allow=(RAD_ERR_WALK,))
        return it.value, na.value, ms.value

    def scene_stats(self, s: int):
        st, cv = C.c_int64(), C.c_int32()
        _check(load().rad_batch_scene_stats(self.h, s, C.byref(st), C.byref(cv)))
        return st.value, bool(cv.value)

    def download(self, s: int, scene: "Scene"):
        _check(load().rad_batch_download(self.h, s, scene.h))

    def trace(self, s: int) -> np.ndarray:
        n = C.c_int64()
        _check(load().rad_batch_trace(self.h, s, None, 0, C.byref(n)))
        out = np.zeros(n.value, np.int32)
        if n.value:
            _check(load().rad_batch_trace(self.h, s, out.ctypes.data, n.value, C.byref(n)))
        return out.reshape(-1, self.P)

    def stats(self) -> Dict[str, int]:
        s = Stats()
        _check(load().rad_batch_stats(self.h, C.byref(s)))
        return {k: getattr(s, k) for k, _ in Stats._fields_}

    def set_counting(self, on: bool):
        _check(load().rad_batch_set_counting(self.h, 1 if on else 0))

    @property
    def form(self) -> int:
        return int(load().rad_batch_form(self.h))

    def set_form(self, form: int):
        _check(load().rad_batch_set_form(self.h, form))

    def autotune(self, iters_per_trial: int = 4, rounds: int = 3) -> int:
        ch = C.c_int32()
        _check(load().rad_batch_autotune(self.h, iters_per_trial, rounds, C.byref(ch)))
        return ch.value

    def close(self):
        if self.h:
            load().rad_batch_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Adaptive:
    """Adaptive split variant (``rad_adapt``); updates ``scene`` in place."""

    def __init__(self, scene: Scene, tree: Octree, opts: Options, device: int = 0):
        self.scene = scene
        self.h = C.c_void_p()
        _check(load().rad_adapt_create(scene.h, tree.h, C.byref(opts), device, C.byref(self.h)))

    def run(self, max_steps: int = 1 << 62):
        sd, cv = C.c_int64(), C.c_int32()
        rc = _check(load().rad_adapt_run(self.h, max_steps, C.byref(sd), C.byref(cv)), allow=(RAD_ERR_WALK,))
        return sd.value, bool(cv.value), rc

    def set_speculation(self, wait: bool):
        """False: race the device's sample points (default); True: wait for each speculation."""
        _check(load().rad_adapt_set_speculation(self.h, 1 if wait else 0))

    def trace(self) -> np.ndarray:
        n = C.c_int64()
        _check(load().rad_adapt_trace(self.h, None, 0, C.byref(n)))
        out = np.zeros(n.value, np.int32)
        if n.value:
            _check(load().rad_adapt_trace(self.h, out.ctypes.data, n.value, C.byref(n)))
        return out.reshape(-1, 1)

    def stats(self) -> Dict[str, int]:
        s = Stats()
        hp, sp, sm = C.c_int64(), C.c_int64(), C.c_int64()
        _check(load().rad_adapt_stats(self.h, C.byref(s), C.byref(hp), C.byref(sp), C.byref(sm)))
        d = {k: getattr(s, k) for k, _ in Stats._fields_}
        d.update(host_points=hp.value, splits=sp.value, samples=sm.value)
        dp, sl, sc = C.c_int64(), C.c_int64(), C.c_int64()
        _check(load().rad_adapt_device_stats(self.h, C.byref(dp), C.byref(sl), C.byref(sc)))
        d.update(device_points=dp.value, speculations=sl.value, split_candidates=sc.value)
        return d

    def close(self):
        if self.h:
            load().rad_adapt_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class RenderOptions(C.Structure):
    """rad_render_options: the headless viewer's canvas, shading and rotation."""
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("shading", C.c_int32), ("pad", C.c_int32),
                ("x_rot", C.c_float), ("y_rot", C.c_float)]


def render_options(width=None, height=None, shading="flat", x_rot=0.0, y_rot=0.0) -> RenderOptions:
    o = RenderOptions()
    load().rad_render_options_default(C.byref(o))
    if width is not None:
        o.width = int(width)
    if height is not None:
        o.height = int(height)
    o.shading = {"flat": 0, "gouraud": 1}[shading]
    o.x_rot = float(x_rot)
    o.y_rot = float(y_rot)
    return o


def _render(call, arg, o: RenderOptions, device: int):
    import numpy as np
    img = np.empty((o.height, o.width, 4), dtype=np.uint8)
    _check(call(arg, C.byref(o), device, img.ctypes.data))
    return img


def render_fin(path: str, device: int = 0, **kw):
    """RGBA8 image (height, width, 4), top row first, of a .fin result as the viewer shows it."""
    return _render(load().rad_render_fin, path.encode(), render_options(**kw), device)


def render_scene(scene: "Scene", device: int = 0, **kw):
    """The same image of a scene in memory (the triangles its .fin would hold)."""
    return _render(load().rad_render_scene, scene.h, render_options(**kw), device)


def solve(tri_path: str, opts: Options, device: int = 0, max_steps: int = 1 << 62):
    """The reference's flow end to end: returns (scene, device solver, steps, converged)."""
    sc = Scene.load(tri_path, opts)
    tree = Octree(sc, opts.jobs)
    sc.init()
    sc.prepartition()
    dv = Device(sc, tree, opts, device)
    steps, conv, _ = dv.run(max_steps)
    dv.download(sc)
    return sc, dv, steps, conv
