"""Seeded synthetic scenes in the reference's ``.tri`` text format.

A ``.tri`` file is a sequence of blocks (reference ``src/rad.cpp:47-111``)::

    Triangle
    Fr Fg Fb Br Bg Bb          # reflectance 0..255, emission (a 255 channel = light)
    x y z                      # three vertices
    x y z
    x y z

Every builder returns a :class:`Scene` (numpy arrays plus the command-line
options the workload runs with).  All randomness comes from a
``numpy.random.Generator(PCG64(seed))`` so a scene is a pure function of its
parameters.  The workloads follow the benchmark definitions:

* :func:`room`     -- closed box room, each wall an ``q x q`` grid of quads split
  into two triangles; ``q=8`` gives the 768-triangle room, ``q=64`` the
  49,152-triangle walls of the 64x64 room.
* :func:`room_with_boxes` -- the room plus seeded, non-overlapping axis-aligned
  boxes (edges U[0.5,3], faces ``b x b`` quads, reflectance U[0.2,0.8]).
* :func:`hall`     -- 40x20x100 hall with hexagonal-prism pillars and four
  rectangular ceiling emitters.
* :func:`batch_rooms` -- the many-scene batch: per-scene seeds, triangle counts
  log-uniform in [500, 50000], 0-32 boxes.

Emission: the ``.tri`` format marks a light by a background channel equal to
255 and scales every light by the one global ``-light`` factor
(``src/rad.cpp:274-280``), so all emitters of a scene share one magnitude.
"""
from __future__ import annotations

import dataclasses
import math
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

GRAY = (191, 191, 191)          # round(255 * 0.75)
RED_WALL = (161, 15, 10)        # round(255 * (0.63, 0.06, 0.04))
GREEN_WALL = (38, 122, 23)      # round(255 * (0.15, 0.48, 0.09))
LIGHT_SCALE_15 = 15.0 / 255.0   # emission (1,1,1)*15 expressed as Brgb 255 * -light


@dataclasses.dataclass
class Scene:
    """Triangles of one scene plus the options it is run with."""
    vtx: np.ndarray                   # float32 [n, 3, 3]
    frgb: np.ndarray                  # int32 [n, 3]
    brgb: np.ndarray                  # int32 [n, 3]
    options: Dict[str, str]           # reference CLI options, e.g. {"-converge": "0.45"}
    name: str = "scene"

    @property
    def n(self) -> int:
        return int(self.vtx.shape[0])

    def to_tri(self) -> str:
        """Render as ``.tri`` text.  Coordinates are printed with 9 significant
        digits, which parse back to the same float32 values."""
        v = self.vtx.astype(np.float32).astype(np.float64).reshape(-1, 9).tolist()
        c = np.concatenate([self.frgb, self.brgb], axis=1).astype(np.int64).tolist()
        blk = "Triangle \n%d %d %d %d %d %d\n%.9g %.9g %.9g\n%.9g %.9g %.9g\n%.9g %.9g %.9g\n"
        return "".join(blk % (tuple(ci) + tuple(vi)) for ci, vi in zip(c, v))

    def write(self, path: str) -> str:
        with open(path, "w") as fh:
            fh.write(self.to_tri())
        return path

    def argv(self, extra: Optional[Dict[str, str]] = None) -> List[str]:
        opts = dict(self.options)
        if extra:
            opts.update(extra)
        args: List[str] = []
        for k, val in opts.items():
            args.append(k)
            if val is not None:
                args.append(str(val))
        return args


def concat(scenes: Sequence[Scene], options: Dict[str, str], name: str) -> Scene:
    return Scene(np.concatenate([s.vtx for s in scenes]).astype(np.float32),
                 np.concatenate([s.frgb for s in scenes]).astype(np.int32),
                 np.concatenate([s.brgb for s in scenes]).astype(np.int32), options, name)


def _grid_quads(origin, u, v, nu: int, nv: int):
    """Quads of a planar grid; returns [nu*nv, 4, 3] corners (o, o+u, o+u+v, o+v)."""
    o = np.asarray(origin, np.float64)
    u = np.asarray(u, np.float64)
    v = np.asarray(v, np.float64)
    i = np.arange(nu)[:, None]
    j = np.arange(nv)[None, :]
    a = o + (i[..., None] / nu) * u + (j[..., None] / nv) * v
    b = o + ((i[..., None] + 1) / nu) * u + (j[..., None] / nv) * v
    c = o + ((i[..., None] + 1) / nu) * u + ((j[..., None] + 1) / nv) * v
    d = o + (i[..., None] / nu) * u + ((j[..., None] + 1) / nv) * v
    q = np.stack([a, b, c, d], axis=2).reshape(nu * nv, 4, 3)
    return q


def _quads_to_tris(q: np.ndarray) -> np.ndarray:
    t1 = q[:, [0, 1, 2]]
    t2 = q[:, [0, 2, 3]]
    return np.stack([t1, t2], axis=1).reshape(-1, 3, 3)


def _wall(origin, u, v, nu, nv, frgb, brgb=(0, 0, 0), light_mask=None):
    q = _grid_quads(origin, u, v, nu, nv)
    tris = _quads_to_tris(q)
    n = tris.shape[0]
    fr = np.tile(np.asarray(frgb, np.int32), (n, 1))
    br = np.tile(np.asarray(brgb, np.int32), (n, 1))
    if light_mask is not None:
        lm = np.repeat(light_mask(q), 2)
        br[lm] = 255
    return tris, fr, br


def room(q: int = 8, size: float = 10.0, light_scale: float = LIGHT_SCALE_15,
         emitter: Tuple[float, float] = (0.375, 0.625), converge: Optional[float] = None,
         name: Optional[str] = None) -> Scene:
    """Closed room [0,size]^3, walls of q x q quads, normals facing inward.

    The emitter is the set of ceiling quads whose centres fall in
    ``[emitter[0]*size, emitter[1]*size]^2`` (the centre 2x2 quads for q=8).
    ``converge`` defaults to 1e-3 of one emitter's initial unshot key
    (3 channels * 100 * 255 * light_scale), the config-1 stopping rule.
    """
    s = float(size)
    lo, hi = emitter[0] * s, emitter[1] * s

    def ceiling_light(quads):
        c = quads.mean(axis=1)
        return (c[:, 0] > lo) & (c[:, 0] < hi) & (c[:, 2] > lo) & (c[:, 2] < hi)

    parts = [
        _wall((0, 0, 0), (0, 0, s), (s, 0, 0), q, q, GRAY),                   # floor y=0, normal +y
        _wall((0, s, 0), (s, 0, 0), (0, 0, s), q, q, GRAY, light_mask=ceiling_light),  # ceiling, -y
        _wall((0, 0, s), (0, s, 0), (s, 0, 0), q, q, GRAY),                   # back z=s, -z
        _wall((0, 0, 0), (s, 0, 0), (0, s, 0), q, q, GRAY),                   # front z=0, +z
        _wall((0, 0, 0), (0, s, 0), (0, 0, s), q, q, RED_WALL),               # left x=0, +x
        _wall((s, 0, 0), (0, 0, s), (0, s, 0), q, q, GREEN_WALL),             # right x=s, -x
    ]
    vtx = np.concatenate([p[0] for p in parts]).astype(np.float32)
    fr = np.concatenate([p[1] for p in parts])
    br = np.concatenate([p[2] for p in parts])
    if converge is None:
        converge = 1e-3 * 3 * 100 * 255 * light_scale
    opts = {"-light": repr(float(np.float32(light_scale))), "-converge": repr(float(np.float32(converge)))}
    return Scene(vtx, fr, br, opts, name or f"room{q}")


def _box_tris(lo, hi, b: int, frgb) -> Tuple[np.ndarray, np.ndarray, np.ndarray]:
    lo = np.asarray(lo, np.float64)
    hi = np.asarray(hi, np.float64)
    d = hi - lo
    ex, ey, ez = np.array([d[0], 0, 0]), np.array([0, d[1], 0]), np.array([0, 0, d[2]])
    faces = [  # outward normals
        (lo, ez, ey), (lo + ex, ey, ez),          # x- , x+
        (lo, ex, ez), (lo + ey, ez, ex),          # y- , y+
        (lo, ey, ex), (lo + ez, ex, ey),          # z- , z+
    ]
    tris = []
    for o, u, v in faces:
        tris.append(_quads_to_tris(_grid_quads(o, u, v, b, b)))
    t = np.concatenate(tris)
    n = t.shape[0]
    return t, np.tile(np.asarray(frgb, np.int32), (n, 1)), np.zeros((n, 3), np.int32)


def _place_boxes(rng, n_boxes: int, size: float, edge=(0.5, 3.0), tries: int = 10000):
    boxes: List[Tuple[np.ndarray, np.ndarray]] = []
    for _ in range(tries):
        if len(boxes) >= n_boxes:
            break
        e = rng.uniform(edge[0], edge[1], 3)
        c = rng.uniform(e / 2 + 1e-3, size - e / 2 - 1e-3)
        lo, hi = c - e / 2, c + e / 2
        if hi[1] > size * 0.9:          # keep clear of the ceiling emitter plane
            continue
        ok = all(np.any(hi <= blo) or np.any(lo >= bhi) for blo, bhi in boxes)
        if ok:
            boxes.append((lo, hi))
    return boxes


def room_with_boxes(q: int = 64, n_boxes: int = 16, box_q: int = 8, seed: int = 2000, size: float = 10.0,
                    light_scale: float = LIGHT_SCALE_15, converge_frac: float = 1e-4,
                    name: Optional[str] = None) -> Scene:
    """The room plus ``n_boxes`` seeded axis-aligned boxes (faces box_q x box_q quads)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    base = room(q, size, light_scale)
    parts = [base]
    for lo, hi in _place_boxes(rng, n_boxes, size):
        fr = np.rint(255 * rng.uniform(0.2, 0.8, 3)).astype(np.int32)
        t, f, b = _box_tris(lo, hi, box_q, fr)
        parts.append(Scene(t.astype(np.float32), f, b, {}))
    converge = converge_frac * 3 * 100 * 255 * light_scale
    opts = {"-light": base.options["-light"], "-converge": repr(float(np.float32(converge)))}
    return concat(parts, opts, name or f"room{q}_boxes{n_boxes}")


def config1() -> Scene:
    """768-triangle room, converge at 1e-3 of an emitter's key (no triangle splits)."""
    return room(8, name="config1_room768")


def config2(seed: int = 2000) -> Scene:
    """64x64-quad walls + 16 seeded boxes (8x8-quad faces); converge at 1e-4."""
    s = room_with_boxes(64, 16, 8, seed=seed, name="config2_room64_boxes16")
    s.options.update({"-adapt_area": "5", "-delta_ff": "5e-6", "-triangle": "200000"})
    return s


def hall(target_tris: int = 400_000, n_pillars: int = 300, seed: int = 3000,
         light_scale: float = 12.5 / 255.0, name: Optional[str] = None) -> Scene:
    """40x20x100 hall (x, y-up, z); walls/floor/ceiling tessellated to about
    ``target_tris``; hexagonal pillars r~U[0.3,1], full height; four
    rectangular ceiling emitters sharing one magnitude."""
    rng = np.random.Generator(np.random.PCG64(seed))
    X, Y, Z = 40.0, 20.0, 100.0
    area = 2 * X * Z + 2 * Y * Z + 2 * X * Y
    s = math.sqrt(area / (target_tris / 2))
    nx, ny, nz = max(1, round(X / s)), max(1, round(Y / s)), max(1, round(Z / s))
    emitters = [(10, 25), (30, 25), (10, 75), (30, 75)]

    def ceiling_light(quads):
        c = quads.mean(axis=1)
        m = np.zeros(len(c), bool)
        for ex, ez in emitters:
            m |= (np.abs(c[:, 0] - ex) < 2.0) & (np.abs(c[:, 2] - ez) < 3.0)
        return m

    parts = [
        _wall((0, 0, 0), (0, 0, Z), (X, 0, 0), nz, nx, GRAY),
        _wall((0, Y, 0), (X, 0, 0), (0, 0, Z), nx, nz, GRAY, light_mask=ceiling_light),
        _wall((0, 0, Z), (0, Y, 0), (X, 0, 0), ny, nx, GRAY),
        _wall((0, 0, 0), (X, 0, 0), (0, Y, 0), nx, ny, GRAY),
        _wall((0, 0, 0), (0, Y, 0), (0, 0, Z), ny, nz, RED_WALL),
        _wall((X, 0, 0), (0, 0, Z), (0, Y, 0), nz, ny, GREEN_WALL),
    ]
    vt = [p[0] for p in parts]
    fr = [p[1] for p in parts]
    br = [p[2] for p in parts]
    placed: List[Tuple[float, float, float]] = []
    for _ in range(100000):
        if len(placed) >= n_pillars:
            break
        r = rng.uniform(0.3, 1.0)
        cx, cz = rng.uniform(r + 0.05, X - r - 0.05), rng.uniform(r + 0.05, Z - r - 0.05)
        if all((cx - px) ** 2 + (cz - pz) ** 2 > (r + pr + 0.05) ** 2 for px, pz, pr in placed):
            placed.append((cx, cz, r))
    for cx, cz, r in placed:
        ang = np.arange(6) * (np.pi / 3)
        ring = np.stack([cx + r * np.cos(ang), np.zeros(6), cz + r * np.sin(ang)], 1)
        top = ring + np.array([0, Y, 0])
        tris = []
        for k in range(6):
            a, b = ring[k], ring[(k + 1) % 6]
            c, d = top[(k + 1) % 6], top[k]
            tris += [[a, c, b], [a, d, c]]
        ctr_b, ctr_t = np.array([cx, 0, cz]), np.array([cx, Y, cz])
        for k in range(6):
            tris.append([ctr_b, ring[k], ring[(k + 1) % 6]])
            tris.append([ctr_t, top[(k + 1) % 6], top[k]])
        t = np.asarray(tris, np.float64)
        vt.append(t)
        fr.append(np.tile(np.rint(255 * rng.uniform(0.2, 0.8, 3)).astype(np.int32), (len(t), 1)))
        br.append(np.zeros((len(t), 3), np.int32))
    key = 3 * 100 * 255 * light_scale
    opts = {"-light": repr(float(np.float32(light_scale))), "-converge": repr(float(np.float32(1e-4 * key))),
            "-triangle": "1000000"}
    return Scene(np.concatenate(vt).astype(np.float32), np.concatenate(fr).astype(np.int32),
                 np.concatenate(br).astype(np.int32), opts, name or "config3_hall")


def _rotation(axis, angle):
    a = np.asarray(axis, np.float64)
    a = a / np.linalg.norm(a)
    c, s_ = math.cos(angle), math.sin(angle)
    x, y, z = a
    return np.array([[c + x * x * (1 - c), x * y * (1 - c) - z * s_, x * z * (1 - c) + y * s_],
                     [y * x * (1 - c) + z * s_, c + y * y * (1 - c), y * z * (1 - c) - x * s_],
                     [z * x * (1 - c) - y * s_, z * y * (1 - c) + x * s_, c + z * z * (1 - c)]])


def precision_stress(n_slabs: int = 64, seed: int = 5000, thickness: float = 1e-3) -> Scene:
    """The 768-triangle room with emitters spanning a 1e4 power range and thin
    slabs at grazing angles to them (the precision stress case).

    Emitters: the centre 2x2 ceiling quads.  A light needs one background
    channel equal to 255 and every light shares the global -light scale, so
    the range is carried by the other channels: one quad is (255, X, X) with
    X chosen so its total emission is 1e4 times that of the three (255, 0, 0)
    quads; with -light = 0.1/255 those emit (0.1, 0, 0) and the strong one
    about (0.1, 500, 500).
    Slabs: 1.5 x thickness x 1.5 boxes, tilted 1-5 degrees off vertical
    (nearly parallel to the downward emitter rays), seeded positions."""
    rng = np.random.Generator(np.random.PCG64(seed))
    scale = 0.1 / 255.0
    X = int(round((1e4 * 255 - 255) / 2))
    base = room(8, light_scale=scale)
    vtx, fr, br = base.vtx.copy(), base.frgb.copy(), base.brgb.copy()
    lights = np.nonzero((br == 255).any(axis=1))[0]
    # the first light quad (two triangles) becomes the strong emitter
    br[lights] = (255, 0, 0)
    br[lights[:2]] = (255, X, X)
    parts = [Scene(vtx, fr, br, {})]
    for _ in range(n_slabs):
        lo = np.array([-0.75, -thickness / 2, -0.75])
        hi = -lo
        t, f, b = _box_tris(lo, hi, 1, np.rint(255 * rng.uniform(0.2, 0.8, 3)).astype(np.int32))
        # stand the slab up (its thin axis horizontal), then tilt it slightly
        R = _rotation((1, 0, 0), math.pi / 2) @ _rotation(rng.normal(size=3), math.radians(rng.uniform(1, 5)))
        R = _rotation((0, 1, 0), rng.uniform(0, 2 * math.pi)) @ R
        c = rng.uniform((1.5, 1.0, 1.5), (8.5, 8.0, 8.5))
        t = t @ R.T + c
        parts.append(Scene(t.astype(np.float32), f, b, {}))
    key = 100.0 * (255 + 2 * X) * scale
    opts = {"-light": repr(float(np.float32(scale))), "-converge": repr(float(np.float32(1e-3 * key)))}
    return concat(parts, opts, "config5_precision")


def batch_rooms(n_scenes: int = 256, seed: int = 4000, lo: int = 500, hi: int = 50_000,
                max_boxes: int = 32) -> List[Scene]:
    """Independent rooms with per-scene seeds; triangle counts log-uniform in
    [lo, hi] (realised through the wall grid size), 0..max_boxes boxes."""
    out: List[Scene] = []
    for s in range(n_scenes):
        rng = np.random.Generator(np.random.PCG64(seed + s))
        target = math.exp(rng.uniform(math.log(lo), math.log(hi)))
        nb = int(rng.integers(0, max_boxes + 1))
        q = max(2, int(math.sqrt(target / 12)))
        b = max(1, q // 8)
        while q > 2 and 12 * q * q + nb * 12 * b * b > target:
            q -= 1
            b = max(1, q // 8)
        sc = room_with_boxes(q, nb, b, seed=seed * 7 + s, name=f"batch{s}")
        out.append(sc)
    return out
