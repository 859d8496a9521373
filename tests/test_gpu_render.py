"""Headless render of a result on the GPU (rad_render_fin / rad_render_scene)
against the C++ restatement of the viewer (oracle/raster_oracle.cpp), bit for
bit: the default view in flat shading, Gouraud from a rotated view, and an
image size that is not a multiple of the 16-pixel tile."""
import os
import subprocess

import numpy as np
import pytest

import runner
from hwrad import capi, scenes
from test_raster_oracle import RASTER, fin_cases

pytestmark = pytest.mark.gpu


def _oracle_image(fin, w, h, shading, xr, yr, workdir):
    out = os.path.join(workdir, f"o_{w}_{h}_{shading}_{xr}_{yr}.rgba")
    subprocess.run([RASTER, fin, out, str(w), str(h), str(shading), str(xr), str(yr)], check=True)
    return np.fromfile(out, np.uint8).reshape(h, w, 4)


def _recoloured(fin, workdir):
    """The same geometry with colours spread over 40..254 (results of a few
    steps are nearly black, which would hide shading differences)."""
    rng = np.random.default_rng(11)
    lines = open(fin).read().split("\n")
    out, i = [], 0
    while i < len(lines):
        if lines[i] == "Triangle ":
            c = rng.integers(40, 255, 3)
            out += [lines[i], f"{c[0]} {c[1]} {c[2]} 0 0 0"] + lines[i + 2:i + 5]
            i += 5
        else:
            i += 1
    path = os.path.join(workdir, os.path.basename(fin) + ".colour.fin")
    with open(path, "w") as fh:
        fh.write("\n".join(out) + "\n")
    return path


VIEWS = [(1024, 768, "flat", 0.0, 0.0), (1024, 768, "gouraud", 25.0, 35.0), (333, 257, "flat", -40.0, 120.0),
         (333, 257, "gouraud", 10.0, -60.0)]


def test_render_equals_restatement(built, workdir):
    for name, fin in fin_cases(workdir):
        for path in (fin, _recoloured(fin, workdir)):
            for w, h, shading, xr, yr in VIEWS:
                got = capi.render_fin(path, width=w, height=h, shading=shading, x_rot=xr, y_rot=yr)
                want = _oracle_image(path, w, h, {"flat": 0, "gouraud": 1}[shading], xr, yr, workdir)
                bad = np.argwhere((got != want).any(axis=2))
                assert len(bad) == 0, (name, path, w, h, shading, xr, yr, len(bad), bad[:5].tolist())
                assert (want[:, :, :3] != [0, 51, 51]).any(), "the model must be in view"


def test_render_scene_equals_render_fin(built, workdir):
    """The image of a solved scene in memory equals the image of its .fin."""
    sc = scenes.room_with_boxes(12, 6, 2, seed=7, size=30.0)
    tri = sc.write(os.path.join(workdir, "rs.tri"))
    o = capi.options_from_argv(sc.argv({"-triangle": "4000"}))
    scene, dv, steps, conv = capi.solve(tri, o, max_steps=80)
    prefix = os.path.join(workdir, "rs_out")
    scene.write_fin(prefix)
    for shading in ("flat", "gouraud"):
        a = capi.render_scene(scene, shading=shading, x_rot=20.0, y_rot=30.0)
        b = capi.render_fin(prefix + ".fin", shading=shading, x_rot=20.0, y_rot=30.0)
        assert np.array_equal(a, b)
    dv.close()


def test_render_empty_fin(built, workdir):
    """No triangles: the clear colour everywhere."""
    path = os.path.join(workdir, "empty.fin")
    open(path, "w").close()
    img = capi.render_fin(path, width=40, height=24)
    assert (img.reshape(-1, 4) == [0, 51, 51, 255]).all()
