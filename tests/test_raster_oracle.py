"""Headless render of a result (rad_render_*), CPU half: the viewer
restatement's input preparation against the reference's own model converter
(WebGL_demo/model-converter/main.cpp, built from its source by oracle/Makefile),
and the render entry points' argument errors, which return before any CUDA
call.  The shader half has no runnable reference here (it is WebGL): the GPU
tests hold the CUDA rasteriser to the C++ restatement bit for bit."""
import json
import os
import subprocess

import numpy as np
import pytest

import runner
from hwrad import capi, scenes

RASTER = os.path.join(runner.HERE, "_build", "raster_oracle")
CONVERTER = os.path.join(runner.HERE, "_ref", "model_converter")


def _fin(workdir, name, scene, extra, steps, binary=None):
    tri = scene.write(os.path.join(workdir, f"{name}.tri"))
    wd = os.path.join(workdir, f"ras_{name}")
    os.makedirs(wd, exist_ok=True)
    if binary:
        runner.run(binary, tri, scene.argv(extra), steps=steps, workdir=wd)
    else:
        runner.oracle(tri, scene.argv(extra), steps=steps, workdir=wd)
    return os.path.join(wd, "out.fin")


def fin_cases(workdir):
    cases = [("boxes", _fin(workdir, "boxes", scenes.room_with_boxes(12, 6, 2, seed=7, size=30.0),
                            {"-triangle": "4000"}, 60))]
    if os.path.exists(runner.REF32):
        cases.append(("room8_ref", _fin(workdir, "room8_ref", scenes.room(8), {}, 200, runner.REF32)))
    return cases


@pytest.mark.skipif(not os.path.exists(CONVERTER), reason="reference converter not built (no reference tree)")
def test_converter_restatement_equals_reference(built, workdir):
    for name, fin in fin_cases(workdir):
        out = os.path.join(workdir, f"{name}.json")
        subprocess.run([CONVERTER, "-i", fin, "-o", out, "--format", "COLOR"], check=True, capture_output=True)
        j = json.load(open(out))
        arr = os.path.join(workdir, f"{name}.arrays")
        subprocess.run([RASTER, "--arrays", fin, arr], check=True)
        a = np.fromfile(arr, np.float32)
        n = len(a) // 27
        assert n > 0
        for k, key in enumerate(("vertexPositions", "vertexNormals", "vertexFrontColors")):
            want = np.array(j[key], dtype=np.float64).astype(np.float32)   # JSON text -> Float32Array
            got = a[k * n * 9:(k + 1) * n * 9]
            assert np.array_equal(want.view(np.uint32), got.view(np.uint32)), (name, key)


def test_render_argument_errors(built, workdir):
    L = capi.load()
    img = np.zeros(16, np.uint8)
    o = capi.render_options(width=2, height=2)
    assert L.rad_render_fin(os.path.join(workdir, "missing.fin").encode(), o, 0, img.ctypes.data) == capi.RAD_ERR_IO
    bad = os.path.join(workdir, "bad.fin")
    with open(bad, "w") as fh:
        fh.write("Triangle \n1 2 3 0 0 0\n1 2 3 0 0 1\nnot numbers\n")
    assert L.rad_render_fin(bad.encode(), o, 0, img.ctypes.data) == capi.RAD_ERR_PARSE
    z = capi.render_options(width=0, height=5)
    assert L.rad_render_fin(bad.encode(), z, 0, img.ctypes.data) == capi.RAD_ERR_CAPACITY
    s = capi.render_options(width=2, height=2)
    s.shading = 7
    assert L.rad_render_fin(bad.encode(), s, 0, img.ctypes.data) == capi.RAD_ERR_ARG


SHADER_PIN = os.path.join(runner.HERE, "_ref", "shader_pin")


@pytest.mark.skipif(not os.path.isdir(os.path.join(runner.HERE, "_ref", "src_shaders")),
                    reason="the viewer's shader sources were not staged (no reference tree)")
def test_viewer_shader_sources_equal_the_restatement(built):
    """The shader half: the viewer's own gouraud.vs, flat.vs and flat.fs,
    compiled as C++ against oracle/glsl_shim.h (builtins as the shim states
    them), against the restatement's vertex and fragment stages that its
    render() and the CUDA rasteriser follow -- bit for bit on 600k seeded
    vertices and fragments in three views.  Clip positions are only reported
    (the shader multiplies P x MV first); they must agree to a small fraction
    of a pixel."""
    import subprocess as sp
    sp.run(["make", "-s", "-C", runner.HERE, "_ref/shader_pin"], check=True)
    r = sp.run([SHADER_PIN, "200000"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    w = r.stdout.split()
    vals = {w[i]: w[i + 1] for i in range(0, len(w) - 1, 2)}
    assert int(vals["samples"]) == 600000
    assert vals["gouraud_vs_mismatch"] == vals["flat_vs_mismatch"] == vals["flat_fs_mismatch"] == "0"
    assert float(vals["gl_position_max_window_diff_px"]) < 0.01
