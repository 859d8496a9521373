"""The C-ABI library loads and exports every entry point include/*.h declares."""
import ctypes
import glob
import os
import re
import subprocess

import pytest

from hwrad import build, capi

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    names = set()
    for h in glob.glob(os.path.join(REPO, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:[A-Za-z_][\w\s\*]*?)\b(rad_\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return names


def test_header_declarations_found():
    d = declared()
    assert "rad_dev_run" in d and "rad_scene_load" in d and len(d) >= 20


def test_library_exports_every_declared_symbol(built):
    lib = ctypes.CDLL(build.LIB)
    missing = [n for n in sorted(declared()) if not hasattr(lib, n)]
    assert not missing, missing
    assert set(capi.EXPORTS) <= declared()


def test_nm_dynamic_symbols(built):
    out = subprocess.run(["nm", "-D", "--defined-only", build.LIB], capture_output=True, text=True).stdout
    syms = {l.split()[-1] for l in out.splitlines() if l.strip()}
    assert declared() <= syms


def test_options_defaults_match_reference(built):
    o = capi.options()
    # src/rad.cpp:17-31
    assert (o.debug, o.adapt_area, o.sample_area, o.converge) == (0, 5.0, -1.0, 1200.0)
    assert abs(o.delta_ff - 0.000005) < 1e-12
    assert (o.write_cycle, o.triangle_limit, o.light_scale, o.jobs, o.parallel_src) == (10, 1000000, 1.0, 2, 1)
    assert o.precision == 32


def test_device_entry_points_fail_cleanly_without_device(built, workdir):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a device is present")
    from hwrad import scenes
    s = scenes.room(2, emitter=(0.0, 1.0))
    tri = s.write(os.path.join(workdir, "nodev.tri"))
    o = capi.options_from_argv(s.argv())
    sc = capi.Scene.load(tri, o)
    tree = capi.Octree(sc)
    sc.init()
    with pytest.raises(capi.RadError) as e:
        capi.Device(sc, tree, o)
    assert e.value.code == capi.RAD_ERR_NODEV


def test_device_preparation_fails_cleanly_without_device(built, workdir):
    """The device forms of the octree build and of InitRadiosity report
    RAD_ERR_NODEV on a machine without a GPU; the host forms still work."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a device is present")
    from hwrad import scenes
    s = scenes.room(2, emitter=(0.0, 1.0))
    tri = s.write(os.path.join(workdir, "nodev2.tri"))
    o = capi.options_from_argv(s.argv())
    sc = capi.Scene.load(tri, o)
    with pytest.raises(capi.RadError) as e:
        capi.Octree(sc, device=0)
    assert e.value.code == capi.RAD_ERR_NODEV
    with pytest.raises(capi.RadError) as e:
        sc.init(device=0)
    assert e.value.code == capi.RAD_ERR_NODEV
    capi.Octree(sc, 1)
    sc.init()
