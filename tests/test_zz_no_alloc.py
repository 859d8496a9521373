"""rad_dev_form_factors_noalloc: the form-factor query for callers that
cannot allocate device memory at the call (a renderer or simulation loop whose
own allocator holds the memory budget, or a real-time loop that cannot take
an allocation's synchronisation).

The caller owns the receiver and output buffers (here: torch tensors); the
entry point keeps its shooter records in a fixed device array.  Its results
must equal rad_dev_form_factors' bit for bit (the tolerance of the other
parity tests), on two calls in a row that reuse that array.
"""
import os

import numpy as np
import pytest

from hwrad import capi, scenes

pytestmark = pytest.mark.gpu


def _device(workdir, fp64=False):
    s = scenes.room_with_boxes(10, 5, 2, seed=31, size=12.0)
    tri = s.write(os.path.join(workdir, f"noalloc_{int(fp64)}.tri"))
    o = capi.options_from_argv(s.argv(), precision=64 if fp64 else 32)
    sc = capi.Scene.load(tri, o)
    tree = capi.Octree(sc, 2)
    sc.init()
    sc.prepartition()
    return sc, tree, capi.Device(sc, tree, o)


@pytest.mark.parametrize("fp64", [False, True])
def test_noalloc_equals_allocating_entry_point(built, workdir, fp64):
    import torch

    sc, tree, dv = _device(workdir, fp64)
    n = sc.view()["n"]
    rcv = np.arange(0, n, 3, dtype=np.int32)
    ft, tt = (np.float64, torch.float64) if fp64 else (np.float32, torch.float32)
    d_rcv = torch.from_numpy(rcv).cuda()
    stream = torch.cuda.current_stream().cuda_stream
    rng = np.random.default_rng(5)
    calls = [rng.choice(n, 7, replace=False).astype(np.int32), rng.choice(n, 64, replace=False).astype(np.int32)]
    for src in calls:   # two calls in a row: the second reuses the first's scratch
        d_ff = torch.full((len(src), len(rcv), 3), float("nan"), dtype=tt, device="cuda")
        dev_before = torch.cuda.current_device()
        rc = dv.form_factors_noalloc(src, d_rcv.data_ptr(), len(rcv), d_ff.data_ptr(), stream)
        assert rc == capi.RAD_OK, capi.load().rad_last_error()
        assert torch.cuda.current_device() == dev_before   # the caller's current device is left as it was
        torch.cuda.synchronize()
        got = d_ff.cpu().numpy()
        for s_i, s in enumerate(src):
            want = dv.form_factors(int(s), rcv, dtype=ft)
            assert np.array_equal(got[s_i].view(np.uint8), want.view(np.uint8)), int(s)
        assert np.isfinite(got).all() and (got > 0).any()


def test_noalloc_limits(built, workdir):
    import torch

    sc, tree, dv = _device(workdir)
    n = sc.view()["n"]
    d_rcv = torch.arange(4, dtype=torch.int32, device="cuda")
    d_ff = torch.zeros((65, 4, 3), dtype=torch.float32, device="cuda")
    assert dv.form_factors_noalloc(np.arange(65, dtype=np.int32), d_rcv.data_ptr(), 4, d_ff.data_ptr()) == \
        capi.RAD_ERR_CAPACITY
    assert dv.form_factors_noalloc(np.array([n], np.int32), d_rcv.data_ptr(), 4, d_ff.data_ptr()) == capi.RAD_ERR_ARG
    # a receiver id outside the scene gives NaN, the others are computed
    bad = torch.tensor([0, n + 5, 1], dtype=torch.int32, device="cuda")
    rc = dv.form_factors_noalloc(np.array([2], np.int32), bad.data_ptr(), 3, d_ff.data_ptr())
    assert rc == capi.RAD_OK
    torch.cuda.synchronize()
    out = d_ff[0, :3].cpu().numpy()
    assert np.isnan(out[1]).all() and np.isfinite(out[0]).all() and np.isfinite(out[2]).all()
