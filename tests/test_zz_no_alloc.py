"""The allocation-free stamp-statistics entry point, xb_stamp_stats_noalloc.

It serves callers that cannot allocate device memory themselves (another
allocator owns the device, or a cudaMalloc would stall their work): its
scratch is a fixed array inside the library.  Here the test owns every
device buffer, calls the entry point through the C ABI twice in a row, and
requires both results to equal, bit for bit, the per-stamp sky and robust
sigma that the stage API (xb_sss) computes for the same image and mask — the
tolerance the other statistics tests use.  This file is collected last.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def stamp_geometry(w, h, nx, ny, fsw):
    """{x, y, width, height} of every grid stamp (createStampBounds,
    cl_kern/sss.cl:86-105)."""
    g = np.zeros((nx * ny, 4), np.int32)
    for i in range(nx * ny):
        sx, sy = i % nx, i // nx
        x0, y0 = sx * w // nx, sy * h // ny
        g[i] = (x0, y0, min(x0 + fsw, w) - x0, min(y0 + fsw, h) - y0)
    return g


def bind(L):
    vp, i, d = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
    L.xb_stamp_stats_noalloc.argtypes = [vp, vp, i, i, vp, i, i, d, d, vp, vp, vp,
                                         ctypes.c_char_p, ctypes.c_size_t]
    return L.xb_stamp_stats_noalloc


def inputs(case, test01):
    from xbach.synth import make_pair
    if case == "test01":
        return test01["T"].astype(np.float32), test01["S"].astype(np.float32), {}
    T, S, info = make_pair(2)
    return T, S, dict(stampsx=info["stamps"], stampsy=info["stamps"],
                      threshHigh=info["threshHigh"])


@pytest.mark.parametrize("case", ["test01", "config2"])
def test_noalloc_stats_equal_stage_api_twice(case, test01):
    import torch
    import xbach
    T, S, kw = inputs(case, test01)
    h, w = T.shape
    p = xbach.default_params(**kw)
    ctx = xbach.Context(p, trace=True)
    ctx.init(T, S)
    ctx.sss()
    assert ctx.scalar("sss_retry") == 0   # template statistics use the init mask
    mask0 = ctx.array("mask_init", np.uint16).reshape(h, w)
    sky_ref = ctx.array("sky0", np.float64)
    fwhm_ref = ctx.array("fwhm0", np.float64)
    nx, ny, fsw = (int(ctx.scalar(k)) for k in ("stampsx", "stampsy", "fStampWidth"))
    geom = torch.from_numpy(stamp_geometry(w, h, nx, ny, fsw)).cuda()
    img = torch.from_numpy(T).cuda()
    n = nx * ny
    fn = bind(xbach.lib())
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):
        mask = torch.from_numpy(mask0.view(np.int16).copy()).cuda()
        sky = torch.full((n,), float("nan"), dtype=torch.float64, device="cuda")
        fwhm = torch.full((n,), float("nan"), dtype=torch.float64, device="cuda")
        err = ctypes.create_string_buffer(256)
        rc = fn(img.data_ptr(), mask.data_ptr(), w, h, geom.data_ptr(), n, fsw,
                p.sigClipAlpha, p.iqRange, sky.data_ptr(), fwhm.data_ptr(), stream, err, 256)
        assert rc == 0, err.value
        torch.cuda.synchronize()
        got_sky, got_fwhm = sky.cpu().numpy(), fwhm.cpu().numpy()
        assert np.array_equal(got_sky.view(np.uint64), sky_ref.view(np.uint64)), call
        assert np.array_equal(got_fwhm.view(np.uint64), fwhm_ref.view(np.uint64)), call
        # the mask is in/out; without NaN pixels it comes back unchanged
        assert np.array_equal(mask.cpu().numpy().view(np.uint16).reshape(h, w), mask0)


def test_noalloc_rejects_requests_beyond_the_scratch():
    import torch
    import xbach
    fn = bind(xbach.lib())
    img = torch.zeros(64 * 64, dtype=torch.float32, device="cuda")
    mask = torch.zeros(64 * 64, dtype=torch.int16, device="cuda")
    geom = torch.zeros(4 * 4, dtype=torch.int32, device="cuda")
    out = torch.zeros(4, dtype=torch.float64, device="cuda")
    err = ctypes.create_string_buffer(256)
    rc = fn(img.data_ptr(), mask.data_ptr(), 64, 64, geom.data_ptr(), 10000, 200, 3.0, 1.35,
            out.data_ptr(), out.data_ptr(), None, err, 256)
    assert rc == 10   # XB_ERR_UNSUPPORTED, nothing launched
    assert b"32 MiB" in err.value
