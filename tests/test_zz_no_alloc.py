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
    cl_kern/sss.cl:19-38)."""
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


def _call(fn, img, mask, w, h, geom, n, fsw, p, stream):
    import torch
    sky = torch.full((n,), float("nan"), dtype=torch.float64, device="cuda")
    fwhm = torch.full((n,), float("nan"), dtype=torch.float64, device="cuda")
    err = ctypes.create_string_buffer(256)
    rc = fn(img.data_ptr(), mask.data_ptr(), w, h, geom.data_ptr(), n, fsw,
            p.sigClipAlpha, p.iqRange, sky.data_ptr(), fwhm.data_ptr(), stream, err, 256)
    assert rc == 0, err.value
    torch.cuda.synchronize()
    return sky.cpu().numpy(), fwhm.cpu().numpy()


def test_noalloc_edge_stamps_match_oracle(oracle, test01):
    """Caller-given stamps whose fStampWidth^2 window ends exactly at, or is
    clipped by, the right or bottom frame edge (the reference's own grid
    never clips one): sky and sigma equal the CPU oracle's calcStats, bit for
    bit, on two calls in a row, and the mask comes back as the oracle leaves
    it."""
    import torch
    import xbach
    T, S, kw = inputs("test01", test01)
    h, w = T.shape
    p = xbach.default_params(**kw)
    ctx = xbach.Context(p, trace=True)
    ctx.init(T, S)
    mask0 = ctx.array("mask_init", np.uint16).reshape(h, w)
    fsw = 51
    g = np.array([(w - fsw, 0, fsw, fsw),           # touches the right edge
                  (0, h - fsw, fsw, fsw),           # touches the bottom edge
                  (w - fsw, h - fsw, fsw, fsw),     # the corner
                  (w - 30, 100, 30, fsw),           # clipped by the right edge
                  (120, h - 20, fsw, 20),           # clipped by the bottom edge
                  (w - 25, h - 40, 25, 40),         # clipped by both
                  (150, 150, fsw, fsw)], np.int32)
    sky_ref, fwhm_ref, mask_ref = oracle.stamp_stats(T.astype(np.float64), mask0, g, fsw,
                                                     p.sigClipAlpha, p.iqRange)
    fn = bind(xbach.lib())
    img = torch.from_numpy(T).cuda()
    geom = torch.from_numpy(g.ravel().copy()).cuda()
    for call in range(2):
        mask = torch.from_numpy(mask0.view(np.int16).copy()).cuda()
        sky, fwhm = _call(fn, img, mask, w, h, geom, len(g), fsw, p,
                          torch.cuda.current_stream().cuda_stream)
        assert np.array_equal(sky.view(np.uint64), sky_ref.view(np.uint64)), call
        assert np.array_equal(fwhm.view(np.uint64), fwhm_ref.view(np.uint64)), call
        assert np.array_equal(mask.cpu().numpy().view(np.uint16).reshape(h, w), mask_ref)


def test_noalloc_invalid_geometry_gives_nan_and_spares_the_rest(test01):
    """Stamps outside the image, or whose size is not the full stamp width
    clipped by the image edge, get NaN statistics (none of their pixels is
    read); the valid stamps around them keep the stage API's values."""
    import torch
    import xbach
    T, S, kw = inputs("test01", test01)
    h, w = T.shape
    p = xbach.default_params(**kw)
    ctx = xbach.Context(p, trace=True)
    ctx.init(T, S)
    ctx.sss()
    nx, ny, fsw = (int(ctx.scalar(k)) for k in ("stampsx", "stampsy", "fStampWidth"))
    g = stamp_geometry(w, h, nx, ny, fsw)
    n = len(g)
    bad = {1: (w - 5, 0, 10, 10),         # past the right edge
           3: (-1, 0, 10, 10),            # negative x
           5: (0, h - 3, 4, 4),           # past the bottom edge
           7: (0, 0, fsw + 1, 4),         # wider than fStampWidth
           9: (0, 0, 0, 4),               # empty
           11: (10 ** 9, 10 ** 9, 4, 4),  # far outside
           13: (60, 60, 17, 40)}          # narrower than the clipped window
    for i, v in bad.items():
        g[i] = v
    mask0 = ctx.array("mask_init", np.uint16).reshape(h, w)
    mask = torch.from_numpy(mask0.view(np.int16).copy()).cuda()
    sky, fwhm = _call(bind(xbach.lib()), torch.from_numpy(T).cuda(), mask, w, h,
                      torch.from_numpy(g).cuda(), n, fsw, p, torch.cuda.current_stream().cuda_stream)
    isbad = np.zeros(n, bool)
    isbad[list(bad)] = True
    assert np.isnan(sky[isbad]).all() and np.isnan(fwhm[isbad]).all()
    sky_ref, fwhm_ref = ctx.array("sky0", np.float64), ctx.array("fwhm0", np.float64)
    assert np.array_equal(sky[~isbad].view(np.uint64), sky_ref[~isbad].view(np.uint64))
    assert np.array_equal(fwhm[~isbad].view(np.uint64), fwhm_ref[~isbad].view(np.uint64))


def test_noalloc_nan_pixels_are_flagged_like_the_stage_api(test01):
    """NaN pixels inside stamps: the returned mask carries NAN_PIXEL |
    BAD_INPUT at exactly those pixels, and sky and sigma equal xb_sss's."""
    import torch
    import xbach
    T, S, kw = inputs("test01", test01)
    h, w = T.shape
    T = T.copy()
    rng = np.random.default_rng(7)
    ys, xs = rng.integers(40, h - 40, 12), rng.integers(40, w - 40, 12)
    T[ys, xs] = np.nan
    p = xbach.default_params(**kw)
    ctx = xbach.Context(p, trace=True)
    ctx.init(T, S)
    ctx.sss()
    assert ctx.scalar("sss_retry") == 0
    nx, ny, fsw = (int(ctx.scalar(k)) for k in ("stampsx", "stampsy", "fStampWidth"))
    mask0 = ctx.array("mask_init", np.uint16).reshape(h, w)
    assert (mask0[ys, xs] == 0).all()     # NaN passes maskInput's comparisons
    mask = torch.from_numpy(mask0.view(np.int16).copy()).cuda()
    g = stamp_geometry(w, h, nx, ny, fsw)
    sky, fwhm = _call(bind(xbach.lib()), torch.from_numpy(T).cuda(), mask, w, h,
                      torch.from_numpy(g).cuda(), nx * ny, fsw, p,
                      torch.cuda.current_stream().cuda_stream)
    got = mask.cpu().numpy().view(np.uint16).reshape(h, w)
    flag = (1 << 3) | (1 << 7)   # XB_MASK_NAN_PIXEL | XB_MASK_BAD_INPUT
    changed = got != mask0
    covered = np.zeros((h, w), bool)   # pixels inside some stamp's fStampWidth^2 area
    for x0, y0, _, _ in g:
        covered[y0:y0 + fsw, x0:x0 + fsw] = True
    nan_in = np.zeros((h, w), bool)
    nan_in[ys, xs] = True
    nan_in &= covered
    assert nan_in.any()
    assert np.array_equal(changed, nan_in)
    assert (got[nan_in] == (mask0[nan_in] | flag)).all()
    assert np.array_equal(sky.view(np.uint64), ctx.array("sky0", np.float64).view(np.uint64))
    assert np.array_equal(fwhm.view(np.uint64), ctx.array("fwhm0", np.float64).view(np.uint64))


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
