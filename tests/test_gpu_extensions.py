"""HOTPANTS-style extensions on the GPU (xb_params gain / readNoise /
convPerPixel / fitWeighted) against the oracle's restatement.

Plain mode: every decision, the stamp chi^2 and the solution bit-identical;
the per-pixel convolution is an FMA chain in the oracle's order, so its
images are bit-identical too (the per-block images keep the parity suite's
1e-11 tolerance).  Mixed mode: the per-pixel FP32 convolution within the
mixed path's bar (1e-3 sigma) of the plain per-pixel one,
and a frame graph replays it bit for bit.
The defaults reproduce the reference (the parity suite runs with them)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _bits(a):
    return np.ascontiguousarray(a, np.float64).view(np.uint64)


def _same(a, b):
    return a.shape == b.shape and np.array_equal(_bits(a), _bits(b))


CASES = {
    "noise_model": dict(gain=1.7, readNoise=5.0),
    "per_pixel": dict(convPerPixel=1),
    "both": dict(gain=2.3, readNoise=3.0, convPerPixel=1),
    "weighted_fit": dict(fitWeighted=1, readNoise=5.0),
}


@pytest.fixture(scope="module")
def field():
    from xbach.synth import make_pair
    T, S, info = make_pair(1)
    return T, S, dict(stampsx=info["stamps"], stampsy=info["stamps"], threshHigh=info["threshHigh"])


@pytest.fixture(scope="module", params=sorted(CASES))
def both(request, oracle, field):
    import xbach
    T, S, kw = field
    kw = {**kw, **CASES[request.param]}
    ref = oracle.run(oracle.default_params(**kw), T.astype(np.float64), S.astype(np.float64))
    assert ref.status == 0
    ctx = xbach.Context(xbach.default_params(**kw), trace=True)
    ctx.run_all(T, S)
    return request.param, ref, ctx


def test_plain_decisions_and_chi2_bit_exact(both):
    _, ref, ctx = both
    assert ctx.scalar("convTemplate") == ref.scalar("convTemplate")
    assert ctx.scalar("ksc_iterations") == ref.scalar("ksc_iterations")
    for k in ("ksc_rejects", "cur"):
        assert np.array_equal(ctx.array(k, np.int32), ref.array(k, np.int32)), k
    for k in ("ksc_sig_last", "solution"):
        assert _same(ctx.array(k, np.float64), ref.array(k, np.float64)), k
    assert _same(np.array([ctx.scalar("kernSum")]), np.array([ref.scalar("kernSum")]))
    assert np.array_equal(ctx.array("mask", np.uint16), ref.array("mask", np.uint16))


def test_plain_images(both):
    name, ref, ctx = both
    for k in ("conv", "diff"):
        a, b = ctx.array(k, np.float64), ref.array(k, np.float64)
        if CASES[name].get("convPerPixel"):
            assert _same(a, b), k
        else:
            assert np.abs(a - b).max() <= 1e-11 * np.abs(ref.array("conv", np.float64)).max(), k


def test_gain_alone_scales_the_chi2(field):
    """No read noise: chi^2 terms scale by the gain exactly (a power of two),
    decisions and images stay those of the reference's model."""
    import xbach
    T, S, kw = field
    out = []
    for g in (0.0, 4.0):
        ctx = xbach.Context(xbach.default_params(gain=g, **kw), trace=True)
        ctx.run_all(T, S)
        out.append(ctx)
    a, b = out[1].array("ksc_sig_last", np.float64), out[0].array("ksc_sig_last", np.float64)
    valid = b != -1.0
    assert valid.any() and np.array_equal(a[valid], 4.0 * b[valid])
    assert np.array_equal(out[1].array("cur", np.int32), out[0].array("cur", np.int32))
    assert _same(out[1].image(xbach.XB_IMG_DIFF), out[0].image(xbach.XB_IMG_DIFF))


SIGMA_BAR = {"config1": 1e-3, "test01": 1e-3}


@pytest.mark.parametrize("src", ["config1", "test01"])
def test_mixed_per_pixel_within_1e3_sigma_of_plain(field, test01, src):
    import xbach
    from xbach.accuracy import diff_error
    if src == "test01":
        T, S, kw = test01["T"].astype(np.float32), test01["S"].astype(np.float32), {}
    else:
        T, S, kw = field
    res = {}
    for mode in (xbach.XB_MODE_PLAIN, xbach.XB_MODE_MIXED):
        ctx = xbach.Context(xbach.default_params(mode=mode, convPerPixel=1, **kw))
        ctx.run_all(T, S)
        res[mode] = (ctx.image(xbach.XB_IMG_DIFF), ctx.image(xbach.XB_IMG_CONV),
                     ctx.scalar("convTemplate"), ctx.mask())
    d_p, c_p, ct, m_p = res[xbach.XB_MODE_PLAIN]
    d_m, _, ct_m, m_m = res[xbach.XB_MODE_MIXED]
    assert ct == ct_m
    # masks agree except where the FP32 good-fraction test sits on 0.99
    assert np.mean(m_p != m_m) < 1e-4
    target = S if ct == 1 else T
    e = diff_error(d_m, d_p, c_p, target)
    assert e["pixels"] > 0.8 * T.size and e["max_sigma"] <= SIGMA_BAR[src], e


def test_mixed_per_pixel_graph_replays_stage_by_stage(field):
    import xbach
    from xbach.synth import make_pair
    T, S, kw = field
    params = xbach.default_params(mode=xbach.XB_MODE_MIXED, convPerPixel=1, **kw)
    frames = [(T, S), make_pair(1, frame=1)[:2]]
    refs = []
    for t, s in frames:
        ctx = xbach.Context(params)
        ctx.run_all(t, s)
        refs.append(ctx.image(xbach.XB_IMG_DIFF, f64=False))
    g = xbach.Context(params)
    g.set_option("graph", 1)
    for i in (0, 1, 0):
        g.run(*frames[i])
        assert np.array_equal(g.image(xbach.XB_IMG_DIFF, f64=False), refs[i]), i
    # switching the option back is another shape: a new capture, block kernels
    blk = xbach.Context(xbach.default_params(mode=xbach.XB_MODE_MIXED, **kw))
    blk.run_all(T, S)
    g.set_params(xbach.default_params(mode=xbach.XB_MODE_MIXED, **kw))
    g.run(T, S)
    assert np.array_equal(g.image(xbach.XB_IMG_DIFF, f64=False),
                          blk.image(xbach.XB_IMG_DIFF, f64=False))


@pytest.mark.parametrize("mode", ["plain", "mixed"])
def test_weighted_fit_with_constant_weight_two_is_exact(field, mode):
    """Unbounded gain, read noise 0.5: every fit weight is exactly 2, so the
    weighted normal equations are exactly twice the unweighted ones and the
    results are bit-identical (mixed mode compared with its CUDA-core FP64
    Gram, the path a weighted fit takes)."""
    import xbach
    T, S, kw = field
    md = xbach.XB_MODE_PLAIN if mode == "plain" else xbach.XB_MODE_MIXED
    out = []
    for wfit in (0, 1):
        ctx = xbach.Context(xbach.default_params(mode=md, gain=1e300, readNoise=0.5,
                                                 fitWeighted=wfit, **kw))
        if mode == "mixed":
            ctx.set_option("gram_fp64", 1)
        ctx.run_all(T, S)
        out.append((ctx.solution(), ctx.image(xbach.XB_IMG_DIFF), ctx.scalar("ksc_iterations")))
    assert _same(out[0][0], out[1][0]) and _same(out[0][1], out[1][1]) and out[0][2] == out[1][2]


def test_mixed_weighted_fit_within_1e3_sigma_of_plain(field):
    import xbach
    from xbach.accuracy import diff_error
    T, S, kw = field
    res = {}
    for mode in (xbach.XB_MODE_PLAIN, xbach.XB_MODE_MIXED):
        ctx = xbach.Context(xbach.default_params(mode=mode, fitWeighted=1, readNoise=5.0, **kw))
        ctx.run_all(T, S)
        res[mode] = (ctx.image(xbach.XB_IMG_DIFF), ctx.image(xbach.XB_IMG_CONV),
                     ctx.scalar("convTemplate"))
    d_p, c_p, ct = res[xbach.XB_MODE_PLAIN]
    d_m, _, ct_m = res[xbach.XB_MODE_MIXED]
    assert ct == ct_m
    e = diff_error(d_m, d_p, c_p, S if ct == 1 else T)
    assert e["pixels"] > 0.8 * T.size and e["max_sigma"] <= 1e-3, e


def test_plain_input_mask_matches_oracle(oracle, field):
    """An input mask (a block and a bad column): the plain GPU path equals the
    oracle's masked run on the init mask, the substamp sets, every ksc
    decision, the chi^2, the solution and the final mask; images within the
    parity suite's 1e-11."""
    import xbach
    T, S, kw = field
    m = np.zeros(T.shape, np.uint8)
    m[200:230, 300:340] = 1
    m[:, 77] = 1
    ref = oracle.run(oracle.default_params(**kw), T.astype(np.float64), S.astype(np.float64),
                     mask=m)
    assert ref.status == 0
    ctx = xbach.Context(xbach.default_params(**kw), trace=True)
    ctx.set_input_mask(m)
    ctx.run_all(T, S)
    assert np.array_equal(ctx.array("mask_init", np.uint16), ref.array("mask_init", np.uint16))
    for k in ("ss_xy0", "ss_xy1", "ksc_rejects", "cur"):
        assert np.array_equal(ctx.array(k, np.int32), ref.array(k, np.int32)), k
    for k in ("ksc_sig_last", "solution"):
        assert _same(ctx.array(k, np.float64), ref.array(k, np.float64)), k
    assert _same(np.array([ctx.scalar("kernSum")]), np.array([ref.scalar("kernSum")]))
    assert np.array_equal(ctx.array("mask", np.uint16), ref.array("mask", np.uint16))
    scale = np.abs(ref.array("conv", np.float64)).max()
    for k in ("conv", "diff"):
        assert np.abs(ctx.array(k, np.float64) - ref.array(k, np.float64)).max() <= 1e-11 * scale, k
