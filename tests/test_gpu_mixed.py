"""The mixed-precision (chosen) path against the plain path and the oracle.

Acceptance (the throughput metric's accuracy condition): the chosen difference image is within 1e-3 of
the per-pixel noise sigma of the plain GPU result,
sigma_pix = sqrt(|S| + |conv| + 2 sigma_rn^2) with the frames' read noise
sigma_rn = 5 ADU (gain 1), over pixels both paths leave unmasked.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SIGMA_RN = 5.0


def run(mode, T, S, kw, trace=True):
    import xbach
    ctx = xbach.Context(xbach.default_params(mode=mode, **kw), trace=trace)
    ctx.run_all(T, S)
    return ctx


def case(name, test01):
    from xbach.synth import make_pair
    if name == "test01":
        return test01["T"].astype(np.float32), test01["S"].astype(np.float32), {}
    T, S, info = make_pair(int(name[-1]))
    return T, S, dict(stampsx=info["stamps"], stampsy=info["stamps"],
                      threshHigh=info["threshHigh"])


@pytest.fixture(scope="module", params=["test01", "config1", "config2"])
def both(request, test01):
    import xbach
    T, S, kw = case(request.param, test01)
    plain = run(xbach.XB_MODE_PLAIN, T, S, kw)
    mixed = run(xbach.XB_MODE_MIXED, T, S, kw)
    return request.param, T, S, plain, mixed


def test_same_stamp_sets_and_direction(both):
    _, _, _, plain, mixed = both
    for k in ("ss_xy0", "ss_xy1", "ss_count0", "ss_count1"):
        assert np.array_equal(plain.array(k, np.int32), mixed.array(k, np.int32)), k
    assert plain.scalar("convTemplate") == mixed.scalar("convTemplate")


# test01 (the reference's 330x330 golden case) has a global system with
# cond ~6e13 and a negative kernel sum; there rounding W to FP32 alone moves
# the difference image by 1.2e-3 sigma, which is why the mixed path keeps W
# as a hi + lo pair of floats.  Every case is held to the metric's 1e-3 sigma.
SIGMA_BAR = {"test01": 1e-3, "config1": 1e-3, "config2": 1e-3}
KSUM_BAR = {"test01": 1e-5, "config1": 1e-5, "config2": 1e-5}


def test_cd_kernel_sums_and_test_sets(both):
    """The mixed path solves each stamp's test system by a warp-per-stamp
    LDL^T (the kernel sum is the only output cd uses); its kernel sums agree
    with the plain LU's and the cd test lists are the same."""
    _, _, _, plain, mixed = both
    for si in (0, 1):
        a = mixed.array("kernel_sums%d" % si, np.float64)
        b = plain.array("kernel_sums%d" % si, np.float64)
        assert a.shape == b.shape and a.size > 0
        assert np.max(np.abs(a / b - 1)) < 1e-6, (si, np.max(np.abs(a / b - 1)))
        try:
            tp = plain.array("cd_test%d" % si, np.int32)
        except KeyError:
            continue
        assert np.array_equal(mixed.array("cd_test%d" % si, np.int32), tp), si


def test_kernel_sum_close(both):
    name, _, _, plain, mixed = both
    assert abs(mixed.scalar("kernSum") / plain.scalar("kernSum") - 1) < KSUM_BAR[name]


def test_diff_within_1e3_sigma_of_plain(both):
    import xbach
    name, T, S, plain, mixed = both
    dp = plain.image(xbach.XB_IMG_DIFF)
    dm = mixed.image(xbach.XB_IMG_DIFF)
    cp = plain.image(xbach.XB_IMG_CONV)
    ct = plain.scalar("convTemplate")
    target = S if ct else T   # the image subtracted from the convolved one
    from xbach.accuracy import is_bad
    ok = ~is_bad(dp) & ~is_bad(dm)
    assert ok.mean() > 0.5
    sigma = np.sqrt(np.abs(target) + np.abs(cp) + 2 * SIGMA_RN ** 2)
    err = np.abs(dm - dp)[ok] / sigma[ok]
    assert err.max() <= SIGMA_BAR[name], (name, err.max())
    # masks agree except where the FP32 good-fraction test sits on 0.99
    mp, mm = plain.array("mask", np.uint16), mixed.array("mask", np.uint16)
    assert np.mean(mp != mm) < 1e-4


@pytest.mark.parametrize("name", ["test01", "config1"])
def test_tensor_core_gram_matches_fp64_gram(name, test01):
    """Q and B from the tensor-core slicing agree with the FP64 CUDA-core
    accumulation of the same W (hi + lo, exact in FP64).  The slicing rounds
    every element to 2^-36 of its row maximum (the only approximation; the
    slice products are exact), which moves a Gram entry by ~1e-11 of the
    largest entry."""
    import xbach
    T, S, kw = case(name, test01)
    out = {}
    for fp64 in (0, 1):
        ctx = xbach.Context(xbach.default_params(mode=xbach.XB_MODE_MIXED, **kw), trace=True)
        ctx.set_option("gram_fp64", fp64)
        ctx.init(T, S)
        ctx.sss()
        ctx.cmv()
        out[fp64] = {k: ctx.array(k, np.float64) for k in ("Q0", "Q1", "B0", "B1")}
    for k in ("Q0", "Q1", "B0", "B1"):
        a, b = out[0][k], out[1][k]
        scale = np.max(np.abs(b))
        assert scale > 0
        assert np.max(np.abs(a - b)) <= 1e-10 * scale, (k, np.max(np.abs(a - b)) / scale)
