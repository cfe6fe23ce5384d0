"""GPU parity: the plain CUDA path against the CPU oracle on the same inputs.

Integer / index results (masks, stamp and substamp sets, rejection sets) and
every FP64 quantity that decides one of them must be bit-identical; the
output images are compared within the FP tolerances stated per test.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _u64(a):
    return np.ascontiguousarray(a, np.float64).view(np.uint64)


def bit_equal(a, b):
    return a.shape == b.shape and np.array_equal(_u64(a), _u64(b))


CASES = ["test01", "config1", "config2"]


@pytest.fixture(scope="module", params=CASES)
def pair(request, oracle, test01):
    import xbach
    from xbach.synth import make_pair
    if request.param == "test01":
        T, S = test01["T"].astype(np.float32), test01["S"].astype(np.float32)
        kw = {}
    else:
        cfg = int(request.param[-1])
        T, S, info = make_pair(cfg)
        kw = dict(stampsx=info["stamps"], stampsy=info["stamps"],
                  threshHigh=info["threshHigh"])
    ref = oracle.run(oracle.default_params(**kw), T.astype(np.float64),
                     S.astype(np.float64), keep_w=True)
    assert ref.status == 0
    ctx = xbach.Context(xbach.default_params(**kw), trace=True)
    ctx.init(T, S)
    ctx.sss()
    ctx.cmv()
    return request.param, ref, ctx


def test_init_mask(pair):
    _, ref, ctx = pair
    assert np.array_equal(ctx.array("mask_init", np.uint16), ref.array("mask_init", np.uint16))


def test_sss_grid(pair):
    _, ref, ctx = pair
    for k in ("stampsx", "stampsy", "fStampWidth", "sss_retry", "nstamps0", "nstamps1"):
        assert ctx.scalar(k) == ref.scalar(k), k


@pytest.mark.parametrize("name", ["sky0", "fwhm0", "sky1", "fwhm1", "ss_val_all0",
                                  "ss_val_all1", "ss_val0", "ss_val1"])
def test_sss_stats_bit_exact(pair, name):
    _, ref, ctx = pair
    assert bit_equal(ctx.array(name, np.float64), ref.array(name, np.float64)), name


@pytest.mark.parametrize("name", ["ss_count_all0", "ss_count_all1", "ss_xy_all0",
                                  "ss_xy_all1", "stamp_index0", "stamp_index1",
                                  "ss_count0", "ss_count1", "ss_xy0", "ss_xy1"])
def test_sss_sets_identical(pair, name):
    _, ref, ctx = pair
    assert np.array_equal(ctx.array(name, np.int32), ref.array(name, np.int32)), name


def test_sss_mask(pair):
    _, ref, ctx = pair
    assert np.array_equal(ctx.array("mask_sss", np.uint16), ref.array("mask_sss", np.uint16))


@pytest.mark.parametrize("name", ["W0", "W1", "Q0", "Q1", "B0", "B1"])
def test_cmv_bit_exact(pair, name):
    _, ref, ctx = pair
    a, b = ctx.array(name, np.float64), ref.array(name, np.float64)
    assert a.shape == b.shape
    assert bit_equal(a, b), (name, np.abs(a - b).max())
