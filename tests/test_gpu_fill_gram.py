"""The fused fill + tensor-core Gram kernel (csrc/xb_fill_gram.cu) against
the three kernels it replaces (k_fill_w_f32, k_fill_finish_f32, k_gram_tc),
which still run for the shapes it does not take (option fill_gram = 0).

Both compute the same W (hi and lo floats) by the same operations in the
same order and slice it with the same row exponents, and the tensor-core
sums are exact integers, so everything must agree bit for bit: W, Q and B
after cmv, and a whole frame's decisions, solution and images (the ksc
refills run the fused kernel on stamp lists).  The window of a stamp comes
by a TMA tile copy when it lies inside a frame whose rows are 16-byte
multiples (the 512 and 2048 px fields), by clamped loads otherwise (test01
is 330 px wide; stamps at the frame edge); option fill_gram_tma = 0 forces
the loads everywhere.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _case(name, test01):
    from xbach.synth import make_pair
    if name == "test01":
        return test01["T"].astype(np.float32), test01["S"].astype(np.float32), {}
    T, S, info = make_pair(int(name[-1]))
    return T, S, dict(stampsx=info["stamps"], stampsy=info["stamps"],
                      threshHigh=info["threshHigh"])


def _ctx(kw, fused, tma=1, trace=True, timers=False):
    import xbach
    ctx = xbach.Context(xbach.default_params(mode=xbach.XB_MODE_MIXED, **kw), trace=trace)
    ctx.set_option("fill_gram", fused)
    ctx.set_option("fill_gram_tma", tma)
    if timers:
        ctx.set_option("time_kernels", 1)
    return ctx


CMV_ARRAYS = {"Wf0": np.float32, "Wlo0": np.float32, "Wf1": np.float32, "Wlo1": np.float32,
              "Q0": np.float64, "Q1": np.float64, "B0": np.float64, "B1": np.float64}


def _cmv(T, S, kw, fused, tma=1):
    ctx = _ctx(kw, fused, tma, timers=True)
    ctx.init(T, S)
    ctx.sss()
    ctx.cmv()
    out = {k: ctx.array(k, dt) for k, dt in CMV_ARRAYS.items()}
    out["fused_launches"] = ctx.kernel_time("fill_gram")[1]
    out["fill_launches"] = ctx.kernel_time("fill_w")[1]
    ctx.close()
    return out


@pytest.mark.parametrize("name", ["test01", "config1", "config2"])
def test_cmv_fused_equals_separate_kernels(name, test01):
    T, S, kw = _case(name, test01)
    fused = _cmv(T, S, kw, 1)
    sep = _cmv(T, S, kw, 0)
    # the fused kernel ran (one launch per stamp set), the separate ones did not
    assert fused["fused_launches"] == 2 and fused["fill_launches"] == 0
    assert sep["fused_launches"] == 0 and sep["fill_launches"] == 2
    for k in CMV_ARRAYS:
        assert fused[k].shape == sep[k].shape and fused[k].size > 0, k
        assert np.array_equal(fused[k].view(np.uint8), sep[k].view(np.uint8)), k
    if name != "test01":
        # the TMA window copies give the loads' windows bit for bit
        loads = _cmv(T, S, kw, 1, tma=0)
        for k in CMV_ARRAYS:
            assert np.array_equal(fused[k].view(np.uint8), loads[k].view(np.uint8)), k


@pytest.mark.parametrize("name", ["test01", "config2"])
def test_frame_fused_equals_separate_kernels(name, test01):
    import xbach
    T, S, kw = _case(name, test01)
    res = {}
    for fused in (1, 0):
        ctx = _ctx(kw, fused, trace=True)
        ctx.run_all(T, S)
        res[fused] = dict(
            conv=ctx.image(xbach.XB_IMG_CONV), diff=ctx.image(xbach.XB_IMG_DIFF),
            sol=ctx.solution(), cur=ctx.array("cur", np.int32),
            rej=ctx.array("ksc_rejects", np.int32),
            ksc=ctx.scalar("ksc_iterations"), ct=ctx.scalar("convTemplate"),
            ks=ctx.scalar("kernSum"), mask=ctx.array("mask", np.uint16))
        ctx.close()
    a, b = res[1], res[0]
    assert a["ksc"] == b["ksc"] and a["ct"] == b["ct"]
    assert a["ks"] == b["ks"]
    for k in ("conv", "diff", "sol", "cur", "rej", "mask"):
        assert np.array_equal(np.asarray(a[k]).view(np.uint8), np.asarray(b[k]).view(np.uint8)), k
