"""Bounded device-side waits: failure detection without a GPU fault.

Every spin wait in the library's kernels is bounded by a %globaltimer
deadline.  When one runs out, the kernel records a device timeout, gives the
work in flight a second bounded wait, frees its TMEM and returns; the host
turns the record into XB_ERR_DEVICE_TIMEOUT and the context stays usable.

Option test_wait_timeout makes this happen on purpose in the fused fill +
tensor-core Gram kernel: before its first wait for an MMA commit, every CTA
waits with a 1 ms bound on an mbarrier that nothing arrives at, then waits
for the real commit with the full bound.  No wait is removed and nothing
faults; the data path is unchanged.  The tests check the error code, that
the next frame on the same context (option off) equals a clean run bit for
bit, and that the same context then still captures and replays frame
graphs.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _pair():
    from xbach.synth import make_pair
    T, S, info = make_pair(1)
    return T, S, dict(stampsx=info["stamps"], stampsy=info["stamps"],
                      threshHigh=info["threshHigh"])


def _result(ctx):
    import xbach
    return {"conv": ctx.image(xbach.XB_IMG_CONV), "diff": ctx.image(xbach.XB_IMG_DIFF),
            "sol": ctx.solution(), "mask": ctx.mask(), "ks": ctx.scalar("kernSum")}


def _same(a, b):
    for k in ("conv", "diff", "sol", "mask"):
        assert np.array_equal(np.asarray(a[k]).view(np.uint8), np.asarray(b[k]).view(np.uint8)), k
    assert a["ks"] == b["ks"]


def test_timed_out_wait_reports_and_context_recovers():
    import xbach
    T, S, kw = _pair()
    params = xbach.default_params(mode=xbach.XB_MODE_MIXED, **kw)
    clean = xbach.Context(params)
    clean.run_all(T, S)
    ref = _result(clean)
    clean.close()

    ctx = xbach.Context(params)
    ctx.set_option("test_wait_timeout", 1)
    ctx.init(T, S)
    ctx.sss()
    ctx.cmv()  # every fused-kernel CTA runs out of one bounded wait here
    with pytest.raises(xbach.XbError) as err:
        ctx.cd()  # the first stage that reads the device status back
    assert err.value.code == 11  # XB_ERR_DEVICE_TIMEOUT
    # reported once: the same context runs the next frame cleanly
    ctx.set_option("test_wait_timeout", 0)
    ctx.run_all(T, S)
    _same(_result(ctx), ref)
    # and twice in a row the error comes back and goes away again
    for on in (1, 0):
        ctx.set_option("test_wait_timeout", on)
        if on:
            with pytest.raises(xbach.XbError) as err:
                ctx.run_all(T, S)
            assert err.value.code == 11
        else:
            ctx.run_all(T, S)
            _same(_result(ctx), ref)
    ctx.close()


def test_graphs_after_a_timed_out_wait():
    """After the error, frame graphs on the same context capture and replay
    the clean frame bit for bit (the option is part of a graph's shape key)."""
    import torch
    import xbach
    T, S, kw = _pair()
    params = xbach.default_params(mode=xbach.XB_MODE_MIXED, **kw)
    clean = xbach.Context(params)
    clean.run_all(T, S)
    ref = clean.image(xbach.XB_IMG_DIFF, f64=False)
    clean.close()
    ctx = xbach.Context(params)
    ctx.set_option("graph", 1)
    ctx.set_option("test_wait_timeout", 1)
    with pytest.raises(xbach.XbError) as err:
        ctx.run(T, S)
    assert err.value.code == 11
    ctx.set_option("test_wait_timeout", 0)
    h, w = T.shape
    dT, dS = torch.from_numpy(T).cuda(), torch.from_numpy(S).cuda()
    dC, dD = torch.empty_like(dT), torch.empty_like(dT)
    for step in range(3):  # the first run of the shape captures, the others replay
        ctx.run_device(dT.data_ptr(), dS.data_ptr(), w, h, dC.data_ptr(), dD.data_ptr())
        torch.cuda.synchronize()
        assert ctx.scalar("graph_captured" if step == 0 else "graph_replay") == 1
        assert np.array_equal(dD.cpu().numpy().view(np.uint8), ref.view(np.uint8))
    ctx.close()
