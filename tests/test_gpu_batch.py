"""Batches of frame pairs (xb_batch_*): every frame's result equals the same
pair run alone on one context, for frames of different sizes and more frames
than workers."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def frames(test01):
    from xbach.synth import make_pair
    out = [(test01["T"].astype(np.float32), test01["S"].astype(np.float32), {})]
    for f in range(3):
        T, S, info = make_pair(1, frame=f)
        out.append((T, S, dict(stampsx=info["stamps"], stampsy=info["stamps"],
                               threshHigh=info["threshHigh"])))
    return out


@pytest.mark.parametrize("mode", ["plain", "mixed"])
def test_batch_equals_single_runs(test01, mode):
    import xbach
    m = xbach.XB_MODE_PLAIN if mode == "plain" else xbach.XB_MODE_MIXED
    fr = frames(test01)
    # one parameter set per batch: group the synthetic frames (same stamp grid)
    syn = fr[1:]
    params = xbach.default_params(mode=m, **syn[0][2])
    batch = xbach.Batch(params, workers=2)
    convs = [np.empty_like(T) for T, _, _ in syn]
    diffs = [np.empty_like(T) for T, _, _ in syn]
    st, ks = batch.run([T for T, _, _ in syn], [S for _, S, _ in syn], convs, diffs)
    assert st == [0] * len(syn)
    for i, (T, S, kw) in enumerate(syn):
        ctx = xbach.Context(xbach.default_params(mode=m, **kw))
        ctx.run_all(T, S)
        assert np.array_equal(ctx.image(xbach.XB_IMG_DIFF, f64=False), diffs[i]), i
        assert np.array_equal(ctx.image(xbach.XB_IMG_CONV, f64=False), convs[i]), i
        assert ks[i] == ctx.scalar("kernSum")


def test_batch_mixed_sizes_and_device_frames(test01):
    import torch
    import xbach
    fr = frames(test01)
    sel = [fr[0], fr[1]]  # 330x330 and 512x512 with the default stamp grid
    params = xbach.default_params(mode=xbach.XB_MODE_MIXED)
    batch = xbach.Batch(params, workers=2)
    dT = [torch.from_numpy(T).cuda() for T, _, _ in sel]
    dS = [torch.from_numpy(S).cuda() for _, S, _ in sel]
    dD = [torch.empty_like(t) for t in dT]
    s = torch.cuda.Stream()
    batch.set_stream(s.cuda_stream)
    st, _ = batch.run_ptrs([t.data_ptr() for t in dT], [t.data_ptr() for t in dS],
                           [t.shape[1] for t in dT], [t.shape[0] for t in dT],
                           None, [t.data_ptr() for t in dD], device=True)
    s.synchronize()
    assert st == [0, 0]
    for i, (T, S, _) in enumerate(sel):
        ctx = xbach.Context(params)
        ctx.run_all(T, S)
        assert np.array_equal(ctx.image(xbach.XB_IMG_DIFF, f64=False), dD[i].cpu().numpy()), i


def test_batch_reports_failing_frame():
    import xbach
    batch = xbach.Batch(xbach.default_params(mode=xbach.XB_MODE_MIXED), workers=2)
    good = np.full((64, 64), 100.0, np.float32)
    # a frame whose template and science disagree in size cannot be expressed
    # through run(); an all-zero frame has no substamps (XB_ERR_NO_SUBSTAMPS)
    zero = np.zeros((256, 256), np.float32)
    with pytest.raises(xbach.XbError) as e:
        batch.run([zero], [zero])
    assert "frame 0" in str(e.value)
    L = xbach.lib()
    st = (ctypes.c_int * 1)()
    rc = L.xb_batch_run(batch.h, 1, None, None, None, None, None, None, st, None)
    assert rc == 1  # XB_ERR_ARG: null frame arrays
    del good


@pytest.mark.parametrize("graph", [0, 1])
def test_batch_per_frame_parameters(test01, graph):
    """Pairs with their own stamp grids and thresholds in one batch (preset-4
    style); every result equals a single context run with that pair's
    parameters, stage by stage."""
    import xbach
    from xbach.synth import make_pair
    pairs = [(test01["T"].astype(np.float32), test01["S"].astype(np.float32),
              dict(stampsx=10, stampsy=10))]
    for f, grid in enumerate((6, 13, 8)):
        T, S, info = make_pair(1, frame=f)
        pairs.append((T, S, dict(stampsx=grid, stampsy=grid + 1, threshHigh=info["threshHigh"])))
    mode = xbach.XB_MODE_MIXED
    params = [xbach.default_params(mode=mode, **kw) for _, _, kw in pairs]
    batch = xbach.Batch(params[0], workers=3)
    batch.set_params(params)
    if graph:
        batch.set_option("graph", 1)
    refs = []
    for (T, S, _), p in zip(pairs, params):
        ctx = xbach.Context(p)
        ctx.run_all(T, S)
        refs.append((ctx.image(xbach.XB_IMG_DIFF, f64=False), ctx.scalar("kernSum"),
                     ctx.scalar("stampsx")))
    for rep in range(2 if graph else 1):
        diffs = [np.empty_like(T) for T, _, _ in pairs]
        st, ks = batch.run([T for T, _, _ in pairs], [S for _, S, _ in pairs], None, diffs)
        assert st == [0] * len(pairs)
        for i, (d, k, _) in enumerate(refs):
            assert np.array_equal(diffs[i], d), (rep, i)
            assert ks[i] == k, (rep, i)
    # back to the batch's own parameters
    batch.set_params([])
    st, _ = batch.run([pairs[1][0]], [pairs[1][1]])
    assert st == [0]


def test_batch_parameters_must_keep_the_fit():
    import xbach
    base = xbach.default_params(mode=xbach.XB_MODE_MIXED)
    batch = xbach.Batch(base, workers=1)
    with pytest.raises(xbach.XbError):
        batch.set_params([xbach.default_params(mode=xbach.XB_MODE_MIXED, kernelOrder=1)])
    with pytest.raises(xbach.XbError):
        batch.set_params([xbach.default_params(mode=xbach.XB_MODE_PLAIN)])
    ctx = xbach.Context(base)
    with pytest.raises(xbach.XbError):
        ctx.set_params(xbach.default_params(mode=xbach.XB_MODE_MIXED, hKernelWidth=8))
    ctx.set_params(xbach.default_params(mode=xbach.XB_MODE_MIXED, stampsx=7, threshHigh=3e4))
