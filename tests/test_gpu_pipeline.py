"""Streaming pipeline over FITS files (xb_pipeline_*): every pair's output
files hold the images xb_run gives on a single context, in both modes and
with frame graphs, across repeated runs; bad pairs fail alone with the
reference's error kinds; FP64 files run the plain stages."""
import numpy as np
import pytest

from xbach_testlib import read_fits, write_fits

pytestmark = pytest.mark.gpu


def _pairs(tmp, n, config=1, **kw):
    from xbach.synth import make_pair
    out = []
    for f in range(n):
        T, S, info = make_pair(config, frame=f, **kw)
        tp, sp = tmp / f"t{f}.fits", tmp / f"s{f}.fits"
        write_fits(tp, T)
        write_fits(sp, S)
        out.append((tp, sp, T, S, info))
    return out


def _params(mode, info):
    import xbach
    md = {"plain": xbach.XB_MODE_PLAIN, "mixed": xbach.XB_MODE_MIXED}[mode]
    return xbach.default_params(mode=md, stampsx=info["stamps"], stampsy=info["stamps"],
                                threshHigh=info["threshHigh"])


def _single(params, T, S):
    import xbach
    ctx = xbach.Context(params)
    ctx.run(T, S)
    return (ctx.image(xbach.XB_IMG_CONV, f64=False), ctx.image(xbach.XB_IMG_DIFF, f64=False),
            ctx.scalar("kernSum"))


@pytest.mark.parametrize("mode,graph", [("plain", 0), ("mixed", 0), ("mixed", 1)])
def test_pipeline_matches_single_context(tmp_path, mode, graph):
    import xbach
    pr = _pairs(tmp_path, 6)
    params = _params(mode, pr[0][4])
    refs = [_single(params, T, S) for _, _, T, S, _ in pr]
    pl = xbach.Pipeline(params, workers=3, io=2)
    if graph:
        pl.set_option("graph", 1)
    convs = [tmp_path / f"conv{i}.fits" for i in range(len(pr))]
    diffs = [tmp_path / f"sub{i}.fits" for i in range(len(pr))]
    for rep in range(2):
        for p in convs + diffs:
            p.unlink(missing_ok=True)
        st, ks = pl.run_files([p[0] for p in pr], [p[1] for p in pr], convs, diffs)
        assert st == [0] * len(pr)
        for i, (conv, diff, kern) in enumerate(refs):
            assert np.array_equal(read_fits(convs[i]), conv.astype(np.float64)), (rep, i)
            assert np.array_equal(read_fits(diffs[i]), diff.astype(np.float64)), (rep, i)
            assert ks[i] == kern, (rep, i)
        s = pl.stats()
        npx = sum(T.size for _, _, T, _, _ in pr)
        assert s["pairs"] == len(pr)
        assert s["bytes_read"] == 2 * 4 * npx and s["bytes_written"] == 2 * 4 * npx
        assert s["wall_ms"] > 0 and s["compute_ms"] > 0


def test_pipeline_bad_pairs_fail_alone(tmp_path):
    import xbach
    pr = _pairs(tmp_path, 3)
    T, S = pr[0][2], pr[0][3]
    params = _params("plain", pr[0][4])
    # a pair of another size, and an FP64 pair (plain stages on FP64 samples)
    write_fits(tmp_path / "small.fits", S[:256, :256])
    T64 = T.astype(np.float64) + 0.125
    S64 = S.astype(np.float64)
    write_fits(tmp_path / "t64.fits", T64, bitpix=-64)
    write_fits(tmp_path / "s64.fits", S64, bitpix=-64)
    tps = [pr[0][0], tmp_path / "missing.fits", pr[1][0], tmp_path / "t64.fits", pr[2][0]]
    sps = [pr[0][1], pr[1][1], tmp_path / "small.fits", tmp_path / "s64.fits", pr[2][1]]
    diffs = [tmp_path / f"d{i}.fits" for i in range(5)]
    pl = xbach.Pipeline(params, workers=2, io=2)
    st, ks = pl.run_files(tps, sps, None, diffs, check=False)
    assert st == [0, 8, 2, 0, 0]  # XB_ERR_IO, XB_ERR_SIZE_MISMATCH
    assert not diffs[1].exists() and not diffs[2].exists()
    with pytest.raises(xbach.XbError) as e:
        pl.run_files(tps, sps, None, diffs)
    assert e.value.code == 8 and "missing.fits" in str(e.value)
    ref = xbach.Context(params)
    ref.run_all(T64, S64)
    assert np.array_equal(read_fits(diffs[3]),
                          ref.image(xbach.XB_IMG_DIFF, f64=False).astype(np.float64))
    assert ks[3] == ref.scalar("kernSum")
    for i, k in ((0, 0), (4, 2)):
        assert np.array_equal(read_fits(diffs[i]),
                              _single(params, pr[k][2], pr[k][3])[1].astype(np.float64)), i
    # mixed mode takes FP32 images only
    plm = xbach.Pipeline(_params("mixed", pr[0][4]), workers=1, io=1)
    st, _ = plm.run_files(tps[3:4], sps[3:4], None, diffs[3:4], check=False)
    assert st == [10]  # XB_ERR_UNSUPPORTED


def test_pipeline_many_pairs_few_slots(tmp_path):
    """More pairs than slots, one reader and one writer: slots circulate and
    every pair is written once, in the right file."""
    import xbach
    pr = _pairs(tmp_path, 3)
    params = _params("mixed", pr[0][4])
    refs = [_single(params, T, S)[1] for _, _, T, S, _ in pr]
    order = [0, 1, 2, 2, 1, 0, 0, 2, 1, 1, 0, 2, 2]
    diffs = [tmp_path / f"o{j}.fits" for j in range(len(order))]
    pl = xbach.Pipeline(params, workers=2, io=1)
    pl.set_option("graph", 1)
    st, _ = pl.run_files([pr[i][0] for i in order], [pr[i][1] for i in order], None, diffs)
    assert st == [0] * len(order)
    for j, i in enumerate(order):
        assert np.array_equal(read_fits(diffs[j]), refs[i].astype(np.float64)), j


def test_pipeline_pairs_of_two_sizes(tmp_path):
    """Frames of 512^2 and 256^2 interleaved in one run: slots grow and are
    reused across sizes, each worker keeps a graph per shape, and every file
    holds the single-context result."""
    import xbach
    from xbach.synth import make_pair
    frames = []
    for f in range(4):
        T, S, info = make_pair(1, frame=f, size=512 if f % 2 == 0 else 256)
        tp, sp = tmp_path / f"t{f}.fits", tmp_path / f"s{f}.fits"
        write_fits(tp, T)
        write_fits(sp, S)
        frames.append((tp, sp, T, S))
    params = xbach.default_params(mode=xbach.XB_MODE_MIXED, stampsx=6, stampsy=6,
                                  threshHigh=info["threshHigh"])
    refs = [_single(params, T, S)[1] for _, _, T, S in frames]
    order = [0, 1, 2, 3, 1, 0, 3, 2]
    diffs = [tmp_path / f"o{j}.fits" for j in range(len(order))]
    pl = xbach.Pipeline(params, workers=2, io=2)
    pl.set_option("graph", 1)
    for rep in range(2):
        st, _ = pl.run_files([frames[i][0] for i in order], [frames[i][1] for i in order], None,
                             diffs)
        assert st == [0] * len(order)
        for j, i in enumerate(order):
            assert np.array_equal(read_fits(diffs[j]), refs[i].astype(np.float64)), (rep, j)


def test_pipeline_per_pair_parameters(tmp_path):
    """xb_pipeline_set_params: each pair runs with its own stamp grid and
    noise model (graphs captured per parameter set); a set that changes the
    basis is refused."""
    import xbach
    pr = _pairs(tmp_path, 3)
    info = pr[0][4]
    base = _params("mixed", info)
    per = [xbach.default_params(mode=xbach.XB_MODE_MIXED, stampsx=g, stampsy=g, readNoise=rn,
                                threshHigh=info["threshHigh"])
           for g, rn in ((8, 0.0), (12, 5.0), (10, 2.0))]
    refs = [_single(p, T, S)[1] for p, (_, _, T, S, _) in zip(per, pr)]
    pl = xbach.Pipeline(base, workers=2, io=1)
    pl.set_option("graph", 1)
    pl.set_params(per)
    diffs = [tmp_path / f"pp{i}.fits" for i in range(3)]
    for _ in range(2):
        st, _ = pl.run_files([p[0] for p in pr], [p[1] for p in pr], None, diffs)
        assert st == [0, 0, 0]
        for i in range(3):
            assert np.array_equal(read_fits(diffs[i]), refs[i].astype(np.float64)), i
    bad = xbach.default_params(mode=xbach.XB_MODE_MIXED, kernelOrder=1)
    with pytest.raises(xbach.XbError):
        pl.set_params([bad])
    pl.set_params([])
    st, _ = pl.run_files([pr[0][0]], [pr[0][1]], None, diffs[:1])
    assert st == [0]
    assert np.array_equal(read_fits(diffs[0]), _single(base, pr[0][2], pr[0][3])[1].astype(np.float64))
