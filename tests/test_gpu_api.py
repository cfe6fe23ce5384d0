"""The drop-in boundary on the GPU: the BACH CLI against the reference's
test-1 goldens (the check tools/run_test.py:95-151 performs), status codes
for the reference's exit paths, stage ordering, context reuse and
device-resident input."""
import pathlib
import re
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

from xbach_testlib import GOLDEN, diff_fits_metrics, read_fits


def test_cli_test01_matches_hotpants_goldens(tmp_path):
    import build_native
    out = tmp_path / "test1_"
    r = subprocess.run([str(build_native.CLI_BIN), "-ip", str(GOLDEN), "-s", "test0.fits",
                        "-t", "test1.fits", "-op", str(out), "-vt"],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    took = re.findall(r"^(\w+) took (\d+) ms$", r.stdout, flags=re.M)
    assert [t[0] for t in took] == ["Ini", "SSS", "CMV", "CD", "KSC", "Conv", "Sub", "Fin", "BACH"]
    conv = read_fits(f"{out}diff.fits")
    sub = read_fits(f"{out}sub.fits")
    a, rel, nans = diff_fits_metrics(read_fits(GOLDEN / "test01_conv.fits"), conv)
    assert nans == 0 and a < 2e-4 and rel < 5e-3, (a, rel)
    a, rel, nans = diff_fits_metrics(read_fits(GOLDEN / "test01_sub.fits"), sub)
    assert nans == 0 and a < 5e-4 and rel < 4e-3, (a, rel)


def test_size_mismatch_status():
    import xbach
    ctx = xbach.Context()
    with pytest.raises(xbach.XbError) as e:
        ctx.init(np.ones((64, 64), np.float32), np.ones((64, 65), np.float32))
    assert e.value.code == 2  # XB_ERR_SIZE_MISMATCH (bach.cpp:20-24)


def test_no_substamps_status(oracle):
    import xbach
    z = np.zeros((200, 200), np.float32)
    ref = oracle.run(oracle.default_params(), z.astype(np.float64), z.astype(np.float64))
    assert ref.status == 4
    ctx = xbach.Context()
    ctx.init(z, z)
    with pytest.raises(xbach.XbError) as e:
        ctx.sss()
    assert e.value.code == 4  # XB_ERR_NO_SUBSTAMPS (bach.cpp:166-169)


def test_stage_order_is_enforced():
    import xbach
    ctx = xbach.Context()
    with pytest.raises(xbach.XbError) as e:
        ctx.cmv()
    assert e.value.code == 6  # XB_ERR_STATE


def test_context_reuse_gives_identical_results(test01):
    import xbach
    T, S = test01["T"].astype(np.float32), test01["S"].astype(np.float32)
    ctx = xbach.Context()
    ctx.run_all(T, S)
    d1 = ctx.image(xbach.XB_IMG_DIFF)
    n1 = ctx.launches()
    ctx.run_all(T, S)
    d2 = ctx.image(xbach.XB_IMG_DIFF)
    assert np.array_equal(d1, d2)
    assert ctx.launches() == 2 * n1


def test_device_resident_input(test01):
    import torch
    import xbach
    T, S = test01["T"].astype(np.float32), test01["S"].astype(np.float32)
    ref = xbach.Context()
    ref.run_all(T, S)
    dT = torch.from_numpy(T).cuda()
    dS = torch.from_numpy(S).cuda()
    torch.cuda.synchronize()
    ctx = xbach.Context()
    ctx.init_device(dT.data_ptr(), dS.data_ptr(), T.shape[1], T.shape[0])
    ctx.sss(); ctx.cmv(); ctx.cd(); ctx.ksc(); ctx.conv(); ctx.sub()
    assert np.array_equal(ctx.image(xbach.XB_IMG_DIFF), ref.image(xbach.XB_IMG_DIFF))


def test_cli_input_mask_mask_and_noise_outputs(tmp_path):
    """-im excludes the pixels of an input-mask FITS, -om writes the output
    mask and -on writes sqrt(|target| + |conv| + 2 rn^2), the target being the
    frame that is not convolved."""
    import shutil
    import build_native
    import xbach
    BAD_CONV, INPUT_MASK, OK_CONV = 1 << 4, 1 << 5, 1 << 6  # XB_MASK_* of include/xbach.h
    BAD_INPUT, BAD_OUTPUT = 1 << 7, 1 << 12
    L = xbach.lib()
    for f in ("test0.fits", "test1.fits"):
        shutil.copy(GOLDEN / f, tmp_path / f)
    T = read_fits(GOLDEN / "test1.fits")
    S = read_fits(GOLDEN / "test0.fits")
    h, w = T.shape
    m = np.zeros((h, w))
    m[100:110, 150:170] = 1.0  # a block of pixels to exclude
    assert L.xb_fits_write(str(tmp_path / "inmask.fits").encode(), m.ctypes.data, w, h) == 0
    out = tmp_path / "o_"
    r = subprocess.run([str(build_native.CLI_BIN), "-ip", str(tmp_path), "-s", "test0.fits",
                        "-t", "test1.fits", "-op", str(out), "-im", "inmask.fits",
                        "-om", "mask.fits", "-on", "noise.fits", "-rn", "5", "-v"],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    # the convolution treats the excluded pixels as bad input (HOTPANTS'
    # input masks): they are BAD_OUTPUT and every pixel whose kernel covers
    # one is BAD_CONV or OK_CONV
    mask = read_fits(f"{out}mask.fits").astype(np.int64)
    blk = mask[100:110, 150:170]
    assert np.all((blk & (INPUT_MASK | BAD_INPUT | BAD_OUTPUT)) == INPUT_MASK | BAD_INPUT | BAD_OUTPUT)
    assert np.all(blk & (BAD_CONV | OK_CONV))
    assert not np.any(mask[m == 0] & INPUT_MASK)
    assert np.all(read_fits(f"{out}sub.fits")[100:110, 150:170] == np.float32(1e-30))
    r0 = subprocess.run([str(build_native.CLI_BIN), "-ip", str(tmp_path), "-s", "test0.fits",
                         "-t", "test1.fits", "-op", str(tmp_path / "n_"), "-om", "mask.fits"],
                        capture_output=True, text=True, timeout=300)
    assert r0.returncode == 0, r0.stdout + r0.stderr
    mask0 = read_fits(f"{tmp_path / 'n_'}mask.fits").astype(np.int64)
    assert not np.all(mask0[100:110, 150:170] & (BAD_CONV | OK_CONV))
    conv = read_fits(f"{out}diff.fits")
    noise = read_fits(f"{out}noise.fits")
    target = S if "test1.fits chosen to be convolved" in r.stdout else T
    want = np.sqrt(np.abs(target) + np.abs(conv) + 2 * 5.0 ** 2)
    assert np.allclose(noise, want, rtol=2e-6, atol=0)


@pytest.mark.parametrize("mode", ["plain", "mixed"])
def test_input_mask_excludes_pixels(test01, mode):
    """xb_set_input_mask: the pixels get INPUT_MASK | BAD_INPUT at init (before
    the bad-input dilation), no substamp is centred on them, the convolution
    leaves them BAD_OUTPUT, a mask of the wrong size is refused and clearing
    it restores the unmasked run."""
    import xbach
    INPUT_MASK, BAD_INPUT, BAD_OUTPUT = 1 << 5, 1 << 7, 1 << 12  # XB_MASK_* of include/xbach.h
    T, S = test01["T"], test01["S"]
    md = xbach.XB_MODE_PLAIN
    if mode == "mixed":
        T, S, md = T.astype(np.float32), S.astype(np.float32), xbach.XB_MODE_MIXED
    h, w = T.shape
    m = np.zeros((h, w), np.uint8)
    m[100:110, 150:170] = 1
    m[200, :] = 1  # a bad row
    ctx = xbach.Context(xbach.default_params(mode=md), trace=True)
    ctx.set_input_mask(m)
    ctx.init(T, S)
    got = ctx.mask().astype(np.int64)
    assert np.all((got[m != 0] & (INPUT_MASK | BAD_INPUT)) == INPUT_MASK | BAD_INPUT)
    assert not np.any(got[m == 0] & INPUT_MASK)
    ctx.sss()
    for si in (0, 1):
        cnt = ctx.array("ss_count_all%d" % si, np.int32)
        xy = ctx.array("ss_xy_all%d" % si, np.int32).reshape(len(cnt), -1, 2)
        for s in range(len(cnt)):
            for x, y in xy[s, :cnt[s]]:
                assert m[y, x] == 0, (si, s, x, y)
    ctx.cmv(), ctx.cd(), ctx.ksc(), ctx.conv(), ctx.sub()
    masked = ctx.image(xbach.XB_IMG_DIFF)
    got = ctx.mask().astype(np.int64)
    assert np.all((got[m != 0] & (INPUT_MASK | BAD_OUTPUT)) == INPUT_MASK | BAD_OUTPUT)
    assert np.all(masked[m != 0] == (np.float32(1e-30) if mode == "mixed" else 1e-30))
    with pytest.raises(xbach.XbError):
        ctx.set_input_mask(np.zeros((h, w + 1)))
        ctx.init(T, S)
    ctx.set_input_mask(None)
    ctx.run_all(T, S)
    ref = xbach.Context(xbach.default_params(mode=md))
    ref.run_all(T, S)
    assert np.array_equal(ctx.image(xbach.XB_IMG_DIFF), ref.image(xbach.XB_IMG_DIFF))
    assert not np.array_equal(masked, ref.image(xbach.XB_IMG_DIFF))
    if mode == "mixed":  # a frame graph with the mask replays the stage-by-stage run
        g = xbach.Context(xbach.default_params(mode=md))
        g.set_option("graph", 1)
        g.set_input_mask(m)
        for _ in range(2):
            g.run(T, S)
            assert np.array_equal(g.image(xbach.XB_IMG_DIFF, f64=False),
                                  masked.astype(np.float32))


@pytest.mark.parametrize("mode", ["plain", "mixed"])
def test_cli_pairs_stream_matches_single_runs(tmp_path, mode):
    """-pairs: each listed pair's files equal those of a single-pair run of
    the CLI (mixed mode with -graph replays frame graphs)."""
    import shutil
    import build_native
    for f in ("test0.fits", "test1.fits"):
        shutil.copy(GOLDEN / f, tmp_path / f)
    pairs = [("test1.fits", "test0.fits", "a_"), ("test0.fits", "test1.fits", "b_"),
             ("test1.fits", "test0.fits", None)]
    lines = ["# template science prefix"] + [" ".join(x for x in p if x) for p in pairs]
    (tmp_path / "list.txt").write_text("\n".join(lines) + "\n")
    out = tmp_path / "o" / ""
    out.mkdir()
    extra = ["-mode", mode] + (["-graph"] if mode == "mixed" else [])
    r = subprocess.run([str(build_native.CLI_BIN), "-pairs", str(tmp_path / "list.txt"),
                        "-ip", str(tmp_path), "-op", str(out) + "/", "-pw", "2", "-pio", "2"] + extra,
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert re.search(r"^3 of 3 pairs in ", r.stdout, flags=re.M), r.stdout
    for i, (t, s, prefix) in enumerate(pairs):
        prefix = prefix or f"{i}_"
        single = tmp_path / f"single{i}_"
        r1 = subprocess.run([str(build_native.CLI_BIN), "-ip", str(tmp_path), "-t", t, "-s", s,
                             "-op", str(single), "-mode", mode], capture_output=True, text=True,
                            timeout=300)
        assert r1.returncode == 0, r1.stdout + r1.stderr
        for name in ("diff.fits", "sub.fits"):
            assert np.array_equal(read_fits(f"{out}/{prefix}{name}"), read_fits(f"{single}{name}")), \
                (i, name)


def test_cli_pairs_reports_a_failing_pair(tmp_path):
    import shutil
    import build_native
    for f in ("test0.fits", "test1.fits"):
        shutil.copy(GOLDEN / f, tmp_path / f)
    (tmp_path / "list.txt").write_text("test1.fits test0.fits\nnothere.fits test0.fits\n")
    r = subprocess.run([str(build_native.CLI_BIN), "-pairs", str(tmp_path / "list.txt"),
                        "-ip", str(tmp_path), "-op", str(tmp_path) + "/"],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 1
    assert "pair 1 (" in r.stdout and "status 8" in r.stdout, r.stdout
    assert (tmp_path / "0_sub.fits").exists() and not (tmp_path / "1_sub.fits").exists()


def test_measured_fma_peaks_are_plausible():
    """xb_measure_fma_peaks: positive, finite, FP32 well above FP64 (the
    roofline denominators of the CUDA-core-bound kernels)."""
    import math
    import xbach
    fp32, fp64 = xbach.measure_fma_peaks(0)
    assert math.isfinite(fp32) and math.isfinite(fp64) and fp64 > 0
    assert fp32 > 4 * fp64


def test_cli_pairs_with_input_mask(tmp_path):
    """-pairs with -im: every pair of the stream excludes the masked pixels
    (their difference is the bad-output value)."""
    import shutil
    import build_native
    import xbach
    for f in ("test0.fits", "test1.fits"):
        shutil.copy(GOLDEN / f, tmp_path / f)
    T = read_fits(GOLDEN / "test1.fits")
    h, w = T.shape
    m = np.zeros((h, w))
    m[60:70, 200:230] = 1.0
    L = xbach.lib()
    assert L.xb_fits_write(str(tmp_path / "inmask.fits").encode(), m.ctypes.data, w, h) == 0
    (tmp_path / "list.txt").write_text("test1.fits test0.fits p_\ntest0.fits test1.fits q_\n")
    r = subprocess.run([str(build_native.CLI_BIN), "-pairs", str(tmp_path / "list.txt"),
                        "-ip", str(tmp_path), "-op", str(tmp_path) + "/", "-im", "inmask.fits",
                        "-pw", "2", "-pio", "1"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    for prefix in ("p_", "q_"):
        sub = read_fits(tmp_path / f"{prefix}sub.fits")
        assert np.all(sub[60:70, 200:230] == np.float32(1e-30)), prefix
        assert np.mean(sub == np.float32(1e-30)) < 0.5


def test_device_images_hold_the_results(test01):
    """xb_get_device_images: the device conv and diff images are the ones
    xb_get_image copies out (read back here through the CUDA runtime)."""
    import ctypes
    import ctypes.util
    import xbach
    T, S = test01["T"].astype(np.float32), test01["S"].astype(np.float32)
    ctx = xbach.Context(xbach.default_params(mode=xbach.XB_MODE_MIXED))
    ctx.run_all(T, S)
    names = [ctypes.util.find_library("cudart"), "libcudart.so", "/usr/local/cuda/lib64/libcudart.so"]
    rt = None
    for n in names:
        try:
            rt = ctypes.CDLL(n) if n else None
        except OSError:
            rt = None
        if rt is not None:
            break
    if rt is None:
        pytest.skip("no CUDA runtime library to read device memory with")
    rt.cudaMemcpy.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int]
    for ptr, which in zip(ctx.device_images(), (xbach.XB_IMG_CONV, xbach.XB_IMG_DIFF)):
        out = np.empty(T.shape, np.float32)
        assert rt.cudaMemcpy(out.ctypes.data, ptr, out.nbytes, 2) == 0  # device to host
        assert np.array_equal(out, ctx.image(which, f64=False)), which


def test_cli_extension_flags_reach_the_fit(tmp_path):
    """-gain, -rn, -wfit and -pk: the CLI's images equal those of the API with
    gain, readNoise, fitWeighted and convPerPixel set."""
    import build_native
    import xbach
    out = tmp_path / "x_"
    r = subprocess.run([str(build_native.CLI_BIN), "-ip", str(GOLDEN), "-s", "test0.fits",
                        "-t", "test1.fits", "-op", str(out), "-gain", "2.0", "-rn", "4.0",
                        "-wfit", "-pk"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    T, S = read_fits(GOLDEN / "test1.fits"), read_fits(GOLDEN / "test0.fits")
    ctx = xbach.Context(xbach.default_params(gain=2.0, readNoise=4.0, fitWeighted=1,
                                             convPerPixel=1))
    ctx.run_all(T, S)
    assert np.array_equal(read_fits(f"{out}sub.fits"),
                          ctx.image(xbach.XB_IMG_DIFF, f64=False).astype(np.float64))
    assert np.array_equal(read_fits(f"{out}diff.fits"),
                          ctx.image(xbach.XB_IMG_CONV, f64=False).astype(np.float64))
    plain = xbach.Context(xbach.default_params())
    plain.run_all(T, S)
    assert not np.array_equal(read_fits(f"{out}sub.fits"),
                              plain.image(xbach.XB_IMG_DIFF, f64=False).astype(np.float64))
