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
