"""Pins the CPU oracle against the reference's own golden vectors.

* tests/test01_{conv,sub}.fits: HOTPANTS outputs of the reference's test 1
  (tools/run_test.py:13), compared exactly as tools/run_test.py:34-151 does
  (max abs / max rel / NaN mismatches, after the FP32 rounding of the FITS
  writer, src/fitsUtil.cpp:47).
* tools/cond_num.py:3-298: the test01 global normal matrix, printed with six
  significant figures; it equals the first ksc matrix (CPU createMatrix,
  src/cdkscUtil.cpp:307-402).
"""
import numpy as np
import pytest

from xbach_testlib import GOLDEN, diff_fits_metrics


def f32(a):
    return np.asarray(a, np.float32).astype(np.float64)


def test_test01_conv_within_run_test_tolerance(test01_oracle, test01):
    r = test01_oracle
    assert r.status == 0
    abs_err, rel_err, nans = diff_fits_metrics(test01["conv"], f32(r.image("conv")))
    assert nans == 0
    assert abs_err < 2e-4 and rel_err < 5e-3, (abs_err, rel_err)


def test_test01_sub_within_run_test_tolerance(test01_oracle, test01):
    r = test01_oracle
    abs_err, rel_err, nans = diff_fits_metrics(test01["sub"], f32(r.image("diff")))
    assert nans == 0
    assert abs_err < 5e-4 and rel_err < 4e-3, (abs_err, rel_err)


def test_test01_direction_and_kernel_sum(test01_oracle, test01):
    r = test01_oracle
    # the science image (test0) is convolved: sub == conv - template
    assert r.scalar("convTemplate") == 0
    # HOTPANTS header of tests/test01_conv.fits: KSUM00 = '-0.1658'
    assert round(r.scalar("kernSum"), 4) == -0.1658
    interior = np.s_[10:-10, 10:-10]
    d = r.image("conv")[interior] - test01["T"][interior] - r.image("diff")[interior]
    assert np.abs(d).max() < 1e-9


def test_test01_stamp_grid(test01_oracle):
    r = test01_oracle
    # 330/10 - 21 = 12 < 31 -> 51-px stamps, 330/51 = 6 per axis (bach.cpp:51-66)
    assert r.scalar("fStampWidth") == 51
    assert r.scalar("stampsx") == 6 and r.scalar("stampsy") == 6


def test_ksc_matrix_matches_cond_num_fixture(test01_oracle):
    ref = np.load(GOLDEN / "test01_ksc_matrix.npy")
    m = test01_oracle.array("ksc_matrix0", np.float64).reshape(293, 293)
    nz = ref != 0
    assert np.array_equal(nz, m != 0)
    rel = np.abs(m - ref)[nz] / np.abs(ref[nz])
    assert rel.max() < 1e-5   # six significant figures


def test_oracle_is_thread_count_independent(oracle, test01, test01_oracle):
    r1 = oracle.run(oracle.default_params(), test01["T"], test01["S"], nthreads=1)
    for name in ("conv", "diff", "solution", "sky0", "fwhm1", "ss_val1"):
        a = r1.array(name, np.float64)
        b = test01_oracle.array(name, np.float64)
        assert np.array_equal(a.view(np.uint64), b.view(np.uint64)), name
    assert np.array_equal(r1.array("mask", np.uint16),
                          test01_oracle.array("mask", np.uint16))
