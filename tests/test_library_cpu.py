"""Host-side checks that need no GPU: the C-ABI library loads and exports
every entry point include/xbach.h declares, parameter defaults mirror
include/argsUtil.h:7-57, the FITS reader/writer round-trips, and the BACH
CLI rejects bad arguments like src/argsUtil.cpp:23-82."""
import ctypes
import pathlib
import re
import subprocess

import numpy as np
import pytest

REPO = pathlib.Path(__file__).resolve().parent.parent


@pytest.fixture(scope="module")
def xb():
    import build_native
    build_native.build_library()
    import xbach
    return xbach


def header_functions():
    txt = (REPO / "include" / "xbach.h").read_text()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(xb_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol(xb):
    L = xb.lib()
    names = header_functions()
    assert len(names) >= 25
    for n in names:
        assert hasattr(L, n), n
    assert set(names) == set(xb.EXPORTS)


def test_param_defaults_and_basis_count(xb):
    p = xb.default_params()
    assert (p.stampsx, p.stampsy, p.maxKSStamps, p.hSStampWidth, p.hKernelWidth) == (10, 10, 3, 15, 10)
    assert (p.threshLow, p.threshHigh, p.threshKernFit, p.sigKernFit) == (0.0, 25000.0, 20.0, 2.0)
    assert (p.kernelOrder, p.backgroundOrder, p.nGauss) == (2, 1, 3)
    assert list(p.dg[:3]) == [6, 4, 2]
    assert np.float32(p.bg[0]) == np.float32(1.0 / (2 * 0.7 * 0.7))
    assert xb.lib().xb_params_npsf(ctypes.byref(p)) == 49
    # four Gaussians with degrees 6/4/3/2 give 59 functions under the
    # counting rule of src/bach.cpp:181-188
    p4 = xb.default_params(nGauss=4, dg=[6, 4, 3, 2])
    assert xb.lib().xb_params_npsf(ctypes.byref(p4)) == 59


def test_fits_roundtrip(xb, tmp_path):
    from xbach_testlib import GOLDEN, read_fits
    L = xb.lib()
    d = ctypes.c_void_p()
    w, h = ctypes.c_int(), ctypes.c_int()
    assert L.xb_fits_read(str(GOLDEN / "test0.fits").encode(), ctypes.byref(d),
                          ctypes.byref(w), ctypes.byref(h)) == 0
    arr = np.ctypeslib.as_array(ctypes.cast(d, ctypes.POINTER(ctypes.c_double)),
                                shape=(h.value, w.value)).copy()
    L.xb_free(d)
    ref = read_fits(GOLDEN / "test0.fits")
    assert np.array_equal(arr, ref)
    out = tmp_path / "o.fits"
    assert L.xb_fits_write(str(out).encode(), arr.ctypes.data, w.value, h.value) == 0
    assert out.stat().st_size % 2880 == 0
    assert np.array_equal(read_fits(out), ref)


def test_fits_reads_f64_and_scaled_files(xb, tmp_path):
    """BITPIX -64 samples come back as written; BSCALE/BZERO are applied in
    FP64 (bzero + bscale * v) for either width."""
    from xbach_testlib import write_fits
    L = xb.lib()
    rng = np.random.default_rng(3)
    a = rng.normal(100.0, 30.0, (37, 53))

    def read(p):
        d = ctypes.c_void_p()
        w, h = ctypes.c_int(), ctypes.c_int()
        assert L.xb_fits_read(str(p).encode(), ctypes.byref(d), ctypes.byref(w),
                              ctypes.byref(h)) == 0
        out = np.ctypeslib.as_array(ctypes.cast(d, ctypes.POINTER(ctypes.c_double)),
                                    shape=(h.value, w.value)).copy()
        L.xb_free(d)
        return out

    write_fits(tmp_path / "d.fits", a, bitpix=-64)
    assert np.array_equal(read(tmp_path / "d.fits"), a)
    write_fits(tmp_path / "s32.fits", a, bitpix=-32, bscale=2.5, bzero=-7.0)
    assert np.array_equal(read(tmp_path / "s32.fits"), -7.0 + 2.5 * a.astype(np.float32).astype(np.float64))
    write_fits(tmp_path / "s64.fits", a, bitpix=-64, bscale=0.5, bzero=1000.0)
    assert np.array_equal(read(tmp_path / "s64.fits"), 1000.0 + 0.5 * a)


def test_fits_rejects_missing_and_integer_files(xb, tmp_path):
    L = xb.lib()
    d = ctypes.c_void_p()
    w, h = ctypes.c_int(), ctypes.c_int()
    assert L.xb_fits_read(b"/nonexistent.fits", ctypes.byref(d), ctypes.byref(w),
                          ctypes.byref(h)) == 8  # XB_ERR_IO
    hdr = "".join(c.ljust(80) for c in ["SIMPLE  =                    T",
                                        "BITPIX  =                   16",
                                        "NAXIS   =                    2",
                                        "NAXIS1  =                    4",
                                        "NAXIS2  =                    4", "END"])
    p = tmp_path / "i16.fits"
    p.write_bytes(hdr.ljust(2880).encode() + bytes(2880))
    # fitsUtil.cpp:20-24: only float and double images are supported
    assert L.xb_fits_read(str(p).encode(), ctypes.byref(d), ctypes.byref(w),
                          ctypes.byref(h)) == 10  # XB_ERR_UNSUPPORTED


def test_cli_requires_template_and_science(xb):
    import build_native
    exe = str(build_native.CLI_BIN)
    r = subprocess.run([exe, "-s", "a.fits"], capture_output=True, text=True)
    assert r.returncode == 1 and "Template file Input is required!" in r.stdout
    r = subprocess.run([exe, "-t", "a.fits"], capture_output=True, text=True)
    assert r.returncode == 1 and "Science file input is required!" in r.stdout
    r = subprocess.run([exe, "-t", "a", "-s", "b", "-sss", "xx"], capture_output=True, text=True)
    assert r.returncode == 1 and "sss mode should be mp or cl" in r.stdout


def test_context_creation_rejects_bad_params(xb):
    p = xb.default_params(hSStampWidth=0)
    h = ctypes.c_void_p()
    assert xb.lib().xb_ctx_create(ctypes.byref(p), 0, ctypes.byref(h)) == 1
    p = xb.default_params(nGauss=0)
    assert xb.lib().xb_ctx_create(ctypes.byref(p), 0, ctypes.byref(h)) == 1


def test_histogram_density_compare_is_exact():
    """The mode search of the stamp statistics compares S/D > S'/D' (FP64
    quotients of integer counts S < 2^31 and widths D <= 254) as
    S*D' > S'*D; distinct fractions of that form are more than 2^-47 apart
    relatively, so the correctly rounded quotients order the same way."""
    rng = np.random.default_rng(7)
    n = 2_000_000
    S = rng.integers(0, 2**31 - 1, n, dtype=np.int64)
    D = rng.integers(1, 255, n, dtype=np.int64)
    S2 = rng.integers(0, 2**31 - 1, n, dtype=np.int64)
    D2 = rng.integers(1, 255, n, dtype=np.int64)
    # nearby fractions too: S2/D2 close to S/D
    k = n // 2
    S2[:k] = (S[:k] * D2[:k]) // D[:k] + rng.integers(-2, 3, k)
    S2 = np.clip(S2, 0, 2**31 - 1)
    by_float = (S.astype(np.float64) / D) > (S2.astype(np.float64) / D2)
    by_int = S * D2 > S2 * D
    assert np.array_equal(by_float, by_int)
