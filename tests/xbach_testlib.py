"""Shared helpers for the test-suite: FITS I/O (numpy only), ctypes
bindings of the CPU oracle and of the product's C ABI, and the
xb_params mirror.

The oracle is the checker; nothing here is imported by the product.
"""
import ctypes
import os
import pathlib

import numpy as np

REPO = pathlib.Path(__file__).resolve().parent.parent
GOLDEN = REPO / "tests" / "golden"
ORACLE_SO = REPO / "oracle" / "liboracle_xbach.so"

XB_MAX_GAUSS = 8


class XbParams(ctypes.Structure):
    """Mirror of `xb_params` in include/xbach.h."""
    _fields_ = [
        ("stampsx", ctypes.c_int),
        ("stampsy", ctypes.c_int),
        ("threshLow", ctypes.c_double),
        ("threshHigh", ctypes.c_double),
        ("threshKernFit", ctypes.c_double),
        ("sigKernFit", ctypes.c_double),
        ("sigClipAlpha", ctypes.c_double),
        ("iqRange", ctypes.c_double),
        ("maxKSStamps", ctypes.c_int),
        ("hSStampWidth", ctypes.c_int),
        ("hKernelWidth", ctypes.c_int),
        ("inSpreadMaskFactor", ctypes.c_double),
        ("normalizeTemplate", ctypes.c_int),
        ("backgroundOrder", ctypes.c_int),
        ("kernelOrder", ctypes.c_int),
        ("nGauss", ctypes.c_int),
        ("dg", ctypes.c_int * XB_MAX_GAUSS),
        ("bg", ctypes.c_float * XB_MAX_GAUSS),
        ("mode", ctypes.c_int),
        ("verbose", ctypes.c_int),
        ("gain", ctypes.c_double),
        ("readNoise", ctypes.c_double),
        ("convPerPixel", ctypes.c_int),
        ("fitWeighted", ctypes.c_int),
    ]


def read_fits(path):
    """Primary HDU of a BITPIX -32/-64 FITS file as float64 (ny, nx)."""
    raw = pathlib.Path(path).read_bytes()
    hdr, off = {}, 0
    while True:
        blk = raw[off:off + 2880]
        off += 2880
        done = False
        for i in range(36):
            card = blk[i * 80:(i + 1) * 80].decode("ascii")
            key = card[:8].strip()
            if key == "END":
                done = True
                break
            if card[8:10] == "= ":
                hdr[key] = card[10:].split("/")[0].strip()
        if done:
            break
    bitpix = int(hdr["BITPIX"])
    nx, ny = int(hdr["NAXIS1"]), int(hdr["NAXIS2"])
    dt = {-32: ">f4", -64: ">f8"}[bitpix]
    n = nx * ny * abs(bitpix) // 8
    a = np.frombuffer(raw[off:off + n], dtype=dt).reshape(ny, nx)
    return a.astype(np.float64)


def write_fits(path, a, bitpix=-32, bscale=None, bzero=None):
    """Writes a 2-D array as a primary HDU (BITPIX -32 or -64, optional
    BSCALE/BZERO cards; the samples are written as given)."""
    a = np.asarray(a)
    ny, nx = a.shape
    cards = ["SIMPLE  =                    T", "BITPIX  = %20d" % bitpix,
             "NAXIS   =                    2", "NAXIS1  = %20d" % nx, "NAXIS2  = %20d" % ny]
    if bscale is not None:
        cards.append("BSCALE  = %20r" % float(bscale))
    if bzero is not None:
        cards.append("BZERO   = %20r" % float(bzero))
    cards.append("END")
    hdr = "".join(c.ljust(80) for c in cards)
    hdr = hdr.ljust((len(hdr) + 2879) // 2880 * 2880)
    data = np.ascontiguousarray(a, dtype={-32: ">f4", -64: ">f8"}[bitpix]).tobytes()
    data += bytes((2880 - len(data) % 2880) % 2880)
    pathlib.Path(path).write_bytes(hdr.encode() + data)


class Oracle:
    """ctypes view of oracle/liboracle_xbach.so (test infrastructure)."""

    def __init__(self, path=ORACLE_SO):
        lib = ctypes.CDLL(str(path))
        lib.xbo_run.restype = ctypes.c_void_p
        lib.xbo_run.argtypes = [ctypes.POINTER(XbParams), ctypes.c_void_p,
                                ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                ctypes.c_int, ctypes.c_int,
                                ctypes.POINTER(ctypes.c_int)]
        lib.xbo_run_masked.restype = ctypes.c_void_p
        lib.xbo_run_masked.argtypes = [ctypes.POINTER(XbParams), ctypes.c_void_p,
                                       ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                       ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                       ctypes.POINTER(ctypes.c_int)]
        lib.xbo_get_array.argtypes = [ctypes.c_void_p, ctypes.c_char_p,
                                      ctypes.c_void_p, ctypes.c_size_t,
                                      ctypes.POINTER(ctypes.c_size_t)]
        lib.xbo_get_scalar.argtypes = [ctypes.c_void_p, ctypes.c_char_p,
                                       ctypes.POINTER(ctypes.c_double)]
        lib.xbo_free.argtypes = [ctypes.c_void_p]
        lib.xb_params_default.argtypes = [ctypes.POINTER(XbParams)]
        lib.xbo_sigma_clip.argtypes = [ctypes.c_void_p, ctypes.c_int,
                                       ctypes.c_int, ctypes.c_double,
                                       ctypes.POINTER(ctypes.c_double),
                                       ctypes.POINTER(ctypes.c_double)]
        lib.xbo_ran1_seq.argtypes = [ctypes.c_int, ctypes.c_int,
                                     ctypes.c_void_p]
        lib.xbo_lu_solve.argtypes = [ctypes.c_void_p, ctypes.c_int,
                                     ctypes.c_void_p]
        lib.xbo_stamp_stats.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                        ctypes.c_int, ctypes.c_void_p, ctypes.c_int,
                                        ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                        ctypes.c_void_p, ctypes.c_void_p]
        self.lib = lib

    def default_params(self, **kw):
        p = XbParams()
        self.lib.xb_params_default(ctypes.byref(p))
        for k, v in kw.items():
            if k in ("dg", "bg"):
                arr = getattr(p, k)
                for i, x in enumerate(v):
                    arr[i] = x
            else:
                setattr(p, k, v)
        return p

    def stamp_stats(self, img, mask, geom, fsw, alpha, iq_range):
        """calcStats for the stamps geom (n x {x, y, width, height}); returns
        (sky, fwhm, mask after NaN flagging)."""
        img = np.ascontiguousarray(img, dtype=np.float64)
        h, w = img.shape
        m = np.ascontiguousarray(mask, dtype=np.uint16).copy()
        g = np.ascontiguousarray(geom, dtype=np.int32)
        n = len(g)
        sky, fwhm = np.zeros(n), np.zeros(n)
        rc = self.lib.xbo_stamp_stats(img.ctypes.data, m.ctypes.data, w, h, g.ctypes.data, n,
                                      fsw, alpha, iq_range, sky.ctypes.data, fwhm.ctypes.data)
        if rc != 0:
            raise RuntimeError("xbo_stamp_stats status %d" % rc)
        return sky, fwhm, m

    def run(self, params, T, S, nthreads=0, keep_w=False, mask=None):
        """mask: optional (h, w) input mask, nonzero = excluded."""
        T = np.ascontiguousarray(T, dtype=np.float64)
        S = np.ascontiguousarray(S, dtype=np.float64)
        h, w = T.shape
        st = ctypes.c_int(-1)
        if mask is None:
            hd = self.lib.xbo_run(ctypes.byref(params), T.ctypes.data,
                                  S.ctypes.data, w, h, nthreads, int(keep_w),
                                  ctypes.byref(st))
        else:
            m = np.ascontiguousarray(np.asarray(mask) != 0, dtype=np.uint8)
            hd = self.lib.xbo_run_masked(ctypes.byref(params), T.ctypes.data,
                                         S.ctypes.data, m.ctypes.data, w, h, nthreads,
                                         int(keep_w), ctypes.byref(st))
        return OracleResult(self.lib, hd, st.value, w, h)


class OracleResult:
    def __init__(self, lib, handle, status, w, h):
        self.lib, self.h, self.status, self.w, self.hgt = lib, handle, status, w, h

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.xbo_free(self.h)
            self.h = None

    def array(self, name, dtype):
        n = ctypes.c_size_t(0)
        rc = self.lib.xbo_get_array(self.h, name.encode(), None, 0,
                                    ctypes.byref(n))
        if rc != 0:
            raise KeyError(name)
        out = np.empty(n.value // np.dtype(dtype).itemsize, dtype=dtype)
        self.lib.xbo_get_array(self.h, name.encode(), out.ctypes.data,
                               n.value, None)
        return out

    def scalar(self, name):
        v = ctypes.c_double()
        if self.lib.xbo_get_scalar(self.h, name.encode(), ctypes.byref(v)):
            raise KeyError(name)
        return v.value

    def image(self, name):
        return self.array(name, np.float64).reshape(self.hgt, self.w)


def diff_fits_metrics(golden, ours):
    """The comparison of tools/run_test.py:34-93: max |err| over non-NaN
    pixels, max relative error where the golden value is > 0, NaN
    mismatches."""
    g = np.asarray(golden, np.float64)
    b = np.asarray(ours, np.float64)
    gn, bn = np.isnan(g), np.isnan(b)
    wrong_nans = int(np.sum(gn != bn))
    ok = ~(gn | bn)
    err = np.abs(g - b)[ok]
    gv = g[ok]
    pos = gv > 0
    rel = (err[pos] / gv[pos]) if pos.any() else np.zeros(1)
    return float(err.max()), float(rel.max()), wrong_nans
