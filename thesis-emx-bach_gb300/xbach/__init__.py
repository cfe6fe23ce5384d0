"""ctypes binding of libxbach_gb300.so, the C ABI of include/xbach.h.

The stage methods mirror X-BACH's stage API (include/bach.h:66-87): init,
sss, cmv, cd, ksc, conv, sub.  There is no CPU fallback: loading fails
loudly when the native library is missing.
"""
import ctypes
import pathlib

import numpy as np

PKG = pathlib.Path(__file__).resolve().parent.parent
LIB_PATH = PKG / "lib" / "libxbach_gb300.so"

XB_MAX_GAUSS = 8
XB_MODE_PLAIN = 0
XB_MODE_MIXED = 1
XB_IMG_CONV = 0
XB_IMG_DIFF = 1

STATUS = {
    0: "XB_OK", 1: "XB_ERR_ARG", 2: "XB_ERR_SIZE_MISMATCH",
    3: "XB_ERR_STAMP_TOO_SMALL", 4: "XB_ERR_NO_SUBSTAMPS", 5: "XB_ERR_CUDA",
    6: "XB_ERR_STATE", 7: "XB_ERR_NOMEM", 8: "XB_ERR_IO", 9: "XB_ERR_SINGULAR",
    10: "XB_ERR_UNSUPPORTED", 11: "XB_ERR_DEVICE_TIMEOUT",
}


class XbParams(ctypes.Structure):
    """Mirror of `xb_params` (include/xbach.h)."""
    _fields_ = [
        ("stampsx", ctypes.c_int), ("stampsy", ctypes.c_int),
        ("threshLow", ctypes.c_double), ("threshHigh", ctypes.c_double),
        ("threshKernFit", ctypes.c_double), ("sigKernFit", ctypes.c_double),
        ("sigClipAlpha", ctypes.c_double), ("iqRange", ctypes.c_double),
        ("maxKSStamps", ctypes.c_int), ("hSStampWidth", ctypes.c_int),
        ("hKernelWidth", ctypes.c_int), ("inSpreadMaskFactor", ctypes.c_double),
        ("normalizeTemplate", ctypes.c_int), ("backgroundOrder", ctypes.c_int),
        ("kernelOrder", ctypes.c_int), ("nGauss", ctypes.c_int),
        ("dg", ctypes.c_int * XB_MAX_GAUSS), ("bg", ctypes.c_float * XB_MAX_GAUSS),
        ("mode", ctypes.c_int), ("verbose", ctypes.c_int),
        ("gain", ctypes.c_double), ("readNoise", ctypes.c_double), ("convPerPixel", ctypes.c_int),
        ("fitWeighted", ctypes.c_int),
    ]


class XbError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{STATUS.get(code, code)}: {msg}")
        self.code = code


_lib = None

EXPORTS = [
    "xb_params_default", "xb_params_npsf", "xb_ctx_create", "xb_ctx_destroy",
    "xb_last_error", "xb_ctx_set_params", "xb_set_option", "xb_set_input_mask", "xb_init", "xb_init_f32",
    "xb_init_device_f32", "xb_sss", "xb_cmv", "xb_cd", "xb_ksc", "xb_conv",
    "xb_sub", "xb_run", "xb_run_device", "xb_get_image", "xb_get_image_f64", "xb_get_mask",
    "xb_get_device_images", "xb_get_solution", "xb_get_array",
    "xb_get_scalar", "xb_kernel_launches", "xb_get_stream", "xb_fits_read",
    "xb_fits_write", "xb_free", "xb_stamp_stats_noalloc", "xb_batch_create",
    "xb_batch_destroy", "xb_batch_last_error", "xb_batch_run", "xb_batch_run_device",
    "xb_batch_worker", "xb_batch_set_stream", "xb_batch_set_params", "xb_ranker_param_count", "xb_ranker_set",
    "xb_ranker_features", "xb_ranker_forward", "xb_ranker_grad", "xb_ranker_adam",
    "xb_pipeline_create", "xb_pipeline_destroy", "xb_pipeline_last_error", "xb_pipeline_worker",
    "xb_pipeline_run_files", "xb_pipeline_stats_get", "xb_pipeline_set_params",
    "xb_measure_fma_peaks", "xb_ordered_sum_host", "xb_ordered_sum_device",
    "xb_ordered_sum_device_f32",
]


class PipelineStats(ctypes.Structure):
    """xb_pipeline_stats of include/xbach.h."""
    _fields_ = [("wall_ms", ctypes.c_double), ("read_ms", ctypes.c_double),
                ("compute_ms", ctypes.c_double), ("write_ms", ctypes.c_double),
                ("bytes_read", ctypes.c_double), ("bytes_written", ctypes.c_double),
                ("pairs", ctypes.c_int)]


def lib():
    """Loads the native library once (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise RuntimeError(f"native library missing: {LIB_PATH} (run build())")
    L = ctypes.CDLL(str(LIB_PATH))
    P = ctypes.POINTER
    vp, i, d = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
    L.xb_params_default.argtypes = [P(XbParams)]
    L.xb_params_npsf.argtypes = [P(XbParams)]
    L.xb_ctx_create.argtypes = [P(XbParams), i, P(vp)]
    L.xb_ctx_destroy.argtypes = [vp]
    L.xb_last_error.argtypes = [vp]
    L.xb_last_error.restype = ctypes.c_char_p
    L.xb_set_option.argtypes = [vp, ctypes.c_char_p, ctypes.c_longlong]
    L.xb_init.argtypes = [vp, vp, i, i, vp, i, i]
    L.xb_init_f32.argtypes = [vp, vp, i, i, vp, i, i]
    L.xb_init_device_f32.argtypes = [vp, vp, vp, i, i]
    for f in ("xb_sss", "xb_cmv", "xb_ksc", "xb_sub"):
        getattr(L, f).argtypes = [vp]
    L.xb_cd.argtypes = [vp, P(i)]
    L.xb_conv.argtypes = [vp, P(d)]
    L.xb_run.argtypes = [vp, vp, vp, i, i, vp, vp]
    L.xb_run_device.argtypes = [vp, vp, vp, i, i, vp, vp]
    L.xb_get_image.argtypes = [vp, i, vp]
    L.xb_get_image_f64.argtypes = [vp, i, vp]
    L.xb_get_mask.argtypes = [vp, vp]
    L.xb_get_device_images.argtypes = [vp, P(vp), P(vp)]
    L.xb_get_solution.argtypes = [vp, vp, i, P(i)]
    L.xb_get_array.argtypes = [vp, ctypes.c_char_p, vp, ctypes.c_size_t,
                               P(ctypes.c_size_t)]
    L.xb_get_scalar.argtypes = [vp, ctypes.c_char_p, P(d)]
    L.xb_kernel_launches.argtypes = [vp]
    L.xb_kernel_launches.restype = ctypes.c_longlong
    L.xb_get_stream.argtypes = [vp, P(vp)]
    L.xb_fits_read.argtypes = [ctypes.c_char_p, P(vp), P(i), P(i)]
    L.xb_fits_write.argtypes = [ctypes.c_char_p, vp, i, i]
    L.xb_free.argtypes = [vp]
    L.xb_batch_create.argtypes = [P(XbParams), i, i, P(vp)]
    L.xb_batch_destroy.argtypes = [vp]
    L.xb_batch_last_error.argtypes = [vp]
    L.xb_batch_last_error.restype = ctypes.c_char_p
    L.xb_batch_run.argtypes = [vp, i, P(vp), P(vp), P(i), P(i), P(vp), P(vp), P(i), P(d)]
    L.xb_batch_run_device.argtypes = [vp, i, P(vp), P(vp), P(i), P(i), P(vp), P(vp), P(i),
                                      P(d)]
    L.xb_batch_worker.argtypes = [vp, i, P(vp)]
    L.xb_batch_set_stream.argtypes = [vp, vp]
    L.xb_batch_set_params.argtypes = [vp, i, vp]
    L.xb_ctx_set_params.argtypes = [vp, vp]
    L.xb_set_input_mask.argtypes = [vp, vp, i, i]
    L.xb_ranker_param_count.argtypes = []
    L.xb_ranker_set.argtypes = [vp, vp, i]
    L.xb_ranker_features.argtypes = [vp, i, vp, vp, vp, vp, i, P(i)]
    L.xb_ranker_forward.argtypes = [vp, vp, vp, i, vp, vp]
    L.xb_ranker_grad.argtypes = [vp, vp, vp, vp, vp, i, vp, vp, vp, vp]
    L.xb_ranker_adam.argtypes = [vp, vp, vp, vp, i, ctypes.c_float, vp]
    L.xb_pipeline_create.argtypes = [P(XbParams), i, i, i, P(vp)]
    L.xb_pipeline_destroy.argtypes = [vp]
    L.xb_pipeline_last_error.argtypes = [vp]
    L.xb_pipeline_last_error.restype = ctypes.c_char_p
    L.xb_pipeline_worker.argtypes = [vp, i, P(vp)]
    L.xb_pipeline_run_files.argtypes = [vp, i, P(ctypes.c_char_p), P(ctypes.c_char_p),
                                        P(ctypes.c_char_p), P(ctypes.c_char_p), P(i), P(d)]
    L.xb_pipeline_stats_get.argtypes = [vp, P(PipelineStats)]
    L.xb_pipeline_set_params.argtypes = [vp, i, vp]
    L.xb_measure_fma_peaks.argtypes = [i, P(d), P(d)]
    L.xb_ordered_sum_host.argtypes = [vp, i]
    L.xb_ordered_sum_host.restype = d
    L.xb_ordered_sum_device.argtypes = [vp, i, vp, vp]
    L.xb_ordered_sum_device_f32.argtypes = [vp, i, vp, vp]
    _lib = L
    return L


def default_params(**kw):
    p = XbParams()
    lib().xb_params_default(ctypes.byref(p))
    for k, v in kw.items():
        if k in ("dg", "bg"):
            arr = getattr(p, k)
            for j, x in enumerate(v):
                arr[j] = x
        else:
            setattr(p, k, v)
    return p


class Context:
    """One frame pair on one GPU (an `xb_ctx`)."""

    def __init__(self, params=None, device=0, trace=False):
        self.L = lib()
        self.params = params if params is not None else default_params()
        h = ctypes.c_void_p()
        rc = self.L.xb_ctx_create(ctypes.byref(self.params), device, ctypes.byref(h))
        if rc != 0:
            raise XbError(rc, "xb_ctx_create failed")
        self.h = h
        if trace:
            self._check(self.L.xb_set_option(self.h, b"trace", 1))

    def close(self):
        if getattr(self, "h", None):
            self.L.xb_ctx_destroy(self.h)
            self.h = None

    __del__ = close

    def _check(self, rc):
        if rc != 0:
            raise XbError(rc, self.L.xb_last_error(self.h).decode())
        return rc

    # ---- stage API ----
    def init(self, T, S):
        T = np.ascontiguousarray(T)
        S = np.ascontiguousarray(S)
        h, w = T.shape
        sh, sw = S.shape
        if T.dtype == np.float32 and S.dtype == np.float32:
            return self._check(self.L.xb_init_f32(self.h, T.ctypes.data, w, h,
                                                  S.ctypes.data, sw, sh))
        T = T.astype(np.float64)
        S = S.astype(np.float64)
        return self._check(self.L.xb_init(self.h, T.ctypes.data, w, h,
                                          S.ctypes.data, sw, sh))

    def init_device(self, dT, dS, w, h):
        """dT/dS: device pointers (ints) of FP32 images kept alive by the caller."""
        return self._check(self.L.xb_init_device_f32(self.h, ctypes.c_void_p(dT),
                                                     ctypes.c_void_p(dS), w, h))

    def sss(self):
        return self._check(self.L.xb_sss(self.h))

    def cmv(self):
        return self._check(self.L.xb_cmv(self.h))

    def cd(self):
        ct = ctypes.c_int(-1)
        self._check(self.L.xb_cd(self.h, ctypes.byref(ct)))
        return ct.value

    def ksc(self):
        return self._check(self.L.xb_ksc(self.h))

    def conv(self):
        ks = ctypes.c_double()
        self._check(self.L.xb_conv(self.h, ctypes.byref(ks)))
        return ks.value

    def sub(self):
        return self._check(self.L.xb_sub(self.h))

    def run(self, T, S):
        """init..sub through xb_run (FP32 (h, w) arrays; the frame-graph path
        when option "graph" is on); results via image()."""
        T = np.ascontiguousarray(T, dtype=np.float32)
        S = np.ascontiguousarray(S, dtype=np.float32)
        if T.shape != S.shape:
            raise ValueError("template and science differ in shape")
        h, w = T.shape
        return self._check(self.L.xb_run(self.h, T.ctypes.data, S.ctypes.data, w, h, None, None))

    def run_device(self, dT, dS, w, h, dConv=None, dDiff=None):
        """init..sub from device FP32 images (pointers as ints) into optional
        device outputs, through xb_run_device."""
        vp = ctypes.c_void_p
        return self._check(self.L.xb_run_device(self.h, vp(dT), vp(dS), w, h,
                                                vp(dConv) if dConv else None,
                                                vp(dDiff) if dDiff else None))

    def run_all(self, T, S):
        self.init(T, S)
        self.sss()
        self.cmv()
        self.cd()
        self.ksc()
        self.conv()
        self.sub()

    # ---- results ----
    def image(self, which, f64=True):
        n = self.w * self.hgt
        out = np.empty(n, np.float64 if f64 else np.float32)
        fn = self.L.xb_get_image_f64 if f64 else self.L.xb_get_image
        self._check(fn(self.h, which, out.ctypes.data))
        return out.reshape(self.hgt, self.w)

    def device_images(self):
        """(conv, diff) device pointers (ints) of the FP32 result images,
        valid until the next init or destroy."""
        c, d = ctypes.c_void_p(), ctypes.c_void_p()
        self._check(self.L.xb_get_device_images(self.h, ctypes.byref(c), ctypes.byref(d)))
        return c.value, d.value

    def mask(self):
        out = np.empty(self.w * self.hgt, np.uint16)
        self._check(self.L.xb_get_mask(self.h, out.ctypes.data))
        return out.reshape(self.hgt, self.w)

    def solution(self):
        n = ctypes.c_int()
        self._check(self.L.xb_get_solution(self.h, None, 0, ctypes.byref(n)))
        out = np.empty(n.value, np.float64)
        self._check(self.L.xb_get_solution(self.h, out.ctypes.data, n.value, None))
        return out

    def array(self, name, dtype):
        n = ctypes.c_size_t()
        if self.L.xb_get_array(self.h, name.encode(), None, 0, ctypes.byref(n)):
            raise KeyError(name)
        out = np.empty(n.value // np.dtype(dtype).itemsize, dtype)
        self.L.xb_get_array(self.h, name.encode(), out.ctypes.data, n.value, None)
        return out

    def scalar(self, name):
        v = ctypes.c_double()
        if self.L.xb_get_scalar(self.h, name.encode(), ctypes.byref(v)):
            raise KeyError(name)
        return v.value

    def launches(self):
        return self.L.xb_kernel_launches(self.h)

    def stream(self):
        """The context's cudaStream_t as an integer handle."""
        s = ctypes.c_void_p()
        self._check(self.L.xb_get_stream(self.h, ctypes.byref(s)))
        return s.value or 0

    def set_option(self, name, value):
        return self._check(self.L.xb_set_option(self.h, name.encode(), int(value)))

    def set_input_mask(self, mask):
        """Pixels to exclude from the following frames ((h, w), nonzero = bad;
        None clears): they get INPUT_MASK | BAD_INPUT at init."""
        if mask is None:
            return self._check(self.L.xb_set_input_mask(self.h, None, 0, 0))
        m = np.ascontiguousarray(mask != 0, dtype=np.uint8)
        self._keep_mask = m
        h, w = m.shape
        return self._check(self.L.xb_set_input_mask(self.h, m.ctypes.data, w, h))

    def set_params(self, params):
        """Other parameters with the same basis, widths, orders and mode."""
        self._check(self.L.xb_ctx_set_params(self.h, ctypes.byref(params)))
        self.params = params

    def kernel_time(self, name):
        """(total ms, launches) of a timed kernel (option time_kernels)."""
        try:
            return self.scalar(f"kt:{name}:ms"), int(self.scalar(f"kt:{name}:n"))
        except KeyError:
            return 0.0, 0

    @property
    def w(self):
        return int(self.scalar("w"))

    @property
    def hgt(self):
        return int(self.scalar("h"))


class _Borrowed(Context):
    """A worker context owned by a Batch (not destroyed here)."""

    def __init__(self, handle, params):
        self.L = lib()
        self.params = params
        self.h = handle

    def close(self):
        self.h = None

    __del__ = close


class Batch:
    """Independent frame pairs run concurrently by `workers` contexts, each
    on its own stream and host thread (an `xb_batch`)."""

    def __init__(self, params=None, device=0, workers=8):
        self.L = lib()
        self.params = params if params is not None else default_params()
        h = ctypes.c_void_p()
        rc = self.L.xb_batch_create(ctypes.byref(self.params), device, workers, ctypes.byref(h))
        if rc != 0:
            raise XbError(rc, "xb_batch_create failed")
        self.h = h
        self.n_workers = workers

    def close(self):
        if getattr(self, "h", None):
            self.L.xb_batch_destroy(self.h)
            self.h = None

    __del__ = close

    def set_stream(self, stream):
        """Join a cudaStream_t handle (int) to later runs (0 detaches)."""
        if self.L.xb_batch_set_stream(self.h, ctypes.c_void_p(stream or None)):
            raise XbError(5, "xb_batch_set_stream failed")

    def set_params(self, params_list):
        """Parameters per frame for later runs (a list of xb_params; [] or
        None returns to the batch's own)."""
        params_list = list(params_list or [])
        arr = (XbParams * max(len(params_list), 1))(*params_list)
        rc = self.L.xb_batch_set_params(self.h, len(params_list), arr)
        if rc:
            raise XbError(rc, self.L.xb_batch_last_error(self.h).decode())
        self._keep_params = arr

    def set_option(self, name, value):
        """xb_set_option on every worker context (e.g. "graph")."""
        for i in range(self.n_workers):
            self.worker(i).set_option(name, value)

    def worker(self, i):
        c = ctypes.c_void_p()
        if self.L.xb_batch_worker(self.h, i, ctypes.byref(c)):
            raise IndexError(i)
        return _Borrowed(c, self.params)

    @staticmethod
    def _ptrs(vals):
        return (ctypes.c_void_p * max(len(vals), 1))(*[ctypes.c_void_p(v) for v in vals])

    def _finish(self, rc, n, st, ks):
        if rc != 0:
            raise XbError(rc, self.L.xb_batch_last_error(self.h).decode())
        return [int(st[i]) for i in range(n)], [float(ks[i]) for i in range(n)]

    def run(self, Ts, Ss, convs=None, diffs=None):
        """Host frames: lists of FP32 numpy arrays (outputs: preallocated FP32
        arrays or None).  Returns (statuses, kernel sums)."""
        n = len(Ts)
        Ts = [np.ascontiguousarray(t, dtype=np.float32) for t in Ts]
        Ss = [np.ascontiguousarray(s, dtype=np.float32) for s in Ss]
        w = (ctypes.c_int * max(n, 1))(*[t.shape[1] for t in Ts])
        h = (ctypes.c_int * max(n, 1))(*[t.shape[0] for t in Ts])
        cv = self._ptrs([c.ctypes.data for c in convs]) if convs is not None else None
        df = self._ptrs([d.ctypes.data for d in diffs]) if diffs is not None else None
        st = (ctypes.c_int * max(n, 1))()
        ks = (ctypes.c_double * max(n, 1))()
        rc = self.L.xb_batch_run(self.h, n, self._ptrs([t.ctypes.data for t in Ts]),
                                 self._ptrs([s.ctypes.data for s in Ss]), w, h, cv, df, st, ks)
        return self._finish(rc, n, st, ks)

    def run_ptrs(self, T_ptrs, S_ptrs, ws, hs, conv_ptrs=None, diff_ptrs=None, device=False):
        """Frames given as raw pointers (host or, with device=True, device)."""
        n = len(T_ptrs)
        w = (ctypes.c_int * max(n, 1))(*ws)
        h = (ctypes.c_int * max(n, 1))(*hs)
        cv = self._ptrs(conv_ptrs) if conv_ptrs is not None else None
        df = self._ptrs(diff_ptrs) if diff_ptrs is not None else None
        st = (ctypes.c_int * max(n, 1))()
        ks = (ctypes.c_double * max(n, 1))()
        f = self.L.xb_batch_run_device if device else self.L.xb_batch_run
        rc = f(self.h, n, self._ptrs(T_ptrs), self._ptrs(S_ptrs), w, h, cv, df, st, ks)
        return self._finish(rc, n, st, ks)


class Pipeline:
    """Streaming difference imaging over FITS files (an `xb_pipeline`):
    `io` reader threads decode pairs into pinned slots, `workers` contexts run
    them, `io` writer threads encode the outputs."""

    def __init__(self, params=None, device=0, workers=8, io=4):
        self.L = lib()
        self.params = params if params is not None else default_params()
        h = ctypes.c_void_p()
        rc = self.L.xb_pipeline_create(ctypes.byref(self.params), device, workers, io,
                                       ctypes.byref(h))
        if rc != 0:
            raise XbError(rc, "xb_pipeline_create failed")
        self.h = h
        self.n_workers = workers

    def close(self):
        if getattr(self, "h", None):
            self.L.xb_pipeline_destroy(self.h)
            self.h = None

    __del__ = close

    def worker(self, i):
        c = ctypes.c_void_p()
        if self.L.xb_pipeline_worker(self.h, i, ctypes.byref(c)):
            raise IndexError(i)
        return _Borrowed(c, self.params)

    def set_option(self, name, value):
        """xb_set_option on every worker context (e.g. "graph", "rank")."""
        for i in range(self.n_workers):
            self.worker(i).set_option(name, value)

    @staticmethod
    def _paths(vals):
        if vals is None:
            return None
        return (ctypes.c_char_p * max(len(vals), 1))(
            *[None if v is None else str(v).encode() for v in vals])

    def run_files(self, templates, sciences, convs=None, diffs=None, check=True):
        """Pair i: templates[i], sciences[i] in; convs[i], diffs[i] out (None
        skips).  Returns (statuses, kernel sums); raises on the first failing
        pair when `check`."""
        n = len(templates)
        st = (ctypes.c_int * max(n, 1))()
        ks = (ctypes.c_double * max(n, 1))()
        rc = self.L.xb_pipeline_run_files(self.h, n, self._paths(templates), self._paths(sciences),
                                          self._paths(convs), self._paths(diffs), st, ks)
        if rc != 0 and check:
            raise XbError(rc, self.L.xb_pipeline_last_error(self.h).decode())
        return [int(st[i]) for i in range(n)], [float(ks[i]) for i in range(n)]

    def set_params(self, params_list):
        """Parameters per pair for later runs (a list of xb_params; [] or None
        returns to the pipeline's own)."""
        params_list = list(params_list or [])
        arr = (XbParams * max(len(params_list), 1))(*params_list)
        rc = self.L.xb_pipeline_set_params(self.h, len(params_list), arr)
        if rc:
            raise XbError(rc, self.L.xb_pipeline_last_error(self.h).decode())
        self._keep_params = arr

    def stats(self):
        out = PipelineStats()
        if self.L.xb_pipeline_stats_get(self.h, ctypes.byref(out)):
            raise XbError(5, "xb_pipeline_stats_get failed")
        return {k: getattr(out, k) for k, _ in PipelineStats._fields_}


def ordered_sum_host(c):
    """xb_ordered_sum_host: the left-to-right FP64 sum of c by the warp
    algorithm's steps, on the CPU."""
    import numpy as np
    c = np.ascontiguousarray(c, dtype=np.float64)
    return lib().xb_ordered_sum_host(c.ctypes.data, len(c))


def measure_fma_peaks(device=0):
    """(FP32, FP64) CUDA-core FMA throughput of the device, TFLOP/s."""
    a, b = ctypes.c_double(), ctypes.c_double()
    rc = lib().xb_measure_fma_peaks(device, ctypes.byref(a), ctypes.byref(b))
    if rc:
        raise XbError(rc, "xb_measure_fma_peaks failed")
    return a.value, b.value
