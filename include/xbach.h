/*
 * xbach.h — C ABI of the GB300-native X-BACH difference-imaging path.
 *
 * This header is the drop-in boundary for X-BACH's stage API
 * (include/bach.h:66-87 of D0V4HKIIN/Thesis-EMX-BACH): init, sss, cmv, cd,
 * ksc, conv, sub, fin.  The reference passes a `ClData&` (OpenCL context,
 * queue and cl::Buffer members, include/bach.h:25-64) plus a mutable
 * `Arguments&` (include/argsUtil.h:7-57) from stage to stage; here an opaque
 * `xb_ctx` owns the CUDA stream and every device buffer, and `xb_params`
 * carries the Arguments fields that define the arithmetic.
 *
 * Conventions
 *   - Every entry point returns an `int` status: XB_OK (0) or one of the
 *     XB_ERR_* codes below.  Each reference `std::exit(1)` / sentinel path
 *     has its own code (see the list).
 *   - The caller owns host arrays; the context owns device memory.
 *   - A context is not thread-safe; it issues all work on one CUDA stream.
 *   - Image layout is row-major, x fastest: pixel (x, y) at index x + y*w,
 *     the same layout as the FITS primary HDU read by the reference
 *     (src/fitsUtil.cpp:8-37).
 */
#ifndef XBACH_H
#define XBACH_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define XB_OK 0
#define XB_ERR_ARG 1             /* bad argument / parameter                    */
#define XB_ERR_SIZE_MISMATCH 2   /* template/science differ: src/bach.cpp:20-24 */
#define XB_ERR_STAMP_TOO_SMALL 3 /* stamp < 100 px: src/bachUtil.cpp:151-154    */
#define XB_ERR_NO_SUBSTAMPS 4    /* no substamps at all: src/bach.cpp:166-169   */
#define XB_ERR_CUDA 5            /* CUDA runtime error                          */
#define XB_ERR_STATE 6           /* stage called out of order                   */
#define XB_ERR_NOMEM 7           /* device allocation failed                    */
#define XB_ERR_IO 8              /* FITS read/write failure                     */
#define XB_ERR_SINGULAR 9        /* global LU saw an all-zero row; the
                                    reference returns 1 and ignores it
                                    (src/bachUtil.cpp:334-338); reported as a
                                    warning flag, never as a failing status    */
#define XB_ERR_UNSUPPORTED 10    /* parameter outside this build's limits       */
#define XB_ERR_DEVICE_TIMEOUT 11 /* a bounded device-side wait ran out          */

/* ---- mask bits (include/datatypeUtil.h:172-188, cl_kern/ini.cl:1-13) ---- */
#define XB_MASK_BAD_PIX_VAL (1u << 0)
#define XB_MASK_SAT_PIXEL (1u << 1)
#define XB_MASK_LOW_PIXEL (1u << 2)
#define XB_MASK_NAN_PIXEL (1u << 3)
#define XB_MASK_BAD_CONV (1u << 4)
#define XB_MASK_INPUT_MASK (1u << 5)
#define XB_MASK_OK_CONV (1u << 6)
#define XB_MASK_BAD_INPUT (1u << 7)
#define XB_MASK_BAD_PIXEL_T (1u << 8)
#define XB_MASK_SKIP_T (1u << 9)
#define XB_MASK_BAD_PIXEL_S (1u << 10)
#define XB_MASK_SKIP_S (1u << 11)
#define XB_MASK_BAD_OUTPUT (1u << 12)
#define XB_MASK_ALL ((1u << 13) - 1u)

/* ---- precision modes --------------------------------------------------- */
/* XB_MODE_PLAIN: the reference's precision choices (FP64 statistics, FP32
 * Y-pass accumulation, FP64 W/Q/B, FP64 solves, FP64 convolution).  Every
 * quantity that feeds a stamp / substamp / rejection decision is computed in
 * the reference's operation order, so the decision sets are bit-identical to
 * the CPU oracle.
 * XB_MODE_MIXED: FP32 basis convolutions and W; per-stamp Gram matrices on the
 * tensor cores from exact fixed-point BF16 slices of W (FP64-accurate); the
 * global system by FP64 LDL^T (pivoted LU if a pivot fails) plus one FP64
 * iterative-refinement step; FP32 full-frame convolution.  Decision sets
 * match the plain mode; the difference image stays within 1e-3 of the
 * per-pixel noise of the plain result on the synthetic workloads. */
#define XB_MODE_PLAIN 0
#define XB_MODE_MIXED 1

#define XB_MAX_GAUSS 8

/* Fields and defaults of include/argsUtil.h:7-57.  Defaults are produced by
 * xb_params_default(). */
typedef struct xb_params {
  int stampsx;              /* -sx, default 10 */
  int stampsy;              /* -sy, default 10 */
  double threshLow;         /* 0.0 */
  double threshHigh;        /* 25000.0 */
  double threshKernFit;     /* 20.0 */
  double sigKernFit;        /* 2.0 */
  double sigClipAlpha;      /* 3.0 */
  double iqRange;           /* 1.35 */
  int maxKSStamps;          /* 3 */
  int hSStampWidth;         /* 15 (substamp is 2*15+1 = 31 px) */
  int hKernelWidth;         /* 10 (kernel is 2*10+1 = 21 px) */
  double inSpreadMaskFactor;/* 1.0 */
  int normalizeTemplate;    /* 1 */
  int backgroundOrder;      /* 1 */
  int kernelOrder;          /* 2 */
  int nGauss;               /* 3 */
  int dg[XB_MAX_GAUSS];     /* {6, 4, 2} polynomial degree per Gaussian */
  float bg[XB_MAX_GAUSS];   /* 1/(2 sigma^2) stored as float, sigma 0.7/1.5/3.0 */
  int mode;                 /* XB_MODE_PLAIN or XB_MODE_MIXED */
  int verbose;              /* -v */
  /* HOTPANTS-style extensions; the xb_params_default values (all zero) keep
   * the reference's behaviour exactly. */
  double gain;              /* e-/ADU of the noise model of the stamp chi^2:
                             * sigma^2 = (|convolved frame| + |target|) / gain
                             * + 2 readNoise^2 (cd.cl:578 is gain 1, no read
                             * noise); <= 0 means 1 */
  double readNoise;         /* ADU per frame in that model (0) */
  int convPerPixel;         /* 1: the spatially varying kernel is evaluated at
                             * every output pixel instead of once per
                             * fK x fK block (conv.cl, bach.cpp:339-350) */
  int fitWeighted;          /* 1: every substamp pixel enters the normal
                             * equations (Q, B and the background products)
                             * with weight 1 / sigma^2 of the noise model
                             * above; the reference's fit is unweighted */
} xb_params;

/* Fill `p` with the reference defaults (include/argsUtil.h:7-57). */
void xb_params_default(xb_params* p);

/* Number of basis functions implied by nGauss/dg: sum (d+1)(d+2)/2, the
 * counting rule of src/bach.cpp:181-188 (49 for the defaults). */
int xb_params_npsf(const xb_params* p);

/* ---- context ------------------------------------------------------------ */
typedef struct xb_ctx xb_ctx;

/* Replaces main()'s OpenCL set-up (src/main.cpp:41-54): picks CUDA device
 * `device` and creates the context's stream. */
int xb_ctx_create(const xb_params* p, int device, xb_ctx** out);
int xb_ctx_destroy(xb_ctx* ctx);
/* Human-readable message for the last failing call on this context. */
const char* xb_last_error(const xb_ctx* ctx);
/* Switches a context to other parameters that keep its basis, widths,
 * orders and mode (stamp grid, thresholds, clipping may change; XB_ERR_ARG
 * otherwise).  The next frame starts at init. */
int xb_ctx_set_params(xb_ctx* ctx, const xb_params* p);
/* Context options.  "trace" (0/1): keep host copies of the intermediate
 * results of every stage for xb_get_array (parity checks; costs copies).
 * "time_kernels" (0/1): time the main kernels with CUDA events on the
 * context stream; xb_get_scalar("kt:<kernel>:ms" / "kt:<kernel>:n") returns
 * the accumulated milliseconds / launch count (setting it resets them).
 * "autotune" (0/1, default 1): the first launch of a tunable kernel for a
 * frame shape times its tile-shape variants (identical results) and keeps
 * the fastest for the process (XB_TUNE_CACHE=<file> persists the choices);
 * xb_get_scalar("tune:<kernel>") reports the choice.  0 uses the defaults.
 * "tune_variant" (-1 default): launch variant k of every tunable kernel
 * (checks that the variants agree).
 * "rank" (0/1/2): reorder every stamp's substamps by the learned ranker
 * after sss (needs xb_ranker_set): 1 moves the candidates whose accept
 * probability is below "rank_tau" (thousandths, default 500) behind the
 * others, keeping the reference's order within each group; 2 sorts all by
 * score.
 * "rank_candidates" (0..16, default 0 = every candidate): score and reorder
 * only the first n candidates of each stamp (the reference's brightest
 * first); the others keep their places after them.
 * "ldl_panel" (0/1, default 1, mixed mode): let the tuner choose among the
 * column LDL^T kernel and its panel variants (identical factors); 0 keeps
 * the column kernel.
 * "ldl_cluster" (16 or 8, default 16, mixed mode): CTAs of the LDL^T cluster
 * (identical factors).
 * "gram_fp64" (0/1, mixed mode): compute the per-stamp Gram matrices with
 * FP64 accumulation on the CUDA cores instead of the exact tensor-core
 * slicing (a cross-check; the results agree to rounding).
 * "fill_gram" (0/1, default 1, mixed mode): run the substamp fill and the
 * tensor-core Gram of each stamp as one kernel (window by TMA tile copy, W
 * written once) where the shape allows; 0 runs the separate fill, finish
 * and Gram kernels.  The results are the same bit for bit.
 * "fill_gram_tma" (0/1, default 1): let the fused kernel stage its windows
 * by TMA tile copies (0: plain loads; the same results).
 * "test_wait_timeout" (0/1, mixed mode, for tests): every CTA of the fused
 * fill + Gram kernel first waits on a barrier nothing arrives at, with a
 * 1 ms bound; the wait runs out, the CTA records a device timeout and goes
 * on with its real waits, so the frame ends with XB_ERR_DEVICE_TIMEOUT from
 * cd (or from the frame graph's record) while the context stays usable.
 * "graph" (0/1, mixed mode only): xb_run, xb_run_device and batches replay
 * each frame as one captured CUDA graph.  The host decisions of the stages
 * (kept-stamp counts, the sss retry, the cd test lists and direction, the ksc
 * refit loop) run on the device as conditional nodes; the first frame of a
 * shape (size and parameters) runs stage by stage and is captured, later
 * frames of that shape replay it with one synchronisation.  Results are the
 * stage-by-stage results bit for bit (the learned ranking included).
 * Ignored while "trace" or "time_kernels" is on. */
int xb_set_option(xb_ctx* ctx, const char* name, long long value);

/* ---- stage API (include/bach.h:66-87) ------------------------------------ */

/* init (src/bach.cpp:14-42): upload template T and science S (FP64 or FP32
 * host arrays, w*h each) and build the input mask (maskInput + spreadMask).
 * Returns XB_ERR_SIZE_MISMATCH if the sizes differ, as the reference exits. */
int xb_init(xb_ctx* ctx, const double* T, int tw, int th, const double* S,
            int sw, int sh);
int xb_init_f32(xb_ctx* ctx, const float* T, int tw, int th, const float* S,
                int sw, int sh);
/* Same, with T and S already resident in device memory (FP32). */
int xb_init_device_f32(xb_ctx* ctx, const float* dT, const float* dS, int w,
                       int h);

/* sss (src/bach.cpp:44-170): stamps, statistics, substamps, compaction,
 * low-threshold retry. */
int xb_sss(xb_ctx* ctx);
/* cmv (src/bach.cpp:172-268): basis-convolved substamps W, Gram Q, B. */
int xb_cmv(xb_ctx* ctx);
/* cd (src/bach.cpp:270-313): test fits in both directions.  *convTemplate
 * receives 1 when the template is the image to convolve. */
int xb_cd(xb_ctx* ctx, int* convTemplate);
/* ksc (src/bach.cpp:315-323): global kernel fit with substamp rejection. */
int xb_ksc(xb_ctx* ctx);
/* conv (src/bach.cpp:325-413): spatially varying convolution.  *kernSum
 * receives the kernel sum at the image centre. */
int xb_conv(xb_ctx* ctx, double* kernSum);
/* sub (src/bach.cpp:415-440): difference image. */
int xb_sub(xb_ctx* ctx);
/* All of init..sub in order (fin = reading the images back). */
int xb_run(xb_ctx* ctx, const float* T, const float* S, int w, int h,
           float* convOut, float* diffOut);
/* All of init..sub from device images to device images (dConv/dDiff may be
 * NULL); the frame graph path when option "graph" is on.  The caller's input
 * buffers are only read during the call. */
int xb_run_device(xb_ctx* ctx, const float* dT, const float* dS, int w, int h,
                  float* dConv, float* dDiff);

/* ---- results -------------------------------------------------------------- */
#define XB_IMG_CONV 0 /* convolved image, the `-o` output (default diff.fits) */
#define XB_IMG_DIFF 1 /* difference image, `sub.fits` */
#define XB_IMG_MASK 2 /* 16-bit mask word per pixel (use xb_get_mask) */
int xb_get_image(xb_ctx* ctx, int which, float* out);
int xb_get_image_f64(xb_ctx* ctx, int which, double* out);
int xb_get_mask(xb_ctx* ctx, uint16_t* out);
/* Input mask for the following frames (no counterpart in the reference,
 * which defines the INPUT_MASK bit, include/datatypeUtil.h:179, but never
 * sets it): pixels whose byte is nonzero get XB_MASK_INPUT_MASK and
 * XB_MASK_BAD_INPUT when a frame is initialised, before the bad-input mask is
 * dilated, so they are treated like the frame's own bad pixels in the
 * substamp search; the convolution treats them as bad input too, as HOTPANTS
 * does with its input masks: they get XB_MASK_BAD_OUTPUT (difference 1e-30)
 * and the pixels whose kernel covers them XB_MASK_BAD_CONV or XB_MASK_OK_CONV.
 * mask is w x h (row-major); a frame of another size fails with
 * XB_ERR_SIZE_MISMATCH.  NULL clears it. */
int xb_set_input_mask(xb_ctx* ctx, const uint8_t* mask, int w, int h);
/* Device pointers of the FP32 conv / diff images (valid until the next init
 * or destroy); for callers that keep results on the GPU. */
int xb_get_device_images(xb_ctx* ctx, const float** dConv, const float** dDiff);
/* Kernel solution vector (nKernSolComp entries, 1-based like the reference;
 * *n receives the length). */
int xb_get_solution(xb_ctx* ctx, double* out, int cap, int* n);

/* Generic introspection for parity checks: copies the named result array
 * into `out` (at most `cap` bytes) and returns its size in bytes in *nbytes.
 * Names are listed in the library's documentation (e.g. "sky0", "fwhm0",
 * "ss_count0", "ss_xy0", "ss_val0", "cur", "merit", "kernel_sums0"). */
int xb_get_array(xb_ctx* ctx, const char* name, void* out, size_t cap,
                 size_t* nbytes);
/* Scalar introspection ("convTemplate", "kernSum", "ksc_iterations",
 * "stampsx", "stampsy", "fStampWidth", "sss_retry", "nstamps0", ...). */
int xb_get_scalar(xb_ctx* ctx, const char* name, double* out);

/* Number of this library's kernels launched since the context was created
 * (for benchmark accounting). */
long long xb_kernel_launches(const xb_ctx* ctx);
/* The CUDA stream (cudaStream_t) all of the context's work runs on, for
 * callers that record events or order their own work against it. */
int xb_get_stream(xb_ctx* ctx, void** stream);

/* ---- allocation-free stamp statistics ------------------------------------ */
/* No counterpart in the reference.  For callers that cannot allocate device
 * memory (another allocator owns the device, or a cudaMalloc would stall
 * their work): the sky level and robust sigma of every stamp, computed by the
 * same kernel as xb_sss, with all scratch taken from a 32 MiB device array
 * built into the library (held on every GPU that loads it until exit).
 *   dImg   w*h FP32 image, device memory
 *   dMask  w*h mask words (in/out: NaN pixels inside a stamp's fStampWidth^2
 *          area get NAN_PIXEL|BAD_INPUT, as in xb_sss)
 *   dGeom  nStamps x {x, y, width, height} ints, 16-byte aligned, device.
 *          Each stamp must have the form of the reference's stamp grid
 *          (createStampBounds, cl_kern/sss.cl:19-40): 0 <= x < w, 0 <= y < h,
 *          width = min(fStampWidth, w - x), height = min(fStampWidth, h - y),
 *          as every stamp xb_sss builds does.  A stamp that does not gets
 *          NaN in dSky and dFwhm, and none of its pixels is read.
 *   dSky, dFwhm  nStamps doubles each, device memory
 *   stream cudaStream_t to launch on (NULL = legacy default stream); the call
 *          returns after the launch, results are ready when the stream is
 * Limit: nStamps * (9 * P + 16 * ceil(fStampWidth^2 / 32)) bytes, P =
 * fStampWidth^2 rounded up to a multiple of 1024, must fit in 32 MiB (2048^2
 * with 16x16 stamps of 107 px needs 28.4 MiB);
 * larger requests return XB_ERR_UNSUPPORTED and nothing runs.  The first call
 * on each device looks up the array's device address, so make that first call
 * before capturing a stream; the address is kept for the device's context,
 * so do not use the entry point across a cudaDeviceReset.  All calls share
 * the one array: calls whose launches overlap on the GPU race with each
 * other; the kernel needs nothing cleared, it writes every scratch byte
 * before reading it.  Errors: XB_ERR_ARG (null pointer, non-positive size,
 * unaligned dGeom), XB_ERR_UNSUPPORTED (beyond the limit), XB_ERR_CUDA (a
 * CUDA error was already pending when the call began -- reported and left in
 * place, nothing launched -- or the launch itself failed).  `err` (may be
 * NULL) receives a message on failure.  Calls no allocation routine. */
int xb_stamp_stats_noalloc(const float* dImg, uint16_t* dMask, int w, int h,
                           const int* dGeom, int nStamps, int fStampWidth,
                           double sigClipAlpha, double iqRange, double* dSky,
                           double* dFwhm, void* stream, char* err,
                           size_t errCap);

/* ---- batches of frame pairs ---------------------------------------------- */
/* No counterpart in the reference, whose main (src/main.cpp) runs one pair
 * per process.  A batch owns nWorkers contexts, each with its own stream and
 * host thread; the frames of a run are taken from one queue in order and run
 * through the whole stage sequence (init .. sub) concurrently on the GPU.
 * Frames may differ in size.  Results are per frame and identical to xb_run
 * on a single context. */
typedef struct xb_batch xb_batch;
int xb_batch_create(const xb_params* p, int device, int nWorkers, xb_batch** out);
int xb_batch_destroy(xb_batch* b);
const char* xb_batch_last_error(const xb_batch* b);
/* Host frames: T[i], S[i] are w[i] x h[i] FP32 arrays (pinned memory makes
 * the uploads asynchronous); conv[i], diff[i] receive the outputs (either
 * may be NULL).  frameStatus[i] and kernSum[i] (each may be NULL) receive
 * each frame's status and kernel sum.  Returns XB_OK when every frame
 * succeeded, else the status of the first failing frame (its message in
 * xb_batch_last_error). */
int xb_batch_run(xb_batch* b, int nFrames, const float* const* T, const float* const* S,
                 const int* w, const int* h, float* const* conv, float* const* diff,
                 int* frameStatus, double* kernSum);
/* Device frames: the same with device pointers for inputs and outputs. */
int xb_batch_run_device(xb_batch* b, int nFrames, const float* const* dT,
                        const float* const* dS, const int* w, const int* h,
                        float* const* dConv, float* const* dDiff, int* frameStatus,
                        double* kernSum);
/* Worker context i (options such as "time_kernels", timers, launch counts). */
int xb_batch_worker(xb_batch* b, int i, xb_ctx** ctx);
/* Parameters per frame for later runs: params[i] applies to frame i (stamp
 * grid, thresholds, clipping); every set must keep the batch's basis,
 * widths, orders and mode (XB_ERR_ARG otherwise).  nFrames = 0 returns to
 * the batch's parameters.  With option "graph" on every worker, frames are
 * dealt to workers by a fixed schedule (largest first to the least-loaded
 * worker), so a repeated list of frames replays captured graphs. */
int xb_batch_set_params(xb_batch* b, int nFrames, const xb_params* params);
/* Joins a caller's cudaStream_t to every later run: the workers' first
 * launches wait for the work already queued on `stream`, and work queued on
 * `stream` after the run waits for every worker, so CUDA events recorded on
 * `stream` before and after a run bracket all of its GPU work.  NULL detaches. */
int xb_batch_set_stream(xb_batch* b, void* stream);

/* Measured FMA throughput of the device's CUDA cores, FP32 and FP64 (TFLOP/s,
 * one FMA = 2 operations; best of three ~10-20 ms launches): the
 * denominators of the roofline figures of kernels bound by those pipes. */
int xb_measure_fma_peaks(int device, double* fp32Tflops, double* fp64Tflops);

/* The left-to-right FP64 sum of c[0..n) that the stamp statistics use for the
 * reference's serial sigma-clip sums (bachUtil.cpp:34-128): 32 terms per step
 * of one warp, equal bit for bit to `s = 0; for(i) s += c[i]` for every input.
 * _host runs the same steps on the CPU; _device runs the warp on `stream`
 * over device arrays (dC: n doubles, dOut: one double). */
double xb_ordered_sum_host(const double* c, int n);
int xb_ordered_sum_device(const double* dC, int n, double* dOut, void* stream);
/* The same over FP32 terms, each widened to FP64 before it is added (the
 * substamp values of the substamp search, sss.cl:396-541). */
int xb_ordered_sum_device_f32(const float* dC, int n, double* dOut, void* stream);

/* ---- streaming pipeline over FITS files ---------------------------------- */
/* No counterpart in the reference, whose main (src/main.cpp:16-159) reads
 * two FITS files, runs the stages and writes conv and sub once per process.
 * A pipeline overlaps those steps across pairs: nIo reader threads decode
 * FITS pairs into pinned host slots (FP32 for unscaled BITPIX -32, FP64
 * otherwise), nWorkers contexts run xb_run on them (the frame graph when
 * option "graph" is on; FP64 pairs run the plain stages and are refused in
 * mixed mode), and nIo writer threads encode conv and diff as BITPIX -32.
 * Each pair's images are those of xb_run on a single context.  One call at a
 * time per pipeline (its workers and slots are reused by every call). */
typedef struct xb_pipeline xb_pipeline;
typedef struct {
  double wall_ms;       /* last run, start to last write */
  double read_ms;       /* summed over reader threads: open + decode */
  double compute_ms;    /* summed over workers: xb_run, copies included */
  double write_ms;      /* summed over writer threads: encode + write */
  double bytes_read;    /* FITS sample bytes decoded */
  double bytes_written; /* FITS sample bytes encoded */
  int pairs;            /* pairs in the last run */
} xb_pipeline_stats;
int xb_pipeline_create(const xb_params* p, int device, int nWorkers, int nIo,
                       xb_pipeline** out);
int xb_pipeline_destroy(xb_pipeline* pl);
const char* xb_pipeline_last_error(const xb_pipeline* pl);
/* Worker context i (options such as "graph", "rank", an input mask). */
int xb_pipeline_worker(xb_pipeline* pl, int i, xb_ctx** ctx);
/* Pair i: templatePath[i] and sciencePath[i] in; convPath[i] and diffPath[i]
 * out (a NULL list or entry skips that output).  pairStatus[i] and
 * kernSum[i] (each may be NULL) receive each pair's status (XB_ERR_IO for a
 * file that cannot be opened, read or written) and kernel sum.  Returns
 * XB_OK when every pair succeeded, else the first failing pair's status (its
 * message in xb_pipeline_last_error). */
int xb_pipeline_run_files(xb_pipeline* pl, int nPairs, const char* const* templatePath,
                          const char* const* sciencePath, const char* const* convPath,
                          const char* const* diffPath, int* pairStatus, double* kernSum);
/* Parameters per pair for later runs: params[i] applies to pair i (stamp
 * grid, thresholds, clipping, noise model); every set must keep the
 * pipeline's basis, widths, orders and mode (XB_ERR_ARG otherwise).
 * nPairs = 0 returns to the pipeline's parameters. */
int xb_pipeline_set_params(xb_pipeline* pl, int nPairs, const xb_params* params);
/* Timings and byte counts of the last run. */
int xb_pipeline_stats_get(const xb_pipeline* pl, xb_pipeline_stats* out);

/* ---- learned substamp ranking -------------------------------------------- */
/* No counterpart in the reference.  A small network (a 3-layer CNN over the
 * 2x31x31 template/science window pair plus an MLP over 16 window
 * statistics, 2161 parameters) scores every candidate substamp; with
 * option "rank" on and weights loaded, xb_sss reorders each stamp's
 * candidates by descending score, so the ones the ksc fit would reject are
 * tried last.  The ksc sigma-clip check still judges every pick.  The
 * network computes with BF16 weights and FP32 activations and sums: the
 * training calls below take FP32 master weights (which Adam updates) and
 * round each to BF16 (nearest, ties to even) as they load it; xb_ranker_set
 * stores the context's copy as BF16. */
int xb_ranker_param_count(void);
/* Loads the network's parameters (host array of xb_ranker_param_count()). */
int xb_ranker_set(xb_ctx* ctx, const float* weights, int n);
/* Features of every candidate substamp of stamp set `set` (0: stamps found on
 * the template, 1: on the science) after xb_sss: stats (n x 16), pix
 * (n x 2 x 31 x 31), and each candidate's stamp index and slot.  With all
 * four arrays NULL only *nOut is set.  cap is the capacity in candidates. */
int xb_ranker_features(xb_ctx* ctx, int set, float* stats, float* pix, int* stamp, int* slot,
                       int cap, int* nOut);
/* Training and inference kernels on device arrays (stream: cudaStream_t).
 * forward: logits of n candidates.  grad: per-sample gradients of the
 * weighted binary cross-entropy (dGradPerSample: n x param_count scratch),
 * their batch mean in dGrad, per-sample losses in dLoss; dWeight may be
 * NULL.  adam: one Adam step (b1 0.9, b2 0.999, eps 1e-8; step >= 1). */
int xb_ranker_forward(const float* dW, const float* dStats, const float* dPix, int n,
                      float* dLogit, void* stream);
int xb_ranker_grad(const float* dW, const float* dStats, const float* dPix, const float* dLabel,
                   const float* dWeight, int n, float* dGradPerSample, float* dGrad,
                   float* dLoss, void* stream);
int xb_ranker_adam(float* dW, const float* dGrad, float* dM, float* dV, int step, float lr,
                   void* stream);

/* ---- FITS I/O (src/fitsUtil.cpp:8-64 without CCfits) -------------------- */
/* Reads the primary HDU (BITPIX -32 or -64) into a newly malloc'ed FP64
 * array (free with xb_free).  Returns XB_ERR_IO / XB_ERR_UNSUPPORTED. */
int xb_fits_read(const char* path, double** data, int* w, int* h);
/* Writes a BITPIX -32 primary HDU (the reference writes FLOAT_IMG). */
int xb_fits_write(const char* path, const double* data, int w, int h);
void xb_free(void* p);

#ifdef __cplusplus
}
#endif

#endif /* XBACH_H */
