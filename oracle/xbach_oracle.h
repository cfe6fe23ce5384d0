/*
 * xbach_oracle.h — CPU oracle of the X-BACH difference-imaging path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker: a plain FP64 C++
 * restatement of the reference algorithm (D0V4HKIIN/Thesis-EMX-BACH,
 * the src/ C++ files and the cl_kern/ OpenCL kernels), used by tests/, by
 * __graft_entry__.smoke()
 * and by bench.py's CPU-baseline leg.  Nothing in the product links it.
 *
 * Pinned against the reference's golden vectors: tests/test01_{conv,sub}.fits
 * (HOTPANTS outputs for res/test0 + res/test1, tolerances of
 * tools/run_test.py:13) and the test01 global normal matrix of
 * tools/cond_num.py:3-298.
 */
#ifndef XBACH_ORACLE_H
#define XBACH_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#include "../include/xbach.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct xbo_handle xbo_handle;

/* Runs init..sub on FP64 inputs.  `nthreads` <= 0 uses all OpenMP threads.
 * `keep_w` != 0 keeps the initial W of both stamp sets (large).
 * *status receives an XB_* code; the handle is returned even on failure
 * (free it with xbo_free). */
xbo_handle* xbo_run(const xb_params* p, const double* T, const double* S,
                    int w, int h, int nthreads, int keep_w, int* status);
/* The same with an input mask (w*h bytes, nonzero = excluded; the
 * extension of xb_set_input_mask): INPUT_MASK | BAD_INPUT at init before the
 * dilation, bad input for the convolution. */
xbo_handle* xbo_run_masked(const xb_params* p, const double* T, const double* S,
                           const uint8_t* inMask, int w, int h, int nthreads,
                           int keep_w, int* status);
int xbo_get_array(const xbo_handle* h, const char* name, void* out,
                  size_t cap, size_t* nbytes);
int xbo_get_scalar(const xbo_handle* h, const char* name, double* out);
void xbo_free(xbo_handle* h);

/* Unit-level entry points (known-answer tests). */
/* sigmaClip of src/bachUtil.cpp:34-128 with the 32-chunk summation of
 * cl_kern/bach.cl:135-170. */
void xbo_sigma_clip(const double* data, int n, int maxIter, double alpha,
                    double* mean, double* stdDev);
/* calcStats of src/bachUtil.cpp:130-280 (sampling, maskStamp, sigmaClip,
 * createHistogram) for caller-given stamps: geom holds n x {x, y, width,
 * height}, every stamp inside the image with width*height >= 100 (else
 * XB_ERR_STAMP_TOO_SMALL); mask is in/out (NaN pixels get
 * NAN_PIXEL|BAD_INPUT). */
int xbo_stamp_stats(const double* img, uint16_t* mask, int w, int h, const int* geom,
                    int n, int fStampWidth, double sigClipAlpha, double iqRange, double* sky,
                    double* fwhm);
/* Numerical-Recipes ran1 of cl_kern/sss.cl:52-79, seeded with idum; writes
 * n deviates. */
void xbo_ran1_seq(int idum, int n, double* out);
/* CPU ludcmp + lubksb of src/bachUtil.cpp:319-411 on a 1-based
 * (n+1)x(n+1) row-major matrix; rhs has >= n+1 entries.  Returns 1 when a
 * row is all zero (the reference's error return). */
int xbo_lu_solve(double* a, int n, double* rhs);

#ifdef __cplusplus
}
#endif

#endif
