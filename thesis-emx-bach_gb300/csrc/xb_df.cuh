// xb_df.cuh — the mixed path's substamp fill arithmetic, shared by the
// separate fill kernels (xb_mixed.cu) and the fused fill + Gram kernel
// (xb_fill_gram.cu) so that both write the same W bit for bit.
//
// The normal matrices are ill-conditioned enough that a W rounded to FP32
// (2^-24 per element) moves the difference image of the reference's own
// test case (cond ~6e13) by ~1e-3 of the pixel noise.  So W is kept as an
// unevaluated sum hi + lo of two floats (~48 bits), computed on the FP32 pipe
// (GB300's FP64 rate is 1/64 of FP32) with error-free transformations; the
// library is built without FMA contraction, so the two-sums below are exact.
//   * Y pass (convStampY, cl_kern/cmv.cl:70-106): the reference accumulates
//     in float over FP64 products, v = (float)((double)v + img * fy), and
//     the rounding of every step is part of its result.  It is reproduced:
//     fy = fh + fl as floats, img*fh split exactly by an FMA, the sum
//     v + product formed exactly (two-sum) and rounded once to float.  The
//     result equals the reference's except when v + product lies within
//     ~2^-47 of a float rounding boundary (~1 step in 10^7).
//   * X pass (convStampX, :108-135, FP64 there): double-float accumulation.
//   * convStampOdd (:137-154): W[n] - W[0] as a double-float difference.
//   * convStampBg (:156-193): FP64 there; split into hi + lo.
#pragma once

namespace xb {
namespace df {

// the reference's float-normalised coordinate (cl_kern/cmv.cl:156-193)
__device__ __forceinline__ float floatNormF(int x, int w) {
  float hw = (float)w * 0.5f;
  return ((float)x - hw) / hw;
}

// one step of the reference's float Y accumulation: (float)(v + a * (fh + fl))
__device__ __forceinline__ float refStepY(float v, float a, float fh, float fl) {
  const float ph = a * fh;
  const float pe = fmaf(a, fh, -ph);  // a*fh = ph + pe exactly
  const float pl = a * fl;
  const float s = v + ph;             // two-sum: v + ph = s + e exactly
  const float bb = s - v;
  const float e = (v - (s - bb)) + (ph - bb);
  return s + (e + (pe + pl));
}
// (sh, sl) += t * (fh + fl)
__device__ __forceinline__ void dfAccum(float& sh, float& sl, float t, float fh, float fl) {
  const float ph = t * fh;
  const float pe = fmaf(t, fh, -ph);
  const float s = sh + ph;
  const float bb = s - sh;
  const float e = (sh - (s - bb)) + (ph - bb);
  sh = s;
  sl += e + (pe + t * fl);
}
// renormalised hi + lo of sh + sl
__device__ __forceinline__ void dfNorm(float sh, float sl, float& hi, float& lo) {
  const float s = sh + sl;
  const float bb = s - sh;
  hi = s;
  lo = (sh - (s - bb)) + (sl - bb);
}
// (ah + al) - (bh + bl), renormalised (convStampOdd)
__device__ __forceinline__ void dfSub(float ah, float al, float bh, float bl, float& hi, float& lo) {
  const float s = ah - bh;  // two-sum of ah and -bh
  const float bb = s - ah;
  const float er = (ah - (s - bb)) + (-bh - bb);
  dfNorm(s, er + (al - bl), hi, lo);
}
__device__ __forceinline__ void splitF64(double v, float& hi, float& lo) {
  hi = (float)v;
  lo = (float)(v - (double)hi);
}

}  // namespace df
}  // namespace xb
