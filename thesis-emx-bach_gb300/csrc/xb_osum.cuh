// xb_osum.cuh — left-to-right FP64 sums of nonnegative terms, bit for bit,
// 32 terms per step of one warp.
//
// The reference forms its sigma-clip sums on the host as one serial FP64
// loop over the per-work-item partial sums (bachUtil.cpp:34-128), and every
// rounding of that loop is part of the mean and deviation that decide the
// stamp statistics.  A dependent FP64 add costs ~60 cycles on this part, so
// a 512-term chain is ~30k cycles.
//
// While the running sum s stays in one binade [2^E, 2^(E+1)), it is an
// integer multiple S of u = 2^(E-52), and for a term x >= 0 whose quotient
// x/u is not a tie (fraction exactly 1/2), RN(s + x) = (S + rint(x/u)) u as
// long as S + rint(x/u) < 2^53: the exact sum lies within u/2 of that
// multiple and inside the binade, where u is the spacing of the doubles.  So
// a warp rounds 32 terms onto the grid of u with integer operations, takes
// an inclusive prefix sum, and accepts the terms up to the first one that
// would leave the binade, is a tie, or is not a finite nonnegative number;
// that term is added in FP64 exactly as the serial loop does, and the step
// repeats from the new sum.  A running sum that is subnormal, negative or not
// finite also takes the FP64 add; from +0 the zero terms are skipped.  The
// result equals the serial loop for every input; sums of positive terms
// leave a binade about log2(n) times, so most steps take 32 terms.
#pragma once

#include <cstdint>

namespace xb {
namespace osum {

constexpr long long kFrac = (1ll << 52) - 1;

struct Grid {
  long long n;  // rint(x / u)
  bool ok;      // x finite, >= 0, below 2^(E+1), and x/u not a tie
};

__host__ __device__ inline long long bitsOf(double x) {
#ifdef __CUDA_ARCH__
  return __double_as_longlong(x);
#else
  long long b;
  __builtin_memcpy(&b, &x, sizeof b);
  return b;
#endif
}
__host__ __device__ inline double fromBits(long long b) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double(b);
#else
  double x;
  __builtin_memcpy(&x, &b, sizeof x);
  return x;
#endif
}

// x on the grid of u = 2^(sE - 1075), sE the biased exponent of a positive
// normal running sum
__host__ __device__ inline Grid onGrid(double x, int sE) {
  const long long xb = bitsOf(x);
  if(xb < 0) return {0, false};  // negative, or -0.0
  const int xE = (int)(xb >> 52);
  if(xE > sE) return {0, false};  // x >= 2^(E+1), infinite or NaN
  // x = mant * 2^(max(xE,1) - 1075), so x/u = mant * 2^-(sh)
  const long long mant = (xb & kFrac) | (xE ? (1ll << 52) : 0);
  const int sh = sE - (xE ? xE : 1);
  if(sh <= 0) return {mant, true};
  if(sh >= 54) return {0, true};  // x/u < 1/2
  const long long q = mant >> sh, rem = mant & ((1ll << sh) - 1), half = 1ll << (sh - 1);
  if(rem == half) return {0, false};
  return {q + (rem > half ? 1 : 0), true};
}

// a float term, from its bits (no FP64 operation)
__host__ __device__ inline Grid onGrid(float f, int sE) {
#ifdef __CUDA_ARCH__
  const unsigned b = __float_as_uint(f);
#else
  unsigned b;
  __builtin_memcpy(&b, &f, sizeof b);
#endif
  if(b == 0u || b == 0x80000000u) return {0, true};  // +-0 leaves a positive sum unchanged
  if(b >> 31) return {0, false};                      // negative
  const int ef = (int)(b >> 23);
  if(ef == 255) return {0, false};                    // infinite or NaN
  const long long mant = (long long)((b & 0x7FFFFFu) | (ef ? 0x800000u : 0u));
  const int sh = sE - ((ef ? ef : 1) + 925);           // f = mant * 2^(ef - 150), f/u = mant * 2^-sh
  if(sh <= 0) {
    if(-sh > 29) return {0, false};  // f >= 2^53 u
    return {mant << -sh, true};
  }
  if(sh >= 26) return {0, true};  // f/u < 1/4
  const long long q = mant >> sh, rem = mant & ((1ll << sh) - 1), half = 1ll << (sh - 1);
  if(rem == half) return {0, false};
  return {q + (rem > half ? 1 : 0), true};
}
__host__ __device__ inline bool nonZero(double x) { return !(x == 0.0); }
__host__ __device__ inline bool nonZero(float x) {
#ifdef __CUDA_ARCH__
  return (__float_as_uint(x) & 0x7FFFFFFFu) != 0u;
#else
  unsigned b;
  __builtin_memcpy(&b, &x, sizeof b);
  return (b & 0x7FFFFFFFu) != 0u;
#endif
}

// true when s is a positive normal double (the grid steps apply)
__host__ __device__ inline bool gridable(double s, int* sE, long long* S) {
  const long long sb = bitsOf(s);
  const int e = (int)((sb >> 52) & 0x7FF);
  if(sb <= 0 || e == 0 || e == 0x7FF) return false;
  *sE = e;
  *S = (sb & kFrac) | (1ll << 52);
  return true;
}

// The same steps on the host, one term at a time (the reference for tests).
inline double orderedSumHost(const double* c, int n) {
  double s = 0.0;
  int i = 0;
  while(i < n) {
    int sE;
    long long S;
    if(!gridable(s, &sE, &S)) {
      s = s + c[i];
      i++;
      continue;
    }
    const int len = n - i < 32 ? n - i : 32;
    int j = 0;
    for(; j < len; j++) {
      const Grid g = onGrid(c[i + j], sE);
      if(!g.ok || S + g.n >= (1ll << 53)) break;
      S += g.n;
    }
    if(j > 0) {
      s = fromBits(((long long)sE << 52) | (S - (1ll << 52)));
      i += j;
    }
    if(j < len) {
      s = s + c[i];
      i++;
    }
  }
  return s;
}

#ifdef __CUDACC__
// All 32 lanes of a warp call it with the same n and term(i), the i-th term
// as a double or as a float (whose grid steps need no FP64 operation);
// every lane returns the sum.  term is best a shared-memory read (one
// dependent read per step).
template <class F>
__device__ inline double warpOrderedSumOf(int n, F term) {
  const int lane = threadIdx.x & 31;
  double s = 0.0;
  int i = 0;
  while(i < n) {
    int sE;
    long long S0;
    if(!gridable(s, &sE, &S0)) {
      if(bitsOf(s) == 0) {
        // s = +0: zero terms leave it +0 and the first other term x gives
        // exactly x, so skip to it 32 terms at a time
        const int len = min(32, n - i);
        const auto x = lane < len ? term(i + lane) : decltype(term(0))(0);
        const unsigned nz = __ballot_sync(0xffffffffu, lane < len && nonZero(x));
        if(!nz) {
          i += len;
          continue;
        }
        const int j = __ffs(nz) - 1;
        s = s + (double)__shfl_sync(0xffffffffu, x, j);
        i += j + 1;
        continue;
      }
      s = s + (double)term(i);
      i++;
      continue;
    }
    const int len = min(32, n - i);
    Grid g = {0, false};
    if(lane < len) g = onGrid(term(i + lane), sE);
    long long P = g.n;  // inclusive prefix over the lanes
#pragma unroll
    for(int o = 1; o < 32; o <<= 1) {
      const long long t = __shfl_up_sync(0xffffffffu, P, o);
      if(lane >= o) P += t;
    }
    const bool ok = lane < len && g.ok && S0 + P < (1ll << 53);
    const unsigned bad = __ballot_sync(0xffffffffu, !ok);
    const int j = bad ? __ffs(bad) - 1 : 32;  // terms accepted
    const long long Pj = __shfl_sync(0xffffffffu, P, j > 0 ? j - 1 : 0);
    if(j > 0) {
      s = fromBits(((long long)sE << 52) | (S0 + Pj - (1ll << 52)));
      i += j;
    }
    if(j < len) {
      s = s + (double)term(i);
      i++;
    }
  }
  return s;
}
__device__ inline double warpOrderedSum(const double* c, int n) {
  return warpOrderedSumOf(n, [c](int i) { return c[i]; });
}
#endif

}  // namespace osum
}  // namespace xb
