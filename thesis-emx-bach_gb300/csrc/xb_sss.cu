// xb_sss.cu — the sss stage: stamp grid, per-stamp statistics, substamp
// search, empty-stamp compaction and the low-threshold retry
// (src/bach.cpp:44-170, src/sssUtil.cpp, src/bachUtil.cpp:130-280,
// cl_kern/sss.cl).
//
// Every quantity that decides a stamp or substamp is computed in the
// reference's operation order (no contraction: the library is built with
// -fmad=false), so the stamp and substamp sets are bit-identical to the CPU
// oracle.  Where the reference compacts with atomics (maskStamp,
// sss.cl:157-188) the order is the ascending pixel index.

#include <algorithm>
#include <climits>
#include <cmath>

#include "xb_device.cuh"
#include "xb_internal.h"
#include "xb_osum.cuh"

namespace xb {

namespace {

constexpr int NSAMPLES = 100, PADDED = 128;
constexpr int ST_THREADS = 256;
constexpr int ST_CHUNKS_SMEM = 1280;  // chunk sums kept in shared memory (stamps <= 40960 px)

__device__ __forceinline__ int satFloorToInt(double v) {
  double f = floor(v);
  if(f != f) return 0;
  if(f >= 2147483647.0) return INT_MAX;
  if(f <= -2147483648.0) return INT_MIN;
  return (int)f;
}

// Numerical Recipes ran1 (cl_kern/sss.cl:52-79): three LCGs with a
// 97-entry shuffle table; 64-bit integer state, exact.
struct Ran1 {
  long long ix1, ix2, ix3;
  int idum, iff;
  __host__ __device__ void init(int seed) {
    idum = seed;
    iff = 0;
    ix1 = ix2 = ix3 = 0;
  }
  __host__ __device__ double next(double* r) {
    const long long M1 = 259200, IA1 = 7141, IC1 = 54773;
    const long long M2 = 134456, IA2 = 8121, IC2 = 28411;
    const long long M3 = 243000, IA3 = 4561, IC3 = 51349;
    const double RM1 = 1.0 / 259200, RM2 = 1.0 / 134456;
    if(idum < 0 || iff == 0) {
      iff = 1;
      ix1 = (IC1 - idum) % M1;
      ix1 = (IA1 * ix1 + IC1) % M1;
      ix2 = ix1 % M2;
      ix1 = (IA1 * ix1 + IC1) % M1;
      ix3 = ix1 % M3;
      for(int j = 1; j <= 97; j++) {
        ix1 = (IA1 * ix1 + IC1) % M1;
        ix2 = (IA2 * ix2 + IC2) % M2;
        r[j] = ((double)ix1 + (double)ix2 * RM2) * RM1;
      }
      idum = 1;
    }
    ix1 = (IA1 * ix1 + IC1) % M1;
    ix2 = (IA2 * ix2 + IC2) % M2;
    ix3 = (IA3 * ix3 + IC3) % M3;
    int j = 1 + (int)((97 * ix3) / M3);
    double t = r[j];
    r[j] = ((double)ix1 + (double)ix2 * RM2) * RM1;
    return t;
  }
};

// ------------------------------------------------------- stamp statistics --
// One CTA per stamp: sampleStamp + pad + sortSamples (sss.cl:81-150),
// maskStamp (:157-188), sigmaClip with maxIter 3 (bachUtil.cpp:255-266,
// bach.cl:129-184) and createHistogram (sss.cl:190-324).
//
// Every stamp seeds ran1 with -666, so all stamps draw the same sequence:
// with `draws` (that sequence, precomputed on the host) the 32 candidates of
// a sampling round are formed in parallel; without it lane 0 runs ran1.
// The clip test |v - m| * inv > alpha is monotone in v on each side of m, so
// each clip round first finds the exact thresholds v_lo < m < v_hi where it
// turns true (a 32-ary search of one warp over the ordered doubles) and then
// compares pixels against them.  The histogram bin floor((v - lbv) / bs) of
// an FP32 pixel comes from an FP32 estimate whose error is bounded per pass;
// only pixels within that bound of a bin edge redo it in FP64.  All decisions
// and sums are those of the reference's order.

// The good-pixel list of a stamp, chunk-interleaved: entry q lives at
// slot ((q >> 10) << 10) | ((q & 31) << 5) | ((q >> 5) & 31) of the stamp's
// slice, whose length is fSW^2 rounded up to a multiple of 1024.
__host__ __device__ __forceinline__ size_t statsSlice(int fSW) {
  return ((size_t)fSW * fSW + 1023) & ~(size_t)1023;
}
__device__ __forceinline__ int listSlot(int q) {
  return ((q >> 10) << 10) | ((q & 31) << 5) | ((q >> 5) & 31);
}
__device__ __forceinline__ int chunkSlot(int c, int l) {  // entry c * 32 + l
  return ((c >> 5) << 10) | (l << 5) | (c & 31);
}
__device__ __forceinline__ int listEntry(int slot) {  // inverse of listSlot
  return ((slot >> 10) << 10) | ((slot & 31) << 5) | ((slot >> 5) & 31);
}

// Order-preserving map of doubles (no NaN) to 64-bit keys and back.
__device__ __forceinline__ unsigned long long dKey(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double keyD(unsigned long long k) {
  const unsigned long long b = (k >> 63) ? (k & 0x7FFFFFFFFFFFFFFFull) : ~k;
  return __longlong_as_double((long long)b);
}
__device__ __forceinline__ bool clipOut(double v, double m, double inv, double alpha) {
  return fabs(v - m) * inv > alpha;
}

// One warp: the key of the first double (walking away from m, upwards when
// up, downwards otherwise) at which clipOut turns true; `none` when it never
// does.  clipOut is false at m and monotone along the walk.
__device__ unsigned long long clipEdge(double m, double inv, double alpha, bool up, bool* none) {
  const int lane = threadIdx.x & 31;
  const unsigned long long kEnd = dKey(up ? INFINITY : -INFINITY);
  unsigned long long lo = dKey(m), hi = kEnd;  // clipOut(lo) false, clipOut(hi) true
  *none = !clipOut(up ? INFINITY : -INFINITY, m, inv, alpha);
  if(*none) return kEnd;
  for(int guard = 0; guard < 40; guard++) {
    const unsigned long long span = up ? hi - lo : lo - hi;
    if(span <= 1) break;
    unsigned long long step = span / 33;
    if(step == 0) step = 1;
    const unsigned long long off = (unsigned long long)(lane + 1) * step;
    const bool valid = off < span;
    const unsigned long long k = up ? lo + off : lo - off;
    const bool p = valid && clipOut(keyD(k), m, inv, alpha);
    const unsigned bal = __ballot_sync(0xffffffffu, p);
    const unsigned vmask = __ballot_sync(0xffffffffu, valid);
    if(bal) {
      const int j = __ffs(bal) - 1;
      const unsigned long long kj = __shfl_sync(0xffffffffu, k, j);
      const unsigned long long kprev = __shfl_sync(0xffffffffu, k, j > 0 ? j - 1 : 0);
      hi = kj;
      if(j > 0) lo = kprev;
    } else {
      const int jl = 31 - __clz(vmask);
      lo = __shfl_sync(0xffffffffu, k, jl);
    }
  }
  return hi;
}

template <class T>
__global__ void __launch_bounds__(ST_THREADS, 3)
    k_stamp_stats(const T* __restrict__ img, uint16_t* __restrict__ mask,
                  const int4* __restrict__ geom, int w, int h, int fSW,
                  T* __restrict__ good, uint8_t* __restrict__ clip,
                  double* __restrict__ chunkBuf, int maxChunks,
                  double sigClipAlpha, double iqRange, double* __restrict__ skyOut,
                  double* __restrict__ fwhmOut, const double* __restrict__ draws) {
  const int s = blockIdx.x;
  const int4 gm = geom[s];  // cx, cy, sx, sy
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  constexpr bool F32 = sizeof(T) == 4;
  // A stamp must have the form of the reference's grid (createStampBounds,
  // cl_kern/sss.cl:19-40): its origin inside the image and its size the full
  // stamp width clipped by the image edge.  Its histogram is then taken over
  // the good pixels of the clipped fSW^2 window (phase D), which are exactly
  // the stamp's pixels.  The grid that xb_sss builds always has this form;
  // geometry passed in from outside (xb_stamp_stats_noalloc) that does not
  // gets NaN statistics and no pixel of it is read (the test is uniform over
  // the CTA, before any barrier).
  if(gm.x < 0 || gm.y < 0 || gm.x >= w || gm.y >= h || gm.z != min(fSW, w - gm.x) ||
     gm.w != min(fSW, h - gm.y)) {
    if(tid == 0) {
      skyOut[s] = __longlong_as_double(0x7ff8000000000000ll);
      fwhmOut[s] = __longlong_as_double(0x7ff8000000000000ll);
    }
    return;
  }
  __shared__ double samples[PADDED];
  __shared__ double rtab[98];
  __shared__ int cand[32];
  __shared__ int sCount;
  __shared__ int warpTot[ST_THREADS / 32];
  __shared__ int sTotal;
  __shared__ double sMean, sStd, sInv, sSum, sSum2;
  __shared__ int sPrev, sCurr, sClip, sDone;
  __shared__ int bins[256];
  __shared__ long long hC[257], hCE[257];  // prefix sums of the bin counts (and of index * count)
  __shared__ int okCount;
  __shared__ double hLower, hUpper, hSky, hBinSize, hLowerBinVal;
  __shared__ int hState;  // 0 continue, 1 stop (setFwhm), 2 stop (no fwhm)
  __shared__ double tLo, tHi;          // clip thresholds of the current round
  __shared__ float fLo, fHi;           // the same, rounded outward to float
  __shared__ int tNoLo, tNoHi, tDirect;
  __shared__ float bLbv, bInv, bDelta;  // FP32 bin estimate of the current pass
  __shared__ int bExact;

  // ---- phase A: random sampling (warp 0) ----
  if(tid < 32) {
    Ran1 rng;
    if(lane == 0) {
      rng.init(-666);
      sCount = 0;
    }
    const int numPix = gm.z * gm.w;
    // with the draws, the candidates of the first PRE rounds (32 each) are
    // read together
    constexpr int PRE = 4;
    double preV[PRE];
    bool preOk[PRE];
#pragma unroll
    for(int r = 0; r < PRE; r++) {
      preV[r] = 0.0;
      preOk[r] = false;
      if(draws && r * 32 + lane < numPix) {
        const int rx = (int)floor(draws[2 * (r * 32 + lane)] * (int)gm.z);
        const int ry = (int)floor(draws[2 * (r * 32 + lane) + 1] * (int)gm.w);
        const int idx = (rx + gm.x) + (ry + gm.y) * w;
        preV[r] = (double)img[idx];
        preOk[r] = !(mask[idx] > 0 || fabs(preV[r]) <= 1e-10);
      }
    }
    int cnt = 0, iter = 0;
    while(cnt < NSAMPLES && iter < numPix) {
      int b = min(32, numPix - iter);
      int idx = 0;
      const int round = iter / 32;
      if(draws && round < PRE) {
        // taken from preV / preOk below
      } else if(draws) {
        if(lane < b) {
          const int rx = (int)floor(draws[2 * (iter + lane)] * (int)gm.z);
          const int ry = (int)floor(draws[2 * (iter + lane) + 1] * (int)gm.w);
          idx = (rx + gm.x) + (ry + gm.y) * w;
        }
      } else {
        if(lane == 0) {
          for(int k = 0; k < b; k++) {
            int rx = (int)floor(rng.next(rtab) * (int)gm.z);
            int ry = (int)floor(rng.next(rtab) * (int)gm.w);
            cand[k] = (rx + gm.x) + (ry + gm.y) * w;
          }
        }
        __syncwarp();
        if(lane < b) idx = cand[lane];
      }
      bool ok = false;
      double v = 0.0;
      if(draws && round < PRE) {
        v = round == 0 ? preV[0] : round == 1 ? preV[1] : round == 2 ? preV[2] : preV[3];
        ok = round == 0 ? preOk[0] : round == 1 ? preOk[1] : round == 2 ? preOk[2] : preOk[3];
      } else if(lane < b) {
        v = (double)img[idx];
        ok = !(mask[idx] > 0 || fabs(v) <= 1e-10);
      }
      unsigned bal = __ballot_sync(0xffffffffu, ok);
      int pos = cnt + __popc(bal & ((1u << lane) - 1u));
      if(ok && pos < NSAMPLES) samples[pos] = v;
      cnt = min(NSAMPLES, cnt + __popc(bal));
      iter += b;
      __syncwarp();
    }
    if(lane == 0) sCount = cnt;
    __syncwarp();
    for(int i = lane; i < PADDED; i += 32)
      if(i >= cnt) samples[i] = i < NSAMPLES ? 0.0 : INFINITY;
    __syncwarp();
    // bitonic network of the 28 host-launched sortSamples passes
    for(int k = 2; k <= PADDED; k <<= 1)
      for(int j = k >> 1; j > 0; j >>= 1) {
        for(int i = lane; i < PADDED; i += 32) {
          int ixj = i ^ j;
          if(ixj > i) {
            double a = samples[i], c = samples[ixj];
            if((i & k) == 0 && a > c) {
              samples[i] = c;
              samples[ixj] = a;
            } else if((i & k) != 0 && a < c) {
              samples[i] = c;
              samples[ixj] = a;
            }
          }
        }
        __syncwarp();
      }
  }
  __syncthreads();

  // ---- phase B: ordered compaction of good pixels (maskStamp) ----
  // warp w owns a contiguous range of the stamp's pixel indices and reads it
  // 32 consecutive pixels at a time; ballots keep the ascending order inside
  // the warp and one block scan over the warp totals orders the warps.  The
  // good pixels are kept as read (FP32 pixels stay FP32).
  // The list is stored chunk-interleaved: entry q (chunk q/32, position
  // q%32) at slot(q), so that the chunk passes, one chunk per thread, read
  // 32 consecutive chunks' entries at one position with one coalesced load.
  // A stamp's slice is fSW^2 rounded up to a multiple of 1024 (statsSlice).
  T* gd = good + (size_t)s * statsSlice(fSW);
  uint8_t* cl = clip + (size_t)s * statsSlice(fSW);
  const int nPixS = fSW * fSW;
  constexpr int NWARP = ST_THREADS / 32;
  const int perW = ((nPixS + NWARP - 1) / NWARP + 31) & ~31;
  const int w0 = min(warp * perW, nPixS), w1 = min(w0 + perW, nPixS);
  // v <= 1e-10 of the reference: for an FP32 pixel the same test as f <= fTiny,
  // the largest float not above 1e-10
  const float fTiny = __double2float_rd(1e-10);
  auto tiny = [&](T v) -> bool {
    if(F32) return (float)v <= fTiny;
    return (double)v <= 1e-10;
  };
  auto pixelAt = [&](int idxS, size_t* id) -> bool {
    const int xI = idxS % fSW + gm.x, yI = idxS / fSW + gm.y;
    *id = (size_t)xI + (size_t)yI * w;
    return xI < w && yI < h;
  };
  // each pass loads BB rows of 32 pixels (and their mask words) before it
  // tests them, in order
  constexpr int BB = 8;
  int wGood = 0;
  for(int b0 = w0; b0 < w1; b0 += 32 * BB) {
    T px[BB];
    uint16_t mk[BB];
    size_t ids[BB];
    bool in[BB];
#pragma unroll
    for(int u = 0; u < BB; u++) {
      const int idxS = b0 + u * 32 + lane;
      in[u] = idxS < w1 && pixelAt(idxS, &ids[u]);
      px[u] = in[u] ? img[ids[u]] : T(0);
      mk[u] = in[u] ? mask[ids[u]] : (uint16_t)1;
    }
#pragma unroll
    for(int u = 0; u < BB; u++) {
      bool g = false;
      if(in[u] && !(mk[u] > 0 || tiny(px[u]))) {
        if(isnan(px[u])) mask[ids[u]] |= NAN_PIXEL | BAD_INPUT;
        else g = true;
      }
      wGood += __popc(__ballot_sync(0xffffffffu, g));
    }
  }
  const int wBase = blockScanExcl(lane == 0 ? wGood : 0, warpTot, &sTotal);
  const int nGood = sTotal;
  int pos = __shfl_sync(0xffffffffu, wBase, 0);
  for(int b0 = w0; b0 < w1; b0 += 32 * BB) {
    T px[BB];
    uint16_t mk[BB];
    bool in[BB];
#pragma unroll
    for(int u = 0; u < BB; u++) {
      const int idxS = b0 + u * 32 + lane;
      size_t id;
      in[u] = idxS < w1 && pixelAt(idxS, &id);
      px[u] = in[u] ? img[id] : T(0);
      mk[u] = in[u] ? mask[id] : (uint16_t)1;  // NaN pixels carry their mask bits now
    }
#pragma unroll
    for(int u = 0; u < BB; u++) {
      const bool g = in[u] && !(mk[u] > 0 || tiny(px[u]));
      const unsigned bal = __ballot_sync(0xffffffffu, g);
      if(g) {
        const int q = pos + __popc(bal & ((1u << lane) - 1u));
        gd[listSlot(q)] = px[u];
        cl[listSlot(q)] = 0;
      }
      pos += __popc(bal);
    }
  }

  // ---- phase C: sigma clip, maxIter 3 (bachUtil.cpp:34-128) ----
  // the chunk sums, in shared memory when they fit
  __shared__ double chunkSm[2][ST_CHUNKS_SMEM];
  const bool chunksInSmem = (nGood + 31) / 32 <= ST_CHUNKS_SMEM;
  double* cS = chunksInSmem ? chunkSm[0] : chunkBuf + (size_t)s * 2 * maxChunks;
  double* cS2 = chunksInSmem ? chunkSm[1] : cS + maxChunks;
  if(tid == 0) {
    sPrev = nGood;
    sCurr = 0;
    sDone = 0;
    sMean = 0.0;
    sStd = 1e10;
    if(nGood == 0) sDone = 1;
  }
  __syncthreads();
  const int nChunks = (nGood + 31) / 32;
  // exact clip thresholds for (m, inv) into tLo/tHi (warp 0; all threads call)
  // (warp 0 searches the upper edge, warp 1 the lower one)
  auto thresholds = [&](double m, double inv) {
    if(warp < 2) {
      const bool direct = !isfinite(m) || isnan(inv);
      if(!direct) {
        bool none;
        const unsigned long long k = clipEdge(m, inv, sigClipAlpha, warp == 0, &none);
        if(lane == 0) {
          const double t = keyD(k);
          if(warp == 0) {
            tHi = t;
            fHi = __double2float_ru(t);  // f >= tHi  <=>  f >= fHi for a float f
            tNoHi = none;
          } else {
            tLo = t;
            fLo = __double2float_rd(t);
            tNoLo = none;
          }
        }
      }
      if(warp == 0 && lane == 0) tDirect = direct;
    }
    __syncthreads();
  };
  auto isClipped = [&](double v, double m, double inv) -> bool {
    if(tDirect) return clipOut(v, m, inv, sigClipAlpha);
    if(F32) {
      const float f = (float)v;  // exact: v came from a float pixel
      return (!tNoHi && f >= fHi) || (!tNoLo && f <= fLo);
    }
    return (!tNoHi && v >= tHi) || (!tNoLo && v <= tLo);
  };
  // the same for a pixel as read (no FP64 conversion for FP32 pixels)
  auto isClippedPix = [&](T pv, double m, double inv) -> bool {
    if(tDirect) return clipOut((double)pv, m, inv, sigClipAlpha);
    if(F32) {
      const float f = (float)pv;
      return (!tNoHi && f >= fHi) || (!tNoLo && f <= fLo);
    }
    return isClipped((double)pv, m, inv);
  };
  // chunk sums of the unclipped pixels: 32 consecutive good pixels each, in
  // order (all pixels at first; then fused with each round's clip pass, for
  // the next round).  A chunk's pixels and flags are loaded before its sums
  // start; entries past the list's end count as clipped (adding 0.0 leaves a
  // sum unchanged).
  // sums of a chunk's unclipped pixels, 16 loads issued at a time
  auto chunkSums = [&](int c, int lc, bool all) {
    double a = 0.0, a2 = 0.0;
#pragma unroll
    for(int h = 0; h < 32; h += 16) {
      T v[16];
      bool on[16];
#pragma unroll
      for(int l = 0; l < 16; l++) {
        const int at = chunkSlot(c, h + l);
        on[l] = h + l < lc && (all || cl[at] == 0);
        v[l] = h + l < lc ? gd[at] : T(0);
      }
#pragma unroll
      for(int l = 0; l < 16; l++) {
        const double d = on[l] ? (double)v[l] : 0.0;
        a += d;
        a2 += d * d;
      }
    }
    cS[c] = a;
    cS2[c] = a2;
  };
  for(int c = tid; c < nChunks; c += ST_THREADS) chunkSums(c, min(32, nGood - c * 32), true);
  for(int it = 0; it < 3; it++) {
    if(sDone || sCurr == sPrev) break;
    if(sPrev <= 1) {
      if(tid == 0) {
        sMean = 0.0;
        sStd = 1e10;
      }
      break;
    }
    __syncthreads();
    if(tid == 0) sCurr = sPrev;
    __syncthreads();
    // the two sequential chunk sums (the reference's serial FP64 loops, bit
    // for bit) on two warps
    if(warp == 0) {
      const double sum = osum::warpOrderedSum(cS, nChunks);
      if(lane == 0) sSum = sum;
    } else if(warp == 1) {
      const double sum2 = osum::warpOrderedSum(cS2, nChunks);
      if(lane == 0) sSum2 = sum2;
    }
    __syncthreads();
    if(tid == 0) {
      const double sum = sSum, sum2 = sSum2;
      double n = (double)sCurr;
      double m = sum / n;
      double sd = sqrt((sum2 - n * m * m) / (double)(sCurr - 1));
      sMean = m;
      sStd = sd;
      sInv = 1.0 / sd;
      sClip = 0;
    }
    __syncthreads();
    const double m = sMean, inv = sInv;
    thresholds(m, inv);
    int myClip = 0;
    for(int c = tid; c < nChunks; c += ST_THREADS) {
      const int lc = min(32, nGood - c * 32);
      // a chunk none of whose pixels is clipped in this round keeps its sums
      // (the same terms in the same order)
      bool changed = false;
#pragma unroll
      for(int h = 0; h < 32; h += 16) {
        T v[16];
        uint8_t fl[16];
#pragma unroll
        for(int l = 0; l < 16; l++) {
          v[l] = h + l < lc ? gd[chunkSlot(c, h + l)] : T(0);
          fl[l] = h + l < lc ? cl[chunkSlot(c, h + l)] : (uint8_t)1;
        }
#pragma unroll
        for(int l = 0; l < 16; l++) {
          if(fl[l] == 0 && isClippedPix(v[l], m, inv)) {
            cl[chunkSlot(c, h + l)] = 1;
            myClip++;
            changed = true;
          }
        }
      }
      if(changed) chunkSums(c, lc, false);
    }
    if(myClip) atomicAdd(&sClip, myClip);
    __syncthreads();
    if(tid == 0) sPrev = sCurr - sClip;
    __syncthreads();
  }
  __syncthreads();
  const double mean = sMean, invStd = 1.0 / sStd;
  thresholds(mean, invStd);

  // ---- phase D: histogram sky / robust sigma (sss.cl:190-324) ----
  if(tid == 0) {
    int sc = sCount;
    double upS = samples[(int)(0.9 * sc)];
    double midS = samples[(int)(0.5 * sc)];
    hBinSize = (upS - midS) / (double)NSAMPLES;
    hLowerBinVal = midS - (128.0 * hBinSize);
    hLower = hUpper = hSky = 0.0;
    hState = 0;
  }
  __syncthreads();
  for(int attempts = 0;; attempts++) {
    if(attempts >= 5) {
      if(tid == 0) hState = 2;
      break;
    }
    for(int i = tid; i < 256; i += ST_THREADS) bins[i] = 0;
    if(tid == 0) {
      okCount = 0;
      // FP32 estimate q' of q = (v - lbv) / bs: |q' - q| <= delta for |q| <= 512
      // (lbv and 1/bs rounded to float, one FP32 rounding each in the
      // subtraction and the product; the FP64 q itself is within 2^-51 |q|)
      const double lbv = hLowerBinVal, bs = hBinSize;
      const double delta = fabs(lbv) / bs * 0x1p-23 + 512.0 * 0x1p-21;
      const bool ok = F32 && bs > 0.0 && isfinite(bs) && isfinite(lbv) && delta < 0.125;
      bExact = ok ? 0 : 1;
      bLbv = (float)lbv;
      bInv = (float)(1.0 / bs);
      bDelta = (float)delta;
    }
    __syncthreads();
    const double lbv = hLowerBinVal, bs = hBinSize;
    const bool exactAll = bExact != 0;
    const float fl = bLbv, fi = bInv, fd = bDelta;
    int myOk = 0;
    // the pixels of createHistogram (mask 0, above 1e-10, not clipped) are
    // the good list of phase B (the kernel changes no other mask bit of the
    // stamp) less the final clip; a warp-uniform trip count lets the lanes of
    // a warp that land in the same bin (most pixels sit in a few sky bins)
    // add to it with one atomic
    constexpr int HB = 8;  // list entries loaded ahead per thread
    // (the counts do not depend on the order: the slots are read in storage
    // order, coalesced, each standing for list entry listEntry(slot))
    const int nSlots = (nGood + 1023) & ~1023;
    for(int base0 = 0; base0 < nSlots; base0 += ST_THREADS * HB) {
      T pvs[HB];
      bool in[HB];
#pragma unroll
      for(int u = 0; u < HB; u++) {
        const int k = base0 + u * ST_THREADS + tid;
        in[u] = k < nSlots && listEntry(k) < nGood;
        pvs[u] = in[u] ? gd[k] : T(0);
      }
#pragma unroll
      for(int u = 0; u < HB; u++) {
        int index = -1;
        if(in[u]) {
          const T pv = pvs[u];
          if(!isClippedPix(pv, mean, invStd)) {
            if(!exactAll) {
              const float q = ((float)pv - fl) * fi;
              if(q > 300.f) {
                index = 255;
              } else if(q < -50.f) {
                index = 0;
              } else {
                const float f0 = floorf(q), fr = q - f0;
                if(fr > fd && fr < 1.f - fd) index = min(max((int)f0 + 1, 0), 255);
              }
            }
            if(index < 0) {
              const double v = (double)pv;
              index = satFloorToInt((v - lbv) / bs);
              index = index == INT_MAX ? INT_MAX : index + 1;
              index = min(max(index, 0), 255);
            }
          }
        }
        const unsigned grp = __match_any_sync(0xffffffffu, index);
        if(index >= 0) {
          myOk++;
          if(lane == __ffs(grp) - 1) atomicAdd(&bins[index], __popc(grp));
        }
      }
    }
    if(myOk) atomicAdd(&okCount, myOk);
    __syncthreads();
    if(warp == 0) {
      const int ok = okCount;
      const double binSize = hBinSize, lowerBinVal = hLowerBinVal;
      if(ok == 0 || binSize == 0.0) {
        if(lane == 0) hState = 2;
      } else {
        // The reference walks the bins serially (createHistogram,
        // sss.cl:190-324); every quantity it forms is a prefix sum of the
        // counts, so one warp scans the 256 bins once and finds each walk's
        // stopping point by binary search.
        // The running sums of bin counts (sumBins, sumExpect) are FP64 in the
        // reference but hold integers below 2^53, so they are int64 here;
        // S < x for an integer S and a double x is S < ceil(x).
        long long c8[8], e8[8], tc = 0, te = 0;
#pragma unroll
        for(int k = 0; k < 8; k++) {
          const int i = 8 * lane + k;
          tc += bins[i];
          te += (long long)i * bins[i];
          c8[k] = tc;
          e8[k] = te;
        }
        long long pc = tc, pe = te;  // inclusive scan of the lane totals
#pragma unroll
        for(int o = 1; o < 32; o <<= 1) {
          const long long uc = __shfl_up_sync(0xffffffffu, pc, o);
          const long long ue = __shfl_up_sync(0xffffffffu, pe, o);
          if(lane >= o) {
            pc += uc;
            pe += ue;
          }
        }
#pragma unroll
        for(int k = 0; k < 8; k++) {  // hC[i] = sum of bins[0..i), hCE[i] = sum of j * bins[j]
          hC[8 * lane + k + 1] = pc - tc + c8[k];
          hCE[8 * lane + k + 1] = pe - te + e8[k];
        }
        if(lane == 0) hC[0] = hCE[0] = 0;
        __syncwarp();
        const long long tenth = (long long)ceil(ok / 10.0);
        // first i in [lo, hi] with hC[i] >= target, hi when none
        auto firstAtLeast = [&](int lo, int hi, long long target) {
          while(lo < hi) {
            const int mid = (lo + hi) >> 1;
            if(hC[mid] >= target) hi = mid;
            else lo = mid + 1;
          }
          return lo;
        };
        // Densest run of bins holding a tenth of the pixels: the serial
        // window for lower index L ends at U(L) = the first U in [L+1, 255]
        // with hC[U] - hC[L] >= tenth (255 when none; U(L) never decreases,
        // so this is where the two-pointer walk stands), and the walk visits
        // L = 1, 2, ... while the previous window ended below 255.  The
        // reference compares the FP64 quotients S / (U - L); both are integer
        // over integer (sums of counts < 2^31, widths 1..254), and two
        // different such fractions differ by more than 2^-47 relative, so
        // their correctly rounded quotients compare like the fractions:
        // S / D > S' / D'  <=>  S * D' > S' * D, exact in 64-bit integers.
        // The walk keeps the first L of the largest density (strict >), from
        // maxDens = 0.
        long long bN = 0, bD = 1;
        int bL = -1;
        for(int L = 1 + lane; L <= 254; L += 32) {
          if(L > 1 && firstAtLeast(L, 255, hC[L - 1] + tenth) >= 255) continue;
          const int U = firstAtLeast(L + 1, 255, hC[L] + tenth);
          const long long S = hC[U] - hC[L], D = U - L;
          if(S * bD > bN * D) {
            bN = S;
            bD = D;
            bL = L;
          }
        }
#pragma unroll
        for(int o = 16; o > 0; o >>= 1) {
          const long long oN = __shfl_xor_sync(0xffffffffu, bN, o);
          const long long oD = __shfl_xor_sync(0xffffffffu, bD, o);
          const int oL = __shfl_xor_sync(0xffffffffu, bL, o);
          const long long lhs = oN * bD, rhs = bN * oD;
          if(oL >= 0 && (bL < 0 || lhs > rhs || (lhs == rhs && oL < bL))) {
            bN = oN;
            bD = oD;
            bL = oL;
          }
        }
        if(lane == 0) {
          const int maxIndex = bL < 0 ? 0 : bL;
          // the mode's walk from maxIndex adds bins while below a tenth
          const int iEnd = firstAtLeast(maxIndex + 1, 255, hC[maxIndex] + tenth);
          const long long S = hC[iEnd] - hC[maxIndex], E = hCE[iEnd] - hCE[maxIndex];
          double modeBin = (double)E / (double)S + 0.5;
          double skyEst = lowerBinVal + binSize * (modeBin - 1.0);
          double lower = ok * 0.25, upper = ok * 0.75;
          const long long lowerCeil = (long long)ceil(lower), upperCeil = (long long)ceil(upper);
          // the quartile walks from bin 0 (hC[256] = ok bounds both)
          const int i1 = firstAtLeast(0, 256, lowerCeil);
          lower = i1 - ((double)hC[i1] - lower) / bins[i1 - 1];
          const int i2 = firstAtLeast(i1, 256, upperCeil);
          upper = i2 - ((double)hC[i2] - upper) / bins[i2 - 1];
          hSky = skyEst;
          hLower = lower;
          hUpper = upper;
          if(lower < 1.0 || upper > 255.0) {
            hLowerBinVal = lowerBinVal - 128.0 * binSize;
            hBinSize = binSize * 2;
          } else if(upper - lower < 40.0) {
            hBinSize = binSize / 3.0;
            hLowerBinVal = skyEst - 128.0 * hBinSize;
          } else {
            hState = 1;
          }
        }
      }
    }
    __syncthreads();
    if(hState != 0) break;
  }
  if(tid == 0) {
    fwhmOut[s] = hState == 1 ? hBinSize * (hUpper - hLower) / iqRange : 0.0;
    skyOut[s] = hSky;
  }
}

// Mask access shared by the substamp search: volatile 16-bit loads (other
// CTAs of the same launch may set SKIP bits nearby) and a 16-bit OR done as a
// 32-bit atomic on the containing word (the mask buffer has 2 spare entries).
__device__ __forceinline__ uint16_t ldMask(const uint16_t* m, size_t i) {
  return *((volatile const uint16_t*)m + i);
}
__device__ __forceinline__ void orMask(uint16_t* m, size_t i, uint16_t bits) {
  uintptr_t a = (uintptr_t)(m + i);
  unsigned* w32 = (unsigned*)(a & ~(uintptr_t)3);
  unsigned sh = (a & 2) ? 16u : 0u;
  atomicOr(w32, (unsigned)bits << sh);
}

// ---------------------------------------------------------- substamp search --
// One CTA per (stamp, image): findSubStamps (cl_kern/sss.cl:381-505).  The
// reference scans the stamp in raster order, testing each pixel.  Between two
// accepted substamps the mask does not change, so for every pixel of the stamp window
// the reference's local-maximum search (sss.cl:427-459) and window check
// (checkSStamp, :326-361) are tabulated once per mask state:
//   * a separable sliding-window argmax over the qualifying pixels (largest
//     value, ties to the first pixel in raster order: row pass keeps the
//     smallest x, column pass the smallest y), keys compared as the bit
//     patterns of positive doubles;
//   * separable window ORs of "bad", "above kernel-fit threshold" and "above
//     threshold but not positive".
// Each pass then looks for the first candidate in raster order whose window
// passes, in parallel; the scan before it changes nothing, and after an
// acceptance the maps are rebuilt and the scan resumes at the next pixel.
// The accepted substamp's value is the sequential sum of sss.cl:354-357; for
// FP32 input every summand is a float, all partial sums are exact in FP64
// whenever sum|v| < 2^52 * (quantum of the smallest |v|), which is checked,
// and then a parallel sum is the same number.  The reference's writes of the
// bad-pixel bit for pixels above threshHigh (sss.cl:349-352, :417-420,
// :445-448) are unreachable: such pixels carry BAD_INPUT from maskInput
// (ini.cl:29), which every badMask contains, and that test comes first.
constexpr int FM_THREADS = 256;
enum : uint8_t { FL_PRED = 1, FL_NONPOS = 2, FL_KFQ = 4, FL_VPOS = 8 };
enum : uint8_t { OK_BAD = 1, OK_PRED = 2, OK_NONPOS = 4 };


// Bad map and keys of the whole stamp from the mask (the search's start).
template <class T>
__device__ void fmInit(const T* img, const uint16_t* mask, int w, int cx, int cy, int n,
                       uint16_t badMask, const uint8_t* flags, uint8_t* bad,
                       unsigned long long* key) {
  const int N = n * n, tid = threadIdx.x;
  for(int p = tid; p < N; p += FM_THREADS) {
    const int lx = p % n, ly = p / n;
    const size_t a = (size_t)(cx + lx) + (size_t)(cy + ly) * w;
    const uint8_t b = (ldMask(mask, a) & badMask) ? 1 : 0;
    bad[p] = b;
    const uint8_t f = flags[p];
    key[p] = (!b && (f & FL_KFQ) && (f & FL_VPOS))
                 ? (unsigned long long)__double_as_longlong((double)img[a]) : 0ull;
  }
  __syncthreads();
}

// Window maps over the columns [x0, x1] of the rows [k0, k1] (row maps) and
// [r0, r1] (column maps), by the block scans of k_find_substamps_sm (van
// Herk / Gil-Werman: prefix and suffix argmax / OR within blocks of the window
// width; ties keep the smaller index), with 16-bit indices for stamps up to
// 2048 pixels wide.
__device__ void fmMaps(int n, int sx, int sy, int hSS, const uint8_t* flags, const uint8_t* bad,
                       const unsigned long long* key, unsigned short* hx, uint8_t* rowf, int* arg,
                       uint8_t* okw, unsigned short* tPA, unsigned short* tSA, uint8_t* tPO,
                       uint8_t* tSO, int x0, int x1, int k0, int k1, int r0, int r1) {
  const int tid = threadIdx.x, W = 2 * hSS + 1;
  constexpr unsigned short NONE = 0xFFFF;
  auto orAt = [&](int p) -> uint8_t {
    const uint8_t fl = flags[p];
    return (bad[p] ? OK_BAD : 0) | ((fl & FL_PRED) ? OK_PRED : 0) | ((fl & FL_NONPOS) ? OK_NONPOS : 0);
  };
  const int kw = x1 - x0 + 1;
  {
    const int ba = max(x0 - hSS, 0) / W, bb = min(x1 + hSS, n - 1) / W;
    const int nr = k1 - k0 + 1, nTask = nr * (bb - ba + 1);
    for(int t = tid; t < 2 * nTask; t += FM_THREADS) {
      const bool suffix = t >= nTask;
      const int tt = suffix ? t - nTask : t;
      const int ly = k0 + tt % nr, blk = ba + tt / nr;
      const size_t row = (size_t)ly * n;
      const int b0 = blk * W, b1 = min(b0 + W - 1, n - 1);
      unsigned long long bk = 0;
      unsigned short bi = NONE;
      uint8_t o = 0;
      if(!suffix) {
        for(int x = b0; x <= b1; x++) {
          const unsigned long long k = key[row + x];
          if(k > bk) {
            bk = k;
            bi = (unsigned short)x;
          }
          if(x < sx) o |= orAt((int)(row + x));
          tPA[row + x] = bi;
          tPO[row + x] = o;
        }
      } else {
        for(int x = b1; x >= b0; x--) {
          const unsigned long long k = key[row + x];
          if(k != 0 && k >= bk) {
            bk = k;
            bi = (unsigned short)x;
          }
          if(x < sx) o |= orAt((int)(row + x));
          tSA[row + x] = bi;
          tSO[row + x] = o;
        }
      }
    }
  }
  __syncthreads();
  for(int i = tid; i < (k1 - k0 + 1) * kw; i += FM_THREADS) {
    const int ly = k0 + i / kw, lx = x0 + i % kw;
    const size_t row = (size_t)ly * n;
    const int a = max(lx - hSS, 0), b = min(lx + hSS, n - 1);
    unsigned short h;
    uint8_t o;
    if(a / W != b / W) {
      const unsigned short L = tSA[row + a], R = tPA[row + b];
      h = L == NONE ? R : R == NONE ? L : (key[row + R] > key[row + L] ? R : L);
      o = tSO[row + a] | tPO[row + b];
    } else if(a % W == 0) {
      h = tPA[row + b];
      o = tPO[row + b];
    } else {
      h = tSA[row + a];
      o = tSO[row + a];
    }
    hx[row + lx] = h;
    rowf[row + lx] = o;
  }
  __syncthreads();
  {
    auto candKey = [&](int y, int lx) -> unsigned long long {
      const unsigned short xx = hx[(size_t)y * n + lx];
      return xx == NONE ? 0ull : key[(size_t)y * n + xx];
    };
    const int ba = max(r0 - hSS, 0) / W, bb = min(r1 + hSS, n - 1) / W;
    const int nTask = kw * (bb - ba + 1);
    for(int t = tid; t < 2 * nTask; t += FM_THREADS) {
      const bool suffix = t >= nTask;
      const int tt = suffix ? t - nTask : t;
      const int lx = x0 + tt % kw, blk = ba + tt / kw;
      const int b0 = blk * W, b1 = min(b0 + W - 1, n - 1);
      unsigned long long bk = 0;
      unsigned short bi = NONE;
      uint8_t o = 0;
      if(!suffix) {
        for(int y = b0; y <= b1; y++) {
          const unsigned long long k = candKey(y, lx);
          if(k > bk) {
            bk = k;
            bi = (unsigned short)y;
          }
          if(y < sy) o |= rowf[(size_t)y * n + lx];
          tPA[(size_t)y * n + lx] = bi;
          tPO[(size_t)y * n + lx] = o;
        }
      } else {
        for(int y = b1; y >= b0; y--) {
          const unsigned long long k = candKey(y, lx);
          if(k != 0 && k >= bk) {
            bk = k;
            bi = (unsigned short)y;
          }
          if(y < sy) o |= rowf[(size_t)y * n + lx];
          tSA[(size_t)y * n + lx] = bi;
          tSO[(size_t)y * n + lx] = o;
        }
      }
    }
    __syncthreads();
    for(int i = tid; i < (r1 - r0 + 1) * kw; i += FM_THREADS) {
      const int ly = r0 + i / kw, lx = x0 + i % kw;
      const int a = max(ly - hSS, 0), b = min(ly + hSS, n - 1);
      unsigned short yb;
      uint8_t o;
      if(a / W != b / W) {
        const unsigned short L = tSA[(size_t)a * n + lx], R = tPA[(size_t)b * n + lx];
        yb = L == NONE ? R : R == NONE ? L : (candKey(R, lx) > candKey(L, lx) ? R : L);
        o = tSO[(size_t)a * n + lx] | tPO[(size_t)b * n + lx];
      } else if(a % W == 0) {
        yb = tPA[(size_t)b * n + lx];
        o = tPO[(size_t)b * n + lx];
      } else {
        yb = tSA[(size_t)a * n + lx];
        o = tSO[(size_t)a * n + lx];
      }
      arg[(size_t)ly * n + lx] = yb == NONE ? -1 : yb * n + hx[(size_t)yb * n + lx];
      okw[(size_t)ly * n + lx] = o;
    }
  }
  __syncthreads();
}

template <class T>
__global__ void __launch_bounds__(FM_THREADS)
    k_find_substamps_maps(const T* __restrict__ img0, const T* __restrict__ img1,
                          uint16_t* __restrict__ mask, const int4* __restrict__ geom,
                          const double* __restrict__ sky0, const double* __restrict__ fwhm0,
                          const double* __restrict__ sky1, const double* __restrict__ fwhm1,
                          int2* __restrict__ xy0, double* __restrict__ val0, int* __restrict__ cnt0,
                          int2* __restrict__ xy1, double* __restrict__ val1, int* __restrict__ cnt1,
                          int w, int fSW, int hSS, int maxSS, double tH, double tKF,
                          unsigned char* __restrict__ scratch, size_t perCta, int floatInput) {
  const int s = blockIdx.x, im = blockIdx.y, tid = threadIdx.x;
  const T* img = im == 0 ? img0 : img1;
  const double sky = im == 0 ? sky0[s] : sky1[s];
  const double fwhm = im == 0 ? fwhm0[s] : fwhm1[s];
  int2* xyOut = (im == 0 ? xy0 : xy1) + (size_t)s * maxSS;
  double* valOut = (im == 0 ? val0 : val1) + (size_t)s * maxSS;
  const uint16_t badMask =
      (uint16_t)((MASK_ALL & ~OK_CONV) & ~(im == 0 ? (BAD_PIXEL_S | SKIP_S) : (BAD_PIXEL_T | SKIP_T)));
  const uint16_t skipMask = im == 0 ? SKIP_T : SKIP_S;
  const int4 gm = geom[s];
  const int cx = gm.x, cy = gm.y, sx = gm.z, sy = gm.w, n = fSW, N = n * n;
  const double invFwhm = 1.0 / fwhm;
  unsigned char* base = scratch + (size_t)(im * gridDim.x + s) * perCta;
  unsigned long long* key = (unsigned long long*)base;  // N
  int* arg = (int*)(key + N);                           // N
  unsigned short* hx = (unsigned short*)(arg + N);      // N
  uint8_t* flags = (uint8_t*)(hx + N);                  // N
  uint8_t* bad = flags + N;                             // N
  uint8_t* rowf = bad + N;                              // N
  uint8_t* okw = rowf + N;                              // N
  unsigned short* tPA = (unsigned short*)(okw + N);     // N (block scans of fmMaps)
  unsigned short* tSA = tPA + N;                        // N
  uint8_t* tPO = (uint8_t*)(tSA + N);                   // N
  uint8_t* tSO = tPO + N;                               // N
  __shared__ int2 locXY[MAX_MAXSS];
  __shared__ double locVal[MAX_MAXSS];
  __shared__ int sBest;
  __shared__ double rA[FM_THREADS / 32], rB[FM_THREADS / 32];
  __shared__ double sSum;
  // static flags: checkSStamp predicate, kernel-fit qualification, v > 0
  for(int p = tid; p < N; p += FM_THREADS) {
    const double v = (double)img[(size_t)(cx + p % n) + (size_t)(cy + p / n) * w];
    uint8_t f = 0;
    const bool pr = (v - sky) / fwhm > tKF;
    if(pr) f |= FL_PRED;
    if(pr && !(v > 0.0)) f |= FL_NONPOS;
    if(!((v - sky) * invFwhm < tKF)) f |= FL_KFQ;
    if(v > 0.0) f |= FL_VPOS;
    flags[p] = f;
  }
  __syncthreads();
  fmInit(img, mask, w, cx, cy, n, badMask, flags, bad, key);
  fmMaps(n, sx, sy, hSS, flags, bad, key, hx, rowf, arg, okw, tPA, tSA, tPO, tSO, 0, n - 1, 0,
         n - 1, 0, n - 1);
  const double floorV = sky + tKF * fwhm;
  double dfrac = 0.9;
  int cnt = 0, passes = 0;
  while(cnt < maxSS && passes < 256) {
    passes++;
    const double alt = sky + (tH - sky) * dfrac;
    const double lim = floorV < alt ? alt : floorV;  // OpenCL max()
    int start = 0;
    while(cnt < maxSS && start < N) {
      // first candidate >= start whose window passes (or needs the exact sum)
      int mine = INT_MAX;
      for(int p0 = start; p0 < N && mine == INT_MAX; p0 += 4 * FM_THREADS) {
        for(int k = 0; k < 4; k++) {
          const int p = p0 + k * FM_THREADS + tid;
          if(p >= N || p >= mine) break;
          if(bad[p] || !(flags[p] & FL_KFQ)) continue;
          const double v = (double)img[(size_t)(cx + p % n) + (size_t)(cy + p / n) * w];
          if(!(v > lim)) continue;
          const int m = arg[p] >= 0 ? arg[p] : p;
          const uint8_t o = okw[m];
          if(!(o & OK_BAD) && (o & OK_PRED)) {
            mine = p;
            break;
          }
        }
        mine = __reduce_min_sync(0xffffffffu, mine);
        if(tid == 0) sBest = INT_MAX;
        __syncthreads();
        if((tid & 31) == 0 && mine != INT_MAX) atomicMin(&sBest, mine);
        __syncthreads();
        mine = sBest;
        __syncthreads();
      }
      if(mine == INT_MAX) break;
      const int p = mine, m = arg[p] >= 0 ? arg[p] : p;
      const int mx = cx + m % n, my = cy + m / n;
      const int u0 = max(mx - hSS, cx), v0 = max(my - hSS, cy);
      const int u1 = min(mx + hSS, cx + sx - 1), v1 = min(my + hSS, cy + sy - 1);
      const int uw = u1 - u0 + 1, un = uw * (v1 - v0 + 1);
      // value of the substamp: sum of the thresholded pixels in raster order
      double part = 0.0, amin = INFINITY;
      for(int i = tid; i < un; i += FM_THREADS) {
        const int lx = u0 + i % uw - cx, ly = v0 + i / uw - cy;
        if(flags[ly * n + lx] & FL_PRED) {
          const double v = (double)img[(size_t)(cx + lx) + (size_t)(cy + ly) * w];
          part += v;
          amin = fmin(amin, fabs(v));
        }
      }
#pragma unroll
      for(int o = 16; o > 0; o >>= 1) {
        part += __shfl_down_sync(0xffffffffu, part, o);
        amin = fmin(amin, __shfl_down_sync(0xffffffffu, amin, o));
      }
      if((tid & 31) == 0) {
        rA[tid >> 5] = part;
        rB[tid >> 5] = amin;
      }
      __syncthreads();
      if(tid == 0) {
        double t = 0.0, mn = INFINITY;
        for(int i = 0; i < FM_THREADS / 32; i++) {
          t += rA[i];
          mn = fmin(mn, rB[i]);
        }
        int exact = 0;
        if(floatInput && !(okw[m] & OK_NONPOS) && mn > 0.0 && mn < INFINITY) {
          int e;
          frexp(mn, &e);                           // mn in [2^(e-1), 2^e)
          const double quantum = ldexp(1.0, e - 1 - 23);
          exact = t < ldexp(quantum, 52) ? 1 : 0;  // t = sum|v| here (all v > 0)
        }
        if(!exact) {
          t = 0.0;
          for(int yy = v0; yy <= v1; yy++)
            for(int xx = u0; xx <= u1; xx++)
              if(flags[(yy - cy) * n + (xx - cx)] & FL_PRED) t += (double)img[(size_t)xx + (size_t)yy * w];
        }
        sSum = t;
      }
      __syncthreads();
      const double ret = sSum;
      start = p + 1;
      if(ret == 0.0) continue;
      if(tid == 0) {
        locXY[cnt] = make_int2(mx, my);
        locVal[cnt] = ret;
      }
      cnt++;
      // the window turns bad (its skip bit is part of this image's bad mask,
      // and no other CTA touches this image's bits of the stamp): keys inside
      // it vanish, and only maps within hSS of it can change
      for(int i = tid; i < un; i += FM_THREADS) {
        const int gx = u0 + i % uw, gy = v0 + i / uw;
        orMask(mask, (size_t)gx + (size_t)gy * w, skipMask);
        const size_t q = (size_t)(gx - cx) + (size_t)(gy - cy) * n;
        bad[q] = 1;
        key[q] = 0ull;
      }
      __syncthreads();
      if(cnt < maxSS) {
        const int a0 = u0 - cx, a1 = u1 - cx, b0 = v0 - cy, b1 = v1 - cy;
        fmMaps(n, sx, sy, hSS, flags, bad, key, hx, rowf, arg, okw, tPA, tSA, tPO, tSO,
               max(a0 - hSS, 0), min(a1 + hSS, n - 1), b0, b1, max(b0 - hSS, 0),
               min(b1 + hSS, n - 1));
      }
    }
    if(cnt >= maxSS || lim == floorV) break;
    dfrac -= 0.2;
  }
  __syncthreads();
  if(tid == 0) {
    for(int i = 1; i < cnt; i++)
      for(int j = i; j > 0 && locVal[j - 1] < locVal[j]; j--) {
        int2 t = locXY[j - 1];
        locXY[j - 1] = locXY[j];
        locXY[j] = t;
        double tv = locVal[j - 1];
        locVal[j - 1] = locVal[j];
        locVal[j] = tv;
      }
    for(int i = 0; i < maxSS; i++) {
      xyOut[i] = i < cnt ? locXY[i] : make_int2(INT_MAX, INT_MAX);
      valOut[i] = i < cnt ? locVal[i] : -INFINITY;
    }
    (im == 0 ? cnt0 : cnt1)[s] = min(cnt, maxSS / 2);
  }
}

// ------------------------------------------- substamp search in shared memory --
// The decisions of k_find_substamps_maps for FP32 images, with the stamp's
// pixels and every map in shared memory (15 B per pixel, one CTA per SM):
// keys are the float bit patterns (ordered like the doubles of the reference
// for positive values), the bad map is updated in place after an acceptance
// (the skip bit it sets is part of this image's bad mask, and no other CTA
// touches this image's bits of the stamp), and the two static predicates
// (v - sky) / fwhm > tKF and !((v - sky) * (1/fwhm) < tKF), monotone in v,
// become compares against their exact thresholds, found once per stamp by a
// warp search over the ordered doubles; so does the pass threshold v > lim.
constexpr int FS_T = 512;

// One warp: smallest key in (lo, hi] at which pred turns true, given
// pred(lo) false and pred(hi) true (pred monotone between them).
template <class P>
__device__ unsigned long long warpFirstTrue(unsigned long long lo, unsigned long long hi, P pred) {
  const int lane = threadIdx.x & 31;
  for(int guard = 0; guard < 40; guard++) {
    const unsigned long long span = hi - lo;
    if(span <= 1) break;
    unsigned long long step = span / 33;
    if(step == 0) step = 1;
    const unsigned long long off = (unsigned long long)(lane + 1) * step;
    const bool valid = off < span;
    const unsigned long long k = lo + off;
    const bool t = valid && pred(keyD(k));
    const unsigned bal = __ballot_sync(0xffffffffu, t);
    const unsigned vmask = __ballot_sync(0xffffffffu, valid);
    if(bal) {
      const int j = __ffs(bal) - 1;
      const unsigned long long kj = __shfl_sync(0xffffffffu, k, j);
      const unsigned long long kp = __shfl_sync(0xffffffffu, k, j > 0 ? j - 1 : 0);
      hi = kj;
      if(j > 0) lo = kp;
    } else {
      lo = __shfl_sync(0xffffffffu, k, 31 - __clz(vmask));
    }
  }
  return hi;
}

size_t fsSmemBytes(int n) { return (size_t)n * n * 15 + 64; }

__global__ void __launch_bounds__(FS_T, 1)
    k_find_substamps_sm(const float* __restrict__ img0, const float* __restrict__ img1,
                        uint16_t* __restrict__ mask, const int4* __restrict__ geom,
                        const double* __restrict__ sky0, const double* __restrict__ fwhm0,
                        const double* __restrict__ sky1, const double* __restrict__ fwhm1,
                        int2* __restrict__ xy0, double* __restrict__ val0, int* __restrict__ cnt0,
                        int2* __restrict__ xy1, double* __restrict__ val1, int* __restrict__ cnt1,
                        int w, int fSW, int hSS, int maxSS, double tH, double tKF) {
  extern __shared__ __align__(16) unsigned char fs_s[];
  const int s = blockIdx.x, im = blockIdx.y, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  constexpr int NW = FS_T / 32;
  const float* img = im == 0 ? img0 : img1;
  const double sky = im == 0 ? sky0[s] : sky1[s];
  const double fwhm = im == 0 ? fwhm0[s] : fwhm1[s];
  int2* xyOut = (im == 0 ? xy0 : xy1) + (size_t)s * maxSS;
  double* valOut = (im == 0 ? val0 : val1) + (size_t)s * maxSS;
  const uint16_t badMask =
      (uint16_t)((MASK_ALL & ~OK_CONV) & ~(im == 0 ? (BAD_PIXEL_S | SKIP_S) : (BAD_PIXEL_T | SKIP_T)));
  const uint16_t skipMask = im == 0 ? SKIP_T : SKIP_S;
  const int4 gm = geom[s];
  const int cx = gm.x, cy = gm.y, sx = gm.z, sy = gm.w, n = fSW, N = n * n;
  const double invFwhm = 1.0 / fwhm;
  float* V = (float*)fs_s;                 // N pixel values
  uint16_t* arg = (uint16_t*)(V + N);      // N (0xFFFF: none)
  uint8_t* flags = (uint8_t*)(arg + N);    // N
  uint8_t* bad = flags + N;                // N
  uint8_t* hx = bad + N;                   // N (0xFF: none)
  uint8_t* rowf = hx + N;                  // N
  uint8_t* okw = rowf + N;                 // N
  // block scans of the map build: prefix / suffix argmax (index in the row
  // or column, 0xFF: none) and prefix / suffix OR within blocks of the window
  // width
  uint8_t* tPA = okw + N;                  // N
  uint8_t* tSA = tPA + N;                  // N
  uint8_t* tPO = tSA + N;                  // N
  uint8_t* tSO = tPO + N;                  // N
  __shared__ int2 locXY[MAX_MAXSS];
  __shared__ double locVal[MAX_MAXSS];
  __shared__ int sBest;
  __shared__ double rA[NW], rB[NW];
  __shared__ double sSum;
  __shared__ float sfP, sfK, sfLim;
  __shared__ int sDirect;

  // warps 2.. load the stamp while warps 0 and 1 search the exact
  // thresholds of the two static predicates
  if(warp >= 2)
    for(int ly = warp - 2; ly < n; ly += NW - 2)
      for(int lx = lane; lx < n; lx += 32) {
        const size_t a = (size_t)(cx + lx) + (size_t)(cy + ly) * w;
        V[ly * n + lx] = img[a];
        bad[ly * n + lx] = (ldMask(mask, a) & badMask) ? 1 : 0;
      }
  if(warp < 2) {
    auto pr = [&](double v) { return (v - sky) / fwhm > tKF; };
    auto kq = [&](double v) { return !((v - sky) * invFwhm < tKF); };
    const bool direct = !(fwhm > 0.0 && isfinite(fwhm) && isfinite(sky) && isfinite(invFwhm) &&
                          pr(INFINITY) && !pr(-INFINITY) && kq(INFINITY) && !kq(-INFINITY));
    if(!direct) {
      const unsigned long long kLo = dKey(-INFINITY), kHi = dKey(INFINITY);
      if(warp == 0) {
        const unsigned long long kP = warpFirstTrue(kLo, kHi, pr);
        if(lane == 0) sfP = __double2float_ru(keyD(kP));  // pr(v) <=> v >= sfP for a float v
      } else {
        const unsigned long long kK = warpFirstTrue(kLo, kHi, kq);
        if(lane == 0) sfK = __double2float_ru(keyD(kK));
      }
    }
    if(warp == 0 && lane == 0) sDirect = direct;
  }
  __syncthreads();
  const bool direct = sDirect != 0;
  const float fP = sfP, fK = sfK;
  for(int p = tid; p < N; p += FS_T) {
    const float f = V[p];
    bool pr, kq;
    if(direct) {
      pr = ((double)f - sky) / fwhm > tKF;
      kq = !(((double)f - sky) * invFwhm < tKF);
    } else {
      pr = f >= fP;
      kq = isnan(f) || f >= fK;
    }
    const bool vpos = f > 0.f;
    uint8_t fl = 0;
    if(pr) fl |= FL_PRED;
    if(pr && !vpos) fl |= FL_NONPOS;
    if(kq) fl |= FL_KFQ;
    if(vpos) fl |= FL_VPOS;
    flags[p] = fl;
  }
  __syncthreads();
  // maps of the current bad state (window argmax of the keys, window ORs)
  // over the columns [x0, x1] of the rows [k0, k1] (row maps) and [r0, r1]
  // (column maps); the full build covers the stamp.  After an acceptance
  // only the accepted window's bad bits change, so only row maps within hSS
  // of it in x and column maps within hSS of it in x and y can change:
  // rebuilding that region gives the maps of a full rebuild.
  // A key is the float bit pattern of a qualifying pixel (0: none).  Window
  // argmax and OR use the van Herk / Gil-Werman scheme: split the line into
  // blocks of the window width W, scan each block forwards (prefix) and
  // backwards (suffix); the window [a, b] is then suffix(a) with prefix(b)
  // when they lie in different blocks, prefix(b) when a starts its block,
  // suffix(a) otherwise (b is then the line's end).  Ties keep the smaller
  // index: the prefix updates on a larger key, the suffix on a larger or
  // equal one, and prefix(b) wins only with a larger key.
  const int W = 2 * hSS + 1;
  auto keyAt = [&](int p) -> uint32_t {
    const uint8_t fl = flags[p];
    return (!bad[p] && (fl & FL_KFQ) && (fl & FL_VPOS)) ? __float_as_uint(V[p]) : 0u;
  };
  auto orAt = [&](int p) -> uint8_t {
    const uint8_t fl = flags[p];
    return (bad[p] ? OK_BAD : 0) | ((fl & FL_PRED) ? OK_PRED : 0) | ((fl & FL_NONPOS) ? OK_NONPOS : 0);
  };
  auto build = [&](int x0, int x1, int k0, int k1, int r0, int r1) {
    // ---- rows [k0, k1]: block scans along x over the blocks under the windows
    {
      const int ba = max(x0 - hSS, 0) / W, bb = min(x1 + hSS, n - 1) / W;
      const int nr = k1 - k0 + 1, nTask = nr * (bb - ba + 1);
      for(int t = tid; t < 2 * nTask; t += FS_T) {  // prefix and suffix on separate threads
        const bool suffix = t >= nTask;
        const int tt = suffix ? t - nTask : t;
        const int ly = k0 + tt % nr, blk = ba + tt / nr, row = ly * n;
        const int b0 = blk * W, b1 = min(b0 + W - 1, n - 1);
        uint32_t bk = 0;
        int bi = 0xFF;
        uint8_t o = 0;
        if(!suffix) {
          for(int x = b0; x <= b1; x++) {
            const int p = row + x;
            const uint32_t k = keyAt(p);
            if(k > bk) {
              bk = k;
              bi = x;
            }
            if(x < sx) o |= orAt(p);
            tPA[p] = (uint8_t)bi;
            tPO[p] = o;
          }
        } else {
          for(int x = b1; x >= b0; x--) {
            const int p = row + x;
            const uint32_t k = keyAt(p);
            if(k != 0 && k >= bk) {
              bk = k;
              bi = x;
            }
            if(x < sx) o |= orAt(p);
            tSA[p] = (uint8_t)bi;
            tSO[p] = o;
          }
        }
      }
    }
    __syncthreads();
    const int kw = x1 - x0 + 1;
    for(int i = tid; i < (k1 - k0 + 1) * kw; i += FS_T) {
      const int ly = k0 + i / kw, lx = x0 + i % kw, row = ly * n;
      const int a = max(lx - hSS, 0), b = min(lx + hSS, n - 1);
      uint8_t h, o;
      if(a / W != b / W) {
        const uint8_t L = tSA[row + a], R = tPA[row + b];
        h = L == 0xFF ? R : R == 0xFF ? L : (keyAt(row + R) > keyAt(row + L) ? R : L);
        o = tSO[row + a] | tPO[row + b];
      } else if(a % W == 0) {
        h = tPA[row + b];
        o = tPO[row + b];
      } else {
        h = tSA[row + a];
        o = tSO[row + a];
      }
      hx[row + lx] = h;
      rowf[row + lx] = o;
    }
    __syncthreads();
    // ---- columns [x0, x1]: block scans along y of the row winners
    {
      const int ba = max(r0 - hSS, 0) / W, bb = min(r1 + hSS, n - 1) / W;
      const int nTask = kw * (bb - ba + 1);
      auto candKey = [&](int y, int lx) -> uint32_t {
        const uint8_t xx = hx[y * n + lx];
        return xx == 0xFF ? 0u : keyAt(y * n + xx);
      };
      for(int t = tid; t < 2 * nTask; t += FS_T) {
        const bool suffix = t >= nTask;
        const int tt = suffix ? t - nTask : t;
        const int lx = x0 + tt % kw, blk = ba + tt / kw;
        const int b0 = blk * W, b1 = min(b0 + W - 1, n - 1);
        uint32_t bk = 0;
        int bi = 0xFF;
        uint8_t o = 0;
        if(!suffix) {
          for(int y = b0; y <= b1; y++) {
            const uint32_t k = candKey(y, lx);
            if(k > bk) {
              bk = k;
              bi = y;
            }
            if(y < sy) o |= rowf[y * n + lx];
            tPA[y * n + lx] = (uint8_t)bi;
            tPO[y * n + lx] = o;
          }
        } else {
          for(int y = b1; y >= b0; y--) {
            const uint32_t k = candKey(y, lx);
            if(k != 0 && k >= bk) {
              bk = k;
              bi = y;
            }
            if(y < sy) o |= rowf[y * n + lx];
            tSA[y * n + lx] = (uint8_t)bi;
            tSO[y * n + lx] = o;
          }
        }
      }
      __syncthreads();
      for(int i = tid; i < (r1 - r0 + 1) * kw; i += FS_T) {
        const int ly = r0 + i / kw, lx = x0 + i % kw;
        const int a = max(ly - hSS, 0), b = min(ly + hSS, n - 1);
        uint8_t yb, o;
        if(a / W != b / W) {
          const uint8_t L = tSA[a * n + lx], R = tPA[b * n + lx];
          yb = L == 0xFF ? R : R == 0xFF ? L : (candKey(R, lx) > candKey(L, lx) ? R : L);
          o = tSO[a * n + lx] | tPO[b * n + lx];
        } else if(a % W == 0) {
          yb = tPA[b * n + lx];
          o = tPO[b * n + lx];
        } else {
          yb = tSA[a * n + lx];
          o = tSO[a * n + lx];
        }
        arg[ly * n + lx] = yb == 0xFF ? (uint16_t)0xFFFF : (uint16_t)(yb * n + hx[yb * n + lx]);
        okw[ly * n + lx] = o;
      }
    }
    __syncthreads();
  };
  build(0, n - 1, 0, n - 1, 0, n - 1);
  const double floorV = sky + tKF * fwhm;
  double dfrac = 0.9;
  int cnt = 0, passes = 0;
  while(cnt < maxSS && passes < 256) {
    passes++;
    const double alt = sky + (tH - sky) * dfrac;
    const double lim = floorV < alt ? alt : floorV;  // OpenCL max()
    if(tid == 0) sfLim = __double2float_rd(lim);    // v > lim <=> v > sfLim for a float v
    __syncthreads();
    const float fLim = sfLim;
    int start = 0;
    while(cnt < maxSS && start < N) {
      int mine = INT_MAX;
      for(int p0 = start; p0 < N && mine == INT_MAX; p0 += 4 * FS_T) {
        for(int k = 0; k < 4; k++) {
          const int p = p0 + k * FS_T + tid;
          if(p >= N || p >= mine) break;
          if(bad[p] || !(flags[p] & FL_KFQ)) continue;
          if(!(V[p] > fLim)) continue;
          const int m = arg[p] != 0xFFFF ? arg[p] : p;
          const uint8_t o = okw[m];
          if(!(o & OK_BAD) && (o & OK_PRED)) {
            mine = p;
            break;
          }
        }
        mine = __reduce_min_sync(0xffffffffu, mine);
        if(tid == 0) sBest = INT_MAX;
        __syncthreads();
        if(lane == 0 && mine != INT_MAX) atomicMin(&sBest, mine);
        __syncthreads();
        mine = sBest;
        __syncthreads();
      }
      if(mine == INT_MAX) break;
      const int p = mine, m = arg[p] != 0xFFFF ? arg[p] : p;
      const int mx = cx + m % n, my = cy + m / n;
      const int u0 = max(mx - hSS, cx), v0 = max(my - hSS, cy);
      const int u1 = min(mx + hSS, cx + sx - 1), v1 = min(my + hSS, cy + sy - 1);
      const int uw = u1 - u0 + 1, un = uw * (v1 - v0 + 1);
      // value of the substamp: the reference's serial FP64 sum of the
      // thresholded pixels in raster order.  When they are all positive and
      // the sum of their magnitudes stays below 2^52 quanta of the smallest
      // (every pixel is a multiple of that quantum), no partial sum rounds in
      // any order; otherwise warp 0 forms the serial sum bit for bit (osum;
      // a pixel below the threshold adds +0.0, which changes nothing).
      double part = 0.0, amin = INFINITY;
      for(int i = tid; i < un; i += FS_T) {
        const int q = (v0 + i / uw - cy) * n + (u0 + i % uw - cx);
        if(flags[q] & FL_PRED) {
          const double v = (double)V[q];
          part += v;
          amin = fmin(amin, fabs(v));
        }
      }
#pragma unroll
      for(int o = 16; o > 0; o >>= 1) {
        part += __shfl_xor_sync(0xffffffffu, part, o);
        amin = fmin(amin, __shfl_xor_sync(0xffffffffu, amin, o));
      }
      if(lane == 0) {
        rA[warp] = part;
        rB[warp] = amin;
      }
      __syncthreads();
      if(warp == 0) {
        double t = lane < NW ? rA[lane] : 0.0, mn = lane < NW ? rB[lane] : INFINITY;
#pragma unroll
        for(int o = 16; o > 0; o >>= 1) {
          t += __shfl_xor_sync(0xffffffffu, t, o);
          mn = fmin(mn, __shfl_xor_sync(0xffffffffu, mn, o));
        }
        bool exact = false;
        if(!(okw[m] & OK_NONPOS) && mn > 0.0 && mn < INFINITY) {
          int e;
          frexp(mn, &e);  // mn in [2^(e-1), 2^e)
          exact = t < ldexp(1.0, e - 1 - 23 + 52);
        }
        if(!exact)
          t = osum::warpOrderedSumOf(un, [&](int i) {
            const int q = (v0 + i / uw - cy) * n + (u0 + i % uw - cx);
            return (flags[q] & FL_PRED) ? V[q] : 0.f;
          });
        if(lane == 0) sSum = t;
      }
      __syncthreads();
      const double ret = sSum;
      start = p + 1;
      if(ret == 0.0) continue;
      if(tid == 0) {
        locXY[cnt] = make_int2(mx, my);
        locVal[cnt] = ret;
      }
      cnt++;
      for(int i = tid; i < un; i += FS_T) {
        const int gx = u0 + i % uw, gy = v0 + i / uw;
        orMask(mask, (size_t)gx + (size_t)gy * w, skipMask);
        bad[(gy - cy) * n + (gx - cx)] = 1;  // skipMask is part of badMask
      }
      __syncthreads();
      if(cnt < maxSS) {
        // keys change inside the window only; maps within hSS of it
        const int a0 = u0 - cx, a1 = u1 - cx, b0 = v0 - cy, b1 = v1 - cy;
        build(max(a0 - hSS, 0), min(a1 + hSS, n - 1), b0, b1, max(b0 - hSS, 0),
              min(b1 + hSS, n - 1));
      }
    }
    if(cnt >= maxSS || lim == floorV) break;
    dfrac -= 0.2;
  }
  __syncthreads();
  if(tid == 0) {
    for(int i = 1; i < cnt; i++)
      for(int j = i; j > 0 && locVal[j - 1] < locVal[j]; j--) {
        int2 t = locXY[j - 1];
        locXY[j - 1] = locXY[j];
        locXY[j] = t;
        double tv = locVal[j - 1];
        locVal[j - 1] = locVal[j];
        locVal[j] = tv;
      }
    for(int i = 0; i < maxSS; i++) {
      xyOut[i] = i < cnt ? locXY[i] : make_int2(INT_MAX, INT_MAX);
      valOut[i] = i < cnt ? locVal[i] : -INFINITY;
    }
    (im == 0 ? cnt0 : cnt1)[s] = min(cnt, maxSS / 2);
  }
}

// removeEmptyStamps (src/sssUtil.cpp:106-197, sss.cl:543-571): keep stamps
// with at least one substamp in ascending original order.  One CTA per image.
__global__ void __launch_bounds__(256)
    k_compact_stamps(const int* __restrict__ cntAll, const int2* __restrict__ xyAll,
                     const double* __restrict__ valAll, int nAll, int maxSS,
                     int* __restrict__ orig, int* __restrict__ count, int* __restrict__ cur,
                     int2* __restrict__ xy, double* __restrict__ val, int* __restrict__ nOut) {
  __shared__ int warpTot[8];
  __shared__ int sTotal;
  int done = 0;
  for(int base = 0; base < nAll; base += 256) {
    int s = base + threadIdx.x;
    int keep = (s < nAll && cntAll[s] > 0) ? 1 : 0;
    int pos = blockScanExcl(keep, warpTot, &sTotal) + done;
    if(keep) {
      orig[pos] = s;
      count[pos] = cntAll[s];
      cur[pos] = 0;
      for(int k = 0; k < maxSS; k++) {
        bool live = k < cntAll[s];
        xy[(size_t)pos * maxSS + k] = live ? xyAll[(size_t)s * maxSS + k] : make_int2(INT_MAX, INT_MAX);
        val[(size_t)pos * maxSS + k] = live ? valAll[(size_t)s * maxSS + k] : -INFINITY;
      }
    }
    done += sTotal;
    __syncthreads();
  }
  if(threadIdx.x == 0) *nOut = done;
}

// createStampBounds (sss.cl:19-38) on the device, for frame graphs: the
// same integer expressions as the host table of stageSss.
__global__ void k_stamp_geom(int4* __restrict__ geom, int nAll, int stampsx, int stampsy, int w,
                             int h, int fSW) {
  const int id = blockIdx.x * blockDim.x + threadIdx.x;
  if(id >= nAll) return;
  const int sxI = id % stampsx, syI = id / stampsx;
  const int startX = sxI * w / stampsx, startY = syI * h / stampsy;
  const int stopX = min(startX + fSW, w), stopY = min(startY + fSW, h);
  geom[id] = make_int4(startX, startY, stopX - startX, stopY - startY);
}

__global__ void k_reset_skip(uint16_t* mask, long long n) {
  for(long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
      i += (long long)gridDim.x * blockDim.x)
    mask[i] &= (uint16_t)~(SKIP_S | SKIP_T);
}

}  // namespace

// The ran1 sequence of seed -666 (the seed of every stamp, sss.cl:81-116),
// n draws, generated once per context and size.
static const double* ran1Draws(xb_ctx* c, int n) {
  const std::string key = "ran1_draws";
  auto it = c->pool.find(key);
  const bool have = it != c->pool.end() && it->second.bytes >= (size_t)n * sizeof(double) &&
                    c->scalars.count("ran1_draws_n") && c->scalars["ran1_draws_n"] >= n;
  double* d = buf<double>(c, key, n);
  if(!have) {
    std::vector<double> h(n);
    Ran1 rng;
    double r[98];
    rng.init(-666);
    for(int i = 0; i < n; i++) h[i] = rng.next(r);
    toDevice(c, d, h);
    c->scalars["ran1_draws_n"] = n;
  }
  return d;
}

static void sssPass(xb_ctx* c, int* nKept) {
  const Geo& g = c->g;
  const int fSW = c->fStampWidth, nAll = c->nAll;
  const int maxChunks = (fSW * fSW + 31) / 32;
  double* chunkBuf = c->dWork;  // sized by stageSss
  const double* draws = ran1Draws(c, 2 * fSW * fSW);
  for(int im = 0; im < 2; im++) {
    { KT_SCOPE(c, "stamp_stats");
    if(c->imgIsF64)
      k_stamp_stats<double><<<nAll, ST_THREADS, 0, c->stream>>>(
          (const double*)c->img[im], c->mask, c->geomAll, c->w, c->h, fSW,
          c->goodScratch, c->clipScratch, chunkBuf, maxChunks, c->p.sigClipAlpha,
          c->p.iqRange, c->skyAll[im], c->fwhmAll[im], draws);
    else
      k_stamp_stats<float><<<nAll, ST_THREADS, 0, c->stream>>>(
          (const float*)c->img[im], c->mask, c->geomAll, c->w, c->h, fSW,
          reinterpret_cast<float*>(c->goodScratch), c->clipScratch, chunkBuf, maxChunks, c->p.sigClipAlpha,
          c->p.iqRange, c->skyAll[im], c->fwhmAll[im], draws);
    XB_LAUNCHED(c);
    }
  }
  dim3 grid(nAll, 2);
  { KT_SCOPE(c, "find_substamps");
  const size_t perCta = ((size_t)fSW * fSW * 24 + 255) / 256 * 256;
  const size_t fsSmem = fsSmemBytes(fSW);
  const bool inShared = !c->imgIsF64 && fSW <= 120;
  // global-memory maps only for the kernel that uses them
  unsigned char* scratch =
      inShared ? nullptr : buf<unsigned char>(c, "fm_scratch", (size_t)2 * nAll * perCta);
  if(inShared) {
    XB_CUDA(allowMaxDynamicSmem((const void*)k_find_substamps_sm, c->device));
    k_find_substamps_sm<<<grid, FS_T, fsSmem, c->stream>>>(
        (const float*)c->img[0], (const float*)c->img[1], c->mask, c->geomAll, c->skyAll[0],
        c->fwhmAll[0], c->skyAll[1], c->fwhmAll[1], c->ssxyAll[0], c->ssvalAll[0], c->cntAll[0],
        c->ssxyAll[1], c->ssvalAll[1], c->cntAll[1], c->w, fSW, g.hSS, g.maxSS, c->p.threshHigh,
        c->p.threshKernFit);
  } else if(c->imgIsF64)
    k_find_substamps_maps<double><<<grid, FM_THREADS, 0, c->stream>>>(
        (const double*)c->img[0], (const double*)c->img[1], c->mask, c->geomAll,
        c->skyAll[0], c->fwhmAll[0], c->skyAll[1], c->fwhmAll[1], c->ssxyAll[0],
        c->ssvalAll[0], c->cntAll[0], c->ssxyAll[1], c->ssvalAll[1], c->cntAll[1], c->w,
        fSW, g.hSS, g.maxSS, c->p.threshHigh, c->p.threshKernFit, scratch, perCta, 0);
  else
    k_find_substamps_maps<float><<<grid, FM_THREADS, 0, c->stream>>>(
        (const float*)c->img[0], (const float*)c->img[1], c->mask, c->geomAll,
        c->skyAll[0], c->fwhmAll[0], c->skyAll[1], c->fwhmAll[1], c->ssxyAll[0],
        c->ssvalAll[0], c->cntAll[0], c->ssxyAll[1], c->ssvalAll[1], c->cntAll[1], c->w,
        fSW, g.hSS, g.maxSS, c->p.threshHigh, c->p.threshKernFit, scratch, perCta, 1);
  XB_LAUNCHED(c);
  }
  for(int im = 0; im < 2; im++) {
    StampSetDev& S = c->set[im];
    { KT_SCOPE(c, "compact_stamps");
    k_compact_stamps<<<1, 256, 0, c->stream>>>(c->cntAll[im], c->ssxyAll[im], c->ssvalAll[im],
                                               nAll, g.maxSS, S.orig, S.count, S.cur, S.ssxy,
                                               S.ssval, c->dIWork + im);
    XB_LAUNCHED(c);
    }
  }
  if(c->capturing) return;  // frame graphs keep the counts on the device
  std::vector<int> n = toHost(c, c->dIWork, 2);
  nKept[0] = n[0];
  nKept[1] = n[1];
}

void stageSss(xb_ctx* c) {
  const Geo& g = c->g;
  const int w = c->w, h = c->h;
  // stamp width rule of src/bach.cpp:51-66
  c->stampsx = c->p.stampsx;
  c->stampsy = c->p.stampsy;
  int fSW = std::min(w / c->stampsx, h / c->stampsy);
  fSW -= g.fK;
  fSW -= fSW % 2 == 0 ? 1 : 0;
  if(fSW < g.fSS) {
    fSW = g.fSS + g.fK;
    fSW -= fSW % 2 == 0 ? 1 : 0;
    c->stampsx = w / fSW;
    c->stampsy = h / fSW;
  }
  c->fStampWidth = fSW;
  if(c->stampsx <= 0 || c->stampsy <= 0) throw XbError{XB_ERR_ARG, "image too small for one stamp"};
  if(fSW > 2048) throw XbError{XB_ERR_UNSUPPORTED, "stamp width above 2048"};
  if(g.maxSS > MAX_MAXSS || g.fSS > MAX_FSS)
    throw XbError{XB_ERR_UNSUPPORTED, "substamp parameters above this build's limits"};
  const int nAll = c->stampsx * c->stampsy;
  c->nAll = nAll;
  // createStampBounds (sss.cl:19-38)
  std::vector<int4> geom(nAll);
  for(int id = 0; id < nAll; id++) {
    int sxI = id % c->stampsx, syI = id / c->stampsx;
    int startX = sxI * w / c->stampsx, startY = syI * h / c->stampsy;
    int stopX = std::min(startX + fSW, w), stopY = std::min(startY + fSW, h);
    geom[id] = make_int4(startX, startY, stopX - startX, stopY - startY);
    if((stopX - startX) * (stopY - startY) < NSAMPLES)  // bachUtil.cpp:145-155
      throw XbError{XB_ERR_STAMP_TOO_SMALL, "Not enough pixels in a stamp"};
  }
  // buffers for this grid
  c->geomAll = buf<int4>(c, "geomAll", nAll);
  for(int im = 0; im < 2; im++) {
    const std::string sfx = std::to_string(im);
    c->skyAll[im] = buf<double>(c, "skyAll" + sfx, nAll);
    c->fwhmAll[im] = buf<double>(c, "fwhmAll" + sfx, nAll);
    c->cntAll[im] = buf<int>(c, "cntAll" + sfx, nAll);
    c->ssxyAll[im] = buf<int2>(c, "ssxyAll" + sfx, (size_t)nAll * g.maxSS);
    c->ssvalAll[im] = buf<double>(c, "ssvalAll" + sfx, (size_t)nAll * g.maxSS);
    StampSetDev& S = c->set[im];
    S.orig = buf<int>(c, "orig" + sfx, nAll);
    S.count = buf<int>(c, "count" + sfx, nAll);
    S.cur = buf<int>(c, "cur" + sfx, nAll);
    S.ssxy = buf<int2>(c, "ssxy" + sfx, (size_t)nAll * g.maxSS);
    S.ssval = buf<double>(c, "ssval" + sfx, (size_t)nAll * g.maxSS);
  }
  c->goodScratch = buf<double>(c, "goodScratch", (size_t)nAll * statsSlice(fSW));
  c->clipScratch = buf<uint8_t>(c, "clipScratch", (size_t)nAll * statsSlice(fSW));
  const size_t chunkDoubles = (size_t)nAll * 2 * ((fSW * fSW + 31) / 32);
  c->dWork = buf<double>(c, "chunkScratch", chunkDoubles);
  c->dIWork = buf<int>(c, "iwork", 64);
  int nKept[2];
  if(c->capturing) {
    // frame graph: the grid is computed on the device (the upload would be a
    // per-shape constant), the retry is a conditional node on the counts
    k_stamp_geom<<<(nAll + 255) / 256, 256, 0, c->stream>>>(c->geomAll, nAll, c->stampsx,
                                                            c->stampsy, w, h, fSW);
    XB_LAUNCHED(c);
    sssPass(c, nKept);
    graphSssRetry(c, c->dIWork, nAll, [&] {
      const long long n = (long long)w * h;
      k_reset_skip<<<std::min<long long>((n + 255) / 256, c->smCount * 8), 256, 0, c->stream>>>(
          c->mask, n);
      XB_LAUNCHED(c);
      sssPass(c, nKept);
    });
    for(int im = 0; im < 2; im++) {
      c->set[im].n = nAll;  // bound; the kept count is dIWork[im]
      c->set[im].dN = c->dIWork + im;
    }
    if(c->rank && c->rankW) rankSubstamps(c);  // learned order, on the device
    c->scalars["stampsx"] = c->stampsx;
    c->scalars["stampsy"] = c->stampsy;
    c->scalars["fStampWidth"] = c->fStampWidth;
    return;
  }
  c->set[0].dN = c->set[1].dN = nullptr;
  toDevice(c, c->geomAll, geom);
  sssPass(c, nKept);
  const int oldCount = nAll;
  const double fT = (double)nKept[0] / oldCount, fS = (double)nKept[1] / oldCount;
  c->sssRetry = 0;
  if(fT < 0.1 || fS < 0.1) {
    // bach.cpp:142-161: halve threshLow (unused by sss), clear the SKIP bits,
    // recompute everything with the current mask
    c->sssRetry = 1;
    const long long n = (long long)w * h;
    k_reset_skip<<<std::min<long long>((n + 255) / 256, c->smCount * 8), 256, 0, c->stream>>>(c->mask, n);
    XB_LAUNCHED(c);
    sssPass(c, nKept);
  }
  c->set[0].n = nKept[0];
  c->set[1].n = nKept[1];
  c->scalars["nstamps0"] = nKept[0];
  c->scalars["nstamps1"] = nKept[1];
  if(nKept[0] == 0 && nKept[1] == 0) throw XbError{XB_ERR_NO_SUBSTAMPS, "No substamps found"};
  if(c->rank && c->rankW) rankSubstamps(c);  // learned order of each stamp's substamps
  if(c->trace) {
    for(int im = 0; im < 2; im++) {
      const std::string sfx = std::to_string(im);
      c->put("sky" + sfx, toHost(c, c->skyAll[im], nAll));
      c->put("fwhm" + sfx, toHost(c, c->fwhmAll[im], nAll));
      c->put("ss_count_all" + sfx, toHost(c, c->cntAll[im], nAll));
      c->put("ss_xy_all" + sfx, toHost(c, c->ssxyAll[im], (size_t)nAll * g.maxSS));
      c->put("ss_val_all" + sfx, toHost(c, c->ssvalAll[im], (size_t)nAll * g.maxSS));
      const StampSetDev& S = c->set[im];
      c->put("stamp_index" + sfx, toHost(c, S.orig, S.n));
      c->put("ss_count" + sfx, toHost(c, S.count, S.n));
      c->put("ss_xy" + sfx, toHost(c, S.ssxy, (size_t)S.n * g.maxSS));
      c->put("ss_val" + sfx, toHost(c, S.ssval, (size_t)S.n * g.maxSS));
      c->scalars["nstamps" + sfx] = S.n;
    }
    c->put("mask_sss", toHost(c, c->mask, (size_t)w * h));
  }
  c->scalars["stampsx"] = c->stampsx;
  c->scalars["stampsy"] = c->stampsy;
  c->scalars["fStampWidth"] = c->fStampWidth;
  c->scalars["sss_retry"] = c->sssRetry;
}

}  // namespace xb

// ---------------------------------------------------------------------------
// Per-stamp statistics without any allocation.
//
// Some callers cannot allocate device memory: code that runs while another
// allocator (a framework's caching pool, a service's preallocated arena)
// owns the device and must not be bypassed, or code that must not let a
// cudaMalloc/cudaFree implicitly synchronise the device in the middle of
// its own work.  For them the stamp statistics of the sss stage (sky level
// and robust sigma per stamp, the same kernel xb_sss runs) are available
// with all scratch memory taken from a fixed device array that is part of the
// library image: every GPU that loads the library holds these 32 MiB until
// the process exits.  The caller passes the image, the mask, the stamp
// geometry and the two output arrays, all in device memory.

#include <cstring>
#include <mutex>

namespace {

constexpr size_t kStatsScratchBytes = size_t(32) << 20;  // 32 MiB
constexpr int kMaxDevices = 64;
static __device__ __align__(256) unsigned char g_statsScratch[kStatsScratchBytes];

std::mutex g_statsScratchMutex;
void* g_statsScratchAddr[kMaxDevices] = {};

size_t alignUp(size_t v) { return (v + 255) & ~size_t(255); }

int noallocFail(char* err, size_t errCap, int code, const char* msg) {
  if(err && errCap) {
    std::strncpy(err, msg, errCap - 1);
    err[errCap - 1] = '\0';
  }
  return code;
}

}  // namespace

extern "C" int xb_stamp_stats_noalloc(const float* dImg, uint16_t* dMask, int w, int h,
                                      const int* dGeom, int nStamps, int fStampWidth,
                                      double sigClipAlpha, double iqRange, double* dSky,
                                      double* dFwhm, void* stream, char* err, size_t errCap) {
  if(!dImg || !dMask || !dGeom || !dSky || !dFwhm || w <= 0 || h <= 0 || nStamps <= 0 ||
     fStampWidth <= 0)
    return noallocFail(err, errCap, XB_ERR_ARG, "null pointer or non-positive size");
  if(((uintptr_t)dGeom & 15u) != 0)
    return noallocFail(err, errCap, XB_ERR_ARG, "stamp geometry must be 16-byte aligned");
  // scratch carve-up: good pixels (FP64), clip flags (bytes), chunk sums
  const size_t pix = (size_t)fStampWidth * fStampWidth;
  const int maxChunks = (int)((pix + 31) / 32);
  if(pix > (size_t)1 << 26)
    return noallocFail(err, errCap, XB_ERR_UNSUPPORTED, "stamps beyond 8192 px on a side");
  const size_t slice = xb::statsSlice(fStampWidth);
  const size_t goodBytes = alignUp((size_t)nStamps * slice * sizeof(double));
  const size_t clipBytes = alignUp((size_t)nStamps * slice);
  const size_t chunkBytes = alignUp((size_t)nStamps * 2 * maxChunks * sizeof(double));
  if(goodBytes + clipBytes + chunkBytes > kStatsScratchBytes)
    return noallocFail(err, errCap, XB_ERR_UNSUPPORTED,
                       "stamps need more than the 32 MiB scratch: nStamps * (9 * P + 16 * "
                       "ceil(fStampWidth^2 / 32)) bytes must fit, P = fStampWidth^2 rounded up "
                       "to a multiple of 1024");
  // An error left pending by the caller's own work is reported as such and
  // left in place (not cleared), so it is not mistaken for this call's.
  const cudaError_t pending = cudaPeekAtLastError();
  if(pending != cudaSuccess)
    return noallocFail(err, errCap, XB_ERR_CUDA, "a CUDA error was already pending; nothing launched");
  int dev = -1;
  if(cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
    return noallocFail(err, errCap, XB_ERR_CUDA, "no usable current CUDA device");
  void* base = nullptr;
  {
    // The array's device address is looked up once per device, with that
    // device current; host code must not use the symbol itself as an address.
    // The cached address belongs to the device's current context: after a
    // cudaDeviceReset the module is reloaded elsewhere, so the entry point
    // must not be used across a reset.
    std::lock_guard<std::mutex> lock(g_statsScratchMutex);
    if(!g_statsScratchAddr[dev]) {
      void* p = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&p, g_statsScratch);
      if(e != cudaSuccess || !p)
        return noallocFail(err, errCap, XB_ERR_CUDA, cudaGetErrorString(e));
      g_statsScratchAddr[dev] = p;
    }
    base = g_statsScratchAddr[dev];
  }
  unsigned char* b = static_cast<unsigned char*>(base);
  double* good = reinterpret_cast<double*>(b);
  uint8_t* clip = b + goodBytes;
  double* chunks = reinterpret_cast<double*>(b + goodBytes + clipBytes);
  // Nothing needs clearing: within one launch every scratch byte the kernel
  // reads is written first (clip flags and good pixels during the
  // compaction, chunk sums before they are summed).
  xb::k_stamp_stats<float><<<nStamps, xb::ST_THREADS, 0, (cudaStream_t)stream>>>(
      dImg, dMask, reinterpret_cast<const int4*>(dGeom), w, h, fStampWidth,
      reinterpret_cast<float*>(good), clip, chunks,
      maxChunks, sigClipAlpha, iqRange, dSky, dFwhm, nullptr);
  // no error was pending before the launch, so any error now is the launch's
  cudaError_t e = cudaGetLastError();
  if(e != cudaSuccess) return noallocFail(err, errCap, XB_ERR_CUDA, cudaGetErrorString(e));
  return XB_OK;
}

namespace xb {
namespace {
__global__ void k_ordered_sum(const double* __restrict__ c, int n, double* __restrict__ out) {
  const double s = osum::warpOrderedSum(c, n);
  if(threadIdx.x == 0) *out = s;
}
__global__ void k_ordered_sum_f32(const float* __restrict__ c, int n, double* __restrict__ out) {
  const double s = osum::warpOrderedSumOf(n, [c](int i) { return c[i]; });
  if(threadIdx.x == 0) *out = s;
}
}  // namespace
}  // namespace xb

extern "C" double xb_ordered_sum_host(const double* c, int n) {
  return (c == nullptr || n <= 0) ? 0.0 : xb::osum::orderedSumHost(c, n);
}

extern "C" int xb_ordered_sum_device(const double* dC, int n, double* dOut, void* stream) {
  if(dOut == nullptr || n < 0 || (n > 0 && dC == nullptr)) return XB_ERR_ARG;
  xb::k_ordered_sum<<<1, 32, 0, (cudaStream_t)stream>>>(dC, n, dOut);
  return cudaGetLastError() == cudaSuccess ? XB_OK : XB_ERR_CUDA;
}

extern "C" int xb_ordered_sum_device_f32(const float* dC, int n, double* dOut, void* stream) {
  if(dOut == nullptr || n < 0 || (n > 0 && dC == nullptr)) return XB_ERR_ARG;
  xb::k_ordered_sum_f32<<<1, 32, 0, (cudaStream_t)stream>>>(dC, n, dOut);
  return cudaGetLastError() == cudaSuccess ? XB_OK : XB_ERR_CUDA;
}
