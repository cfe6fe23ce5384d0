// xbach_oracle.cpp — CPU oracle of the X-BACH difference-imaging path.
//
// This file restates, as a checker, the algorithms of D0V4HKIIN/Thesis-EMX-BACH
// (X-BACH), which is distributed under the following notice:
//
//   The MIT License (MIT)
//
//   Copyright (c) 2024 MindRoad Öst AB
//
//   Permission is hereby granted, free of charge, to any person obtaining a copy of
//   this software and associated documentation files (the "Software"), to deal in
//   the Software without restriction, including without limitation the rights to
//   use, copy, modify, merge, publish, distribute, sublicense, and/or sell copies of
//   the Software, and to permit persons to whom the Software is furnished to do so,
//   subject to the following conditions:
//
//   The above copyright notice and this permission notice shall be included in all
//   copies or substantial portions of the Software.
//
//   THE SOFTWARE IS PROVIDED "AS IS", WITHOUT WARRANTY OF ANY KIND, EXPRESS OR
//   IMPLIED, INCLUDING BUT NOT LIMITED TO THE WARRANTIES OF MERCHANTABILITY, FITNESS
//   FOR A PARTICULAR PURPOSE AND NONINFRINGEMENT. IN NO EVENT SHALL THE AUTHORS OR
//   COPYRIGHT HOLDERS BE LIABLE FOR ANY CLAIM, DAMAGES OR OTHER LIABILITY, WHETHER
//   IN AN ACTION OF CONTRACT, TORT OR OTHERWISE, ARISING FROM, OUT OF OR IN
//   CONNECTION WITH THE SOFTWARE OR THE USE OR OTHER DEALINGS IN THE SOFTWARE.
//
// TEST INFRASTRUCTURE ONLY: the checker used by tests/, by the smoke test and
// by the benchmark's CPU-baseline leg.  It restates, sequentially and in
// FP64, the host code (src/bach.cpp, src/sssUtil.cpp, src/cmvUtil.cpp,
// src/cdkscUtil.cpp, src/bachUtil.cpp) and the OpenCL kernels (cl_kern/*.cl)
// of D0V4HKIIN/Thesis-EMX-BACH.  Each function names the reference lines it
// follows.  Canonical choices where the reference is not deterministic:
//   * every atomic-order compaction (maskStamp sss.cl:157-188,
//     genCdTestStamps cd.cl:54-94, removeBadSigs cd.cl:657-695,
//     checkBadSubStamps ksc.cl:1-49) keeps ascending index order;
//   * no multiply-add contraction anywhere (built with -ffp-contract=off);
//     sums run in the order the reference source writes them;
//   * OpenCL pown(x, n) is repeated multiplication 1*x*x*...; max(a, b) on
//     doubles is (a < b ? b : a) (OpenCL common-function definition);
//   * float->int conversions of the histogram index saturate (as the GPU
//     cvt instruction does) instead of being undefined;
//   * the substamp threshold loop of findSubStamps (sss.cl:404-490) is capped
//     at 256 passes; it only exceeds ~6 when the sky statistics are NaN, where
//     the reference would loop forever.
// OpenMP parallelises over stamps, entries and pixel rows; every output's
// reduction order stays fixed, so results do not depend on the thread count.

#include "xbach_oracle.h"

#include <algorithm>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr uint16_t BAD_PIX_VAL = 1u << 0, SAT_PIXEL = 1u << 1,
                   LOW_PIXEL = 1u << 2, NAN_PIXEL = 1u << 3,
                   BAD_CONV = 1u << 4, INPUT_MASK = 1u << 5, OK_CONV = 1u << 6,
                   BAD_INPUT = 1u << 7, BAD_PIXEL_T = 1u << 8,
                   SKIP_T = 1u << 9, BAD_PIXEL_S = 1u << 10, SKIP_S = 1u << 11,
                   BAD_OUTPUT = 1u << 12, ALL = (1u << 13) - 1u;

inline int triNum(int t) { return t * (t + 1) / 2; }  // include/mathUtil.h:3

// OpenCL pown as repeated multiplication (canonical choice, see header).
inline double ipow(double x, int n) {
  double r = 1.0;
  for(int i = 0; i < n; i++) r *= x;
  return r;
}
// OpenCL max(gentype) on doubles: "returns y if x < y, otherwise x".
inline double clmax(double a, double b) { return a < b ? b : a; }

// (x - (w * 0.5f)) / (w * 0.5f) evaluated in float, as cl_kern/cmv.cl:180
// and cl_kern/cd.cl:170 write it (int * float -> float).
inline double floatNorm(int x, int w) {
  float hw = (float)w * 0.5f;
  float r = ((float)x - hw) / hw;
  return (double)r;
}

// Saturating floor-to-int (the GPU cvt semantics; NaN -> 0).
inline int satFloorToInt(double v) {
  double f = std::floor(v);
  if(f != f) return 0;
  if(f >= 2147483647.0) return INT_MAX;
  if(f <= -2147483648.0) return INT_MIN;
  return (int)f;
}

struct Geo {
  int fSS, hSS, fK, hK, nPSF, nComp1, nComp2, nComp, nBG, matSize, nSol;
  int wRows, wCols, qCount, bCount, maxSS;
};

struct SubSt {
  int x = INT_MAX, y = INT_MAX;
  double val = -INFINITY;
};

struct StampSet {
  int n = 0;
  std::vector<int> orig, cx, cy, sx, sy, count, cur;
  std::vector<double> sky, fwhm;
  std::vector<SubSt> subs;           // n * maxSS
  std::vector<double> W, Q, B;       // n * wRows*wCols, n * q^2, n * b
  std::vector<double> omega;         // weighted fit: n * wCols pixel weights
};

double msSince(std::chrono::steady_clock::time_point t0) {
  return std::chrono::duration<double, std::milli>(
             std::chrono::steady_clock::now() - t0)
      .count();
}

}  // namespace

struct xbo_handle {
  xb_params p{};
  Geo g{};
  int w = 0, h = 0;
  std::vector<double> img[2];   // 0 = template, 1 = science
  std::vector<uint16_t> mask;
  std::vector<uint8_t> inMask;   // input mask (nonzero: excluded), or empty
  // basis (cl_kern/cmv.cl:1-68, include/datatypeUtil.h:46-118)
  std::vector<int> kgauss, kx, ky;          // per basis function
  std::vector<double> fX, fY, vec;          // nPSF*fK, nPSF*fK, nPSF*fK*fK
  std::vector<int> bgX, bgY;                // background exponents
  std::vector<int> kpX, kpY;                // spatial-kernel exponents
  int stampsx = 0, stampsy = 0, fStampWidth = 0;
  StampSet set[2];
  int chosen = 0;            // set index of the image being convolved
  int convTemplate = 0;
  std::vector<double> solution;
  double kernSum = 0.0;
  std::vector<double> conv, diff;
  int status = XB_OK;
  int singular = 0;
  bool keepW = false;
  std::map<std::string, std::vector<uint8_t>> arrays;
  std::map<std::string, double> scalars;

  template <class T>
  void put(const std::string& k, const std::vector<T>& v) {
    std::vector<uint8_t> b(v.size() * sizeof(T));
    if(!v.empty()) std::memcpy(b.data(), v.data(), b.size());
    arrays[k] = std::move(b);
  }
};

namespace {

// ---------------------------------------------------------------- init ----
// maskInput: src/bachUtil.cpp:8-21 -> cl_kern/ini.cl:15-35
void maskInput(xbo_handle& o) {
  const int w = o.w, h = o.h, border = o.p.hSStampWidth + o.p.hKernelWidth;
  const double tH = o.p.threshHigh, tL = o.p.threshLow;
  o.mask.assign((size_t)w * h, 0);
#pragma omp parallel for schedule(static)
  for(int y = 0; y < h; y++) {
    for(int x = 0; x < w; x++) {
      size_t id = (size_t)x + (size_t)y * w;
      uint16_t m = 0;
      double t = o.img[0][id], s = o.img[1][id];
      if(t == 0.0 || s == 0.0) m |= BAD_INPUT | BAD_PIX_VAL;
      if(t >= tH || s >= tH) m |= BAD_INPUT | SAT_PIXEL;
      if(t <= tL || s <= tL) m |= BAD_INPUT | LOW_PIXEL;
      if(x < border || x >= w - border || y < border || y >= h - border)
        m |= BAD_PIXEL_S | BAD_PIXEL_T;
      o.mask[id] = m;
    }
  }
  // input mask (extension; the reference defines INPUT_MASK, datatypeUtil.h:179,
  // but never sets it): excluded pixels are bad input before the dilation
  if(!o.inMask.empty())
    for(size_t id = 0; id < o.mask.size(); id++)
      if(o.inMask[id]) o.mask[id] |= INPUT_MASK | BAD_INPUT;
  // spreadMask: src/bachUtil.cpp:22-31 -> cl_kern/ini.cl:37-67.  Only
  // BAD_INPUT is read and only OK_CONV is written, so a snapshot of the
  // BAD_INPUT bits gives the in-place kernel's result.
  const int spreadWidth = (int)(o.p.hKernelWidth * o.p.inSpreadMaskFactor);
  const int w2 = spreadWidth / 2;
  std::vector<uint8_t> bad((size_t)w * h);
  for(size_t i = 0; i < bad.size(); i++) bad[i] = (o.mask[i] & BAD_INPUT) != 0;
#pragma omp parallel for schedule(static)
  for(int y = 0; y < h; y++) {
    for(int x = 0; x < w; x++) {
      size_t id = (size_t)x + (size_t)y * w;
      if(bad[id]) continue;
      int sx = std::max(x - w2, 0), sy = std::max(y - w2, 0);
      int ex = std::min(x + w2, w - 1), ey = std::min(y + w2, h - 1);
      bool hit = false;
      for(int y2 = sy; y2 <= ey && !hit; y2++)
        for(int x2 = sx; x2 <= ex; x2++)
          if(bad[(size_t)y2 * w + x2]) {
            hit = true;
            break;
          }
      if(hit) o.mask[id] |= OK_CONV;
    }
  }
}

// ------------------------------------------------------------ sigmaClip --
// src/bachUtil.cpp:34-128 with sigmaClipCalc (cl_kern/bach.cl:135-170): sums
// in chunks of 32 (sequential inside a chunk), chunk sums added sequentially
// on the host (std::accumulate, bachUtil.cpp:103-104).
void sigmaClip(const double* data, int count, double* mean, double* stdDev,
               int maxIter, double alpha) {
  if(count == 0) {
    *mean = 0.0;
    *stdDev = 1e10;
    return;
  }
  std::vector<uint8_t> m(count, 0);
  size_t curr = 0, prev = (size_t)count;
  const int nChunks = (count + 31) / 32;
  for(int it = 0; it < maxIter && curr != prev; it++) {
    if(prev <= 1) {
      *mean = 0.0;
      *stdDev = 1e10;
      return;
    }
    curr = prev;
    double sum = 0.0, sum2 = 0.0;
    for(int c = 0; c < nChunks; c++) {
      double s = 0.0, s2 = 0.0;
      int lc = std::min(32, count - c * 32);
      for(int l = 0; l < lc; l++) {
        int k = c * 32 + l;
        double d = m[k] == 0 ? data[k] : 0.0;
        s += d;
        s2 += d * d;
      }
      sum += s;
      sum2 += s2;
    }
    double n = (double)prev;
    double tMean = sum / n;
    double tStd = std::sqrt((sum2 - n * tMean * tMean) / (double)(prev - 1));
    double inv = 1.0 / tStd;
    size_t clip = 0;
    for(int k = 0; k < count; k++) {
      if(m[k] == 0 && std::fabs(data[k] - tMean) * inv > alpha) {
        m[k] = 1;
        clip++;
      }
    }
    prev = curr - clip;
    *mean = tMean;
    *stdDev = tStd;
  }
}

// ---------------------------------------------------------------- ran1 ---
// Numerical Recipes ran1 as written in cl_kern/sss.cl:52-79 (three LCGs
// and a 97-entry shuffle table, `long` = 64-bit).
struct Ran1 {
  int idum;
  long ix1 = 0, ix2 = 0, ix3 = 0;
  double r[98];
  int iff = 0;
  explicit Ran1(int seed) : idum(seed) { std::memset(r, 0, sizeof(r)); }
  double next() {
    const long M1 = 259200, IA1 = 7141, IC1 = 54773;
    const long M2 = 134456, IA2 = 8121, IC2 = 28411;
    const long M3 = 243000, IA3 = 4561, IC3 = 51349;
    const double RM1 = 1.0 / M1, RM2 = 1.0 / M2;
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

// ------------------------------------------------------------ calcStats --
// src/bachUtil.cpp:130-280: sampleStamp (sss.cl:81-116), pad (:118-133),
// bitonic sortSamples (:135-150, host loop bachUtil.cpp:229-240), maskStamp
// (:157-188), per-stamp sigmaClip (bachUtil.cpp:255-266), createHistogram
// (:190-324).
struct AllStamps {
  int n = 0;
  std::vector<int> cx, cy, sx, sy;
};

int calcStats(xbo_handle& o, const AllStamps& st, int which,
              std::vector<double>& skyOut, std::vector<double>& fwhmOut) {
  const int w = o.w, h = o.h, n = st.n, fSW = o.fStampWidth;
  const std::vector<double>& img = o.img[which];
  constexpr int nSamples = 100, padded = 128;
  for(int i = 0; i < n; i++)
    if(st.sx[i] * st.sy[i] < nSamples) return XB_ERR_STAMP_TOO_SMALL;

  std::vector<double> samples((size_t)n * padded);
  std::vector<int> sampleCounts(n);
  // sampleStamp + pad
#pragma omp parallel for schedule(dynamic)
  for(int s = 0; s < n; s++) {
    Ran1 rng(-666);
    int numPix = st.sx[s] * st.sy[s];
    int cnt = 0;
    double tmp[nSamples];
    for(int iter = 0; cnt < nSamples && iter < numPix; iter++) {
      int rx = (int)std::floor(rng.next() * (int)st.sx[s]);
      int ry = (int)std::floor(rng.next() * (int)st.sy[s]);
      size_t idx = (size_t)(rx + st.cx[s]) + (size_t)(ry + st.cy[s]) * w;
      if(o.mask[idx] > 0 || std::fabs(img[idx]) <= 1e-10) continue;
      tmp[cnt++] = img[idx];
    }
    sampleCounts[s] = cnt;
    double* a = &samples[(size_t)s * padded];
    for(int i = 0; i < padded; i++)
      a[i] = i < nSamples ? (i < cnt ? tmp[i] : 0.0) : INFINITY;
    // bitonic network exactly as the 28 host-launched passes
    for(int k = 2; k <= padded; k *= 2)
      for(int j = k >> 1; j > 0; j >>= 1)
        for(int i = 0; i < padded; i++) {
          int ixj = i ^ j;
          if(ixj > i) {
            if((i & k) == 0 && a[i] > a[ixj]) std::swap(a[i], a[ixj]);
            if((i & k) != 0 && a[i] < a[ixj]) std::swap(a[i], a[ixj]);
          }
        }
  }
  // maskStamp: good pixels of the fStampWidth^2 window, ascending index order.
  std::vector<std::vector<double>> good(n);
#pragma omp parallel for schedule(dynamic)
  for(int s = 0; s < n; s++) {
    auto& gv = good[s];
    for(int idxS = 0; idxS < fSW * fSW; idxS++) {
      int x = idxS % fSW, y = idxS / fSW;
      int xI = x + st.cx[s], yI = y + st.cy[s];
      if(xI >= w || yI >= h) continue;
      size_t id = (size_t)xI + (size_t)yI * w;
      double pix = img[id];
      if(o.mask[id] > 0 || pix <= 1e-10) continue;
      if(std::isnan(pix)) {
        o.mask[id] |= NAN_PIXEL | BAD_INPUT;
        continue;
      }
      gv.push_back(pix);
    }
  }
  std::vector<double> means(n), invStd(n);
#pragma omp parallel for schedule(dynamic)
  for(int s = 0; s < n; s++) {
    double mean = 0.0, sd = 0.0;
    sigmaClip(good[s].data(), (int)good[s].size(), &mean, &sd, 3,
              o.p.sigClipAlpha);
    means[s] = mean;
    invStd[s] = 1.0 / sd;
  }
  skyOut.assign(n, 0.0);
  fwhmOut.assign(n, 0.0);
  // createHistogram
#pragma omp parallel for schedule(dynamic)
  for(int s = 0; s < n; s++) {
    const double* ps = &samples[(size_t)s * padded];
    int sampleCount = sampleCounts[s];
    double upS = ps[(int)(0.9 * sampleCount)];
    double midS = ps[(int)(0.5 * sampleCount)];
    double binSize = (upS - midS) / (double)nSamples;
    double lowerBinVal = midS - (128.0 * binSize);
    int bins[256];
    int attempts = 0, okCount = 0;
    double lower = 0.0, upper = 0.0, skyEst = 0.0;
    bool setFwhm = true;
    const double mean = means[s], inv = invStd[s];
    while(true) {
      if(attempts >= 5) {
        setFwhm = false;
        break;
      }
      for(int i = 0; i < 256; i++) bins[i] = 0;
      okCount = 0;
      for(int y = 0; y < st.sy[s]; y++)
        for(int x = 0; x < st.sx[s]; x++) {
          size_t id = (size_t)(st.cx[s] + x) + (size_t)(st.cy[s] + y) * w;
          double v = img[id];
          if(o.mask[id] != 0 || v <= 1e-10) continue;
          if(std::fabs(v - mean) * inv > o.p.sigClipAlpha) continue;
          double fi = std::floor((v - lowerBinVal) / binSize);
          int index = satFloorToInt(fi);
          index = index == INT_MAX ? INT_MAX : index + 1;
          index = std::min(std::max(index, 0), 255);
          bins[index] = bins[index] + 1;
          okCount++;
        }
      if(okCount == 0 || binSize == 0.0) {
        setFwhm = false;
        break;
      }
      double sumBins = 0.0, maxDens = 0.0;
      int lowerIndex = 1, upperIndex = 1, maxIndex = -1;
      while(upperIndex < 255) {
        while(sumBins < okCount / 10.0 && upperIndex < 255)
          sumBins += bins[upperIndex++];
        if(sumBins / (upperIndex - lowerIndex) > maxDens) {
          maxDens = sumBins / (upperIndex - lowerIndex);
          maxIndex = lowerIndex;
        }
        sumBins -= bins[lowerIndex++];
      }
      if(maxIndex < 0 || maxIndex > 255) maxIndex = 0;
      sumBins = 0.0;
      double sumExpect = 0.0;
      for(int i = maxIndex; sumBins < okCount / 10.0 && i < 255; i++) {
        sumBins += bins[i];
        sumExpect += i * bins[i];
      }
      double modeBin = sumExpect / sumBins + 0.5;
      skyEst = lowerBinVal + binSize * (modeBin - 1.0);
      lower = okCount * 0.25;
      upper = okCount * 0.75;
      sumBins = 0.0;
      int i = 0;
      while(sumBins < lower) sumBins += bins[i++];
      lower = i - (sumBins - lower) / bins[i - 1];
      while(sumBins < upper) sumBins += bins[i++];
      upper = i - (sumBins - upper) / bins[i - 1];
      if(lower < 1.0 || upper > 255.0) {
        lowerBinVal -= 128.0 * binSize;
        binSize *= 2;
      } else if(upper - lower < 40.0) {
        binSize /= 3.0;
        lowerBinVal = skyEst - 128.0 * binSize;
      } else {
        break;
      }
      attempts++;
    }
    fwhmOut[s] = setFwhm ? binSize * (upper - lower) / o.p.iqRange : 0.0;
    skyOut[s] = skyEst;
  }
  return XB_OK;
}

// -------------------------------------------------------- findSubStamps --
// src/sssUtil.cpp:40-104 -> cl_kern/sss.cl:381-505 (checkSStamp :326-361,
// sortSubStamps :363-379).  One stamp at a time; writes only inside the
// stamp's own window, so stamps are independent.
double checkSStamp(xbo_handle& o, const std::vector<double>& img, double sky,
                   double fwhm, int mx, int my, int cx, int cy, int sx, int sy,
                   uint16_t badMask, uint16_t badPixelMask) {
  const int hSS = o.p.hSStampWidth, w = o.w;
  double ret = 0.0;
  int x0 = std::max(mx - hSS, cx), y0 = std::max(my - hSS, cy);
  int x1 = std::min(mx + hSS, cx + sx - 1), y1 = std::min(my + hSS, cy + sy - 1);
  for(int y = y0; y <= y1; y++)
    for(int x = x0; x <= x1; x++) {
      size_t a = (size_t)x + (size_t)y * w;
      if(o.mask[a] & badMask) return 0.0;
      double v = img[a];
      if(v > o.p.threshHigh) {
        o.mask[a] |= badPixelMask;
        return 0.0;
      }
      if((v - sky) / fwhm > o.p.threshKernFit) ret += v;
    }
  return ret;
}

void findSubStampsOne(xbo_handle& o, const AllStamps& st, int which, int s,
                      double sky, double fwhm, uint16_t badMask,
                      uint16_t badPixelMask, uint16_t skipMask, SubSt* out,
                      int* countOut) {
  const std::vector<double>& img = o.img[which];
  const int w = o.w, fSW = o.fStampWidth, hSS = o.p.hSStampWidth;
  const int maxSS = o.g.maxSS;
  const double tH = o.p.threshHigh, tKF = o.p.threshKernFit;
  const int cx = st.cx[s], cy = st.cy[s], sx = st.sx[s], sy = st.sy[s];
  double floorV = sky + tKF * fwhm;
  double dfrac = 0.9;
  std::vector<SubSt> loc(maxSS);
  int cnt = 0, passes = 0;
  while(cnt < maxSS && passes < 256) {
    passes++;
    double lim = clmax(floorV, sky + (tH - sky) * dfrac);
    for(int y = 0; y < fSW; y++) {
      int absy = y + cy;
      for(int x = 0; x < fSW; x++) {
        int absx = x + cx;
        size_t a = (size_t)absx + (size_t)absy * w;
        if(o.mask[a] & badMask) continue;
        double v = img[a];
        if(v > tH) {
          o.mask[a] |= badPixelMask;
          continue;
        }
        if((v - sky) * (1.0 / fwhm) < tKF) continue;
        if(v > lim) {
          double maxVal = 0;
          int mx = absx, my = absy;
          int x0 = std::max(absx - hSS, cx), y0 = std::max(absy - hSS, cy);
          int x1 = std::min(absx + hSS, cx + fSW - 1);
          int y1 = std::min(absy + hSS, cy + fSW - 1);
          for(int ky = y0; ky <= y1; ky++)
            for(int kx = x0; kx <= x1; kx++) {
              size_t ka = (size_t)kx + (size_t)ky * w;
              double kv = img[ka];
              if(o.mask[ka] & badMask) continue;
              if(kv >= tH) {
                o.mask[ka] |= badPixelMask;
                continue;
              }
              if((kv - sky) * (1.0 / fwhm) < tKF) continue;
              if(kv > maxVal) {
                maxVal = kv;
                mx = kx;
                my = ky;
              }
            }
          maxVal = checkSStamp(o, img, sky, fwhm, mx, my, cx, cy, sx, sy,
                               badMask, badPixelMask);
          if(maxVal == 0.0) continue;
          loc[cnt].x = mx;
          loc[cnt].y = my;
          loc[cnt].val = maxVal;
          cnt++;
          int x2a = std::max(mx - hSS, cx), y2a = std::max(my - hSS, cy);
          int x2b = std::min(mx + hSS, cx + sx - 1);
          int y2b = std::min(my + hSS, cy + sy - 1);
          for(int yy = y2a; yy <= y2b; yy++)
            for(int xx = x2a; xx <= x2b; xx++)
              o.mask[(size_t)xx + (size_t)yy * w] |= skipMask;
        }
        if(cnt >= maxSS) break;
      }
      if(cnt >= maxSS) break;
    }
    if(lim == floorV) break;
    dfrac -= 0.2;
  }
  // insertion sort, descending by value (sortSubStamps)
  for(int i = 1; i < cnt; i++)
    for(int j = i; j > 0 && loc[j - 1].val < loc[j].val; j--)
      std::swap(loc[j - 1], loc[j]);
  *countOut = std::min(cnt, maxSS / 2);
  for(int i = 0; i < maxSS; i++) out[i] = i < cnt ? loc[i] : SubSt{};
}

// ------------------------------------------------------------- basis -----
// cmv(): basis enumeration (src/bach.cpp:181-188), background exponents
// (:210-216), createKernelFilter (cl_kern/cmv.cl:1-43) and
// createKernelVector (:45-68); identical to the host Kernel struct
// (include/datatypeUtil.h:46-118).
void buildBasis(xbo_handle& o) {
  const int fK = o.g.fK, hK = o.g.hK;
  o.kgauss.clear();
  o.kx.clear();
  o.ky.clear();
  for(int gs = 0; gs < o.p.nGauss; gs++)
    for(int x = 0; x <= o.p.dg[gs]; x++)
      for(int y = 0; y <= o.p.dg[gs] - x; y++) {
        o.kgauss.push_back(gs);
        o.kx.push_back(x);
        o.ky.push_back(y);
      }
  const int nPSF = (int)o.kx.size();
  o.fX.assign((size_t)nPSF * fK, 0.0);
  o.fY.assign((size_t)nPSF * fK, 0.0);
  for(int n = 0; n < nPSF; n++) {
    double b = (double)o.p.bg[o.kgauss[n]];
    double sumX = 0.0, sumY = 0.0;
    for(int i = 0; i < fK; i++) {
      double x = (double)(i - hK);
      double qe = std::exp(-x * x * b);
      double fx = qe * ipow(x, o.kx[n]);
      double fy = qe * ipow(x, o.ky[n]);
      o.fX[(size_t)n * fK + i] = fx;
      o.fY[(size_t)n * fK + i] = fy;
      sumX += fx;
      sumY += fy;
    }
    if(o.kx[n] % 2 == 0 && o.ky[n] % 2 == 0) {
      double ix = 1.0 / sumX, iy = 1.0 / sumY;
      for(int i = 0; i < fK; i++) {
        o.fX[(size_t)n * fK + i] *= ix;
        o.fY[(size_t)n * fK + i] *= iy;
      }
    }
  }
  o.vec.assign((size_t)nPSF * fK * fK, 0.0);
  for(int n = 0; n < nPSF; n++)
    for(int v = 0; v < fK; v++)
      for(int u = 0; u < fK; u++) {
        double vv = o.fX[(size_t)n * fK + u] * o.fY[(size_t)n * fK + v];
        if(o.kx[n] % 2 == 0 && o.ky[n] % 2 == 0 && n > 0)
          vv -= o.fX[u] * o.fY[v];
        o.vec[(size_t)n * fK * fK + (size_t)v * fK + u] = vv;
      }
  o.bgX.clear();
  o.bgY.clear();
  for(int x = 0; x <= o.p.backgroundOrder; x++)
    for(int y = 0; y <= o.p.backgroundOrder - x; y++) {
      o.bgX.push_back(x);
      o.bgY.push_back(y);
    }
  o.kpX.clear();
  o.kpY.clear();
  for(int i = 0; i <= o.p.kernelOrder; i++)
    for(int j = 0; j <= o.p.kernelOrder - i; j++) {
      o.kpX.push_back(i);
      o.kpY.push_back(j);
    }
}

// ------------------------------------------------------------ fillStamp --
// src/cmvUtil.cpp:37-187: convStampY (cl_kern/cmv.cl:70-106, FP32
// accumulation of FP64 products), convStampX (:108-135), convStampOdd
// (:137-154), convStampBg (:156-193), createQ (:195-215), createB
// (:217-248).  `I` is the image convolved, `O` the image projected on.
void fillStamp(xbo_handle& o, StampSet& S, int s, const std::vector<double>& I,
               const std::vector<double>& O) {
  const Geo& g = o.g;
  const int w = o.w, hK = g.hK, fK = g.fK, hSS = g.hSS, fSS = g.fSS;
  const int xHalf = hSS + hK, yHalf = hSS;
  const int tW = 2 * xHalf + 1, tH = 2 * yHalf + 1, tPix = tW * tH;
  double* W = &S.W[(size_t)s * g.wRows * g.wCols];
  double* Q = &S.Q[(size_t)s * g.qCount * g.qCount];
  double* B = &S.B[(size_t)s * g.bCount];
  const bool live = S.cur[s] < S.count[s];
  int ssx = 0, ssy = 0;
  if(live) {
    ssx = S.subs[(size_t)s * g.maxSS + S.cur[s]].x;
    ssy = S.subs[(size_t)s * g.maxSS + S.cur[s]].y;
  }
  std::vector<float> tmp(tPix);
  for(int n = 0; n < g.nPSF; n++) {
    for(int p = 0; p < tPix; p++) {
      float v = 0.0f;
      if(live) {
        int j = ssy + p / tW - yHalf;
        int i = ssx + p % tW - xHalf;
        for(int y = -hK; y <= hK; y++) {
          float imgV = (float)I[(size_t)i + (size_t)(j + y) * w];
          v = (float)((double)v + (double)imgV * o.fY[(size_t)n * fK + hK - y]);
        }
      }
      tmp[p] = v;
    }
    for(int p = 0; p < fSS * fSS; p++) {
      int jj = p / fSS - hSS, ii = p % fSS - hSS;
      double w0 = 0.0;
      for(int x = -hK; x <= hK; x++) {
        int index = (ii + x) + tW / 2 + (jj + hSS) * tW;
        w0 += (double)tmp[index] * o.fX[(size_t)n * fK + hK - x];
      }
      W[(size_t)n * g.wCols + p] = w0;
    }
  }
  for(int n = 1; n < g.nPSF; n++)
    if(o.kx[n] % 2 == 0 && o.ky[n] % 2 == 0)
      for(int p = 0; p < g.wCols; p++) W[(size_t)n * g.wCols + p] -= W[p];
  for(int b = 0; b < g.nBG; b++)
    for(int p = 0; p < g.wCols; p++) {
      double a = 0.0;
      if(live) {
        int x = ssx - hSS + p % fSS, y = ssy - hSS + p / fSS;
        double xf = floatNorm(x, o.w), yf = floatNorm(y, o.h);
        a = ipow(xf, o.bgX[b]) * ipow(yf, o.bgY[b]);
      }
      W[(size_t)(g.nPSF + b) * g.wCols + p] = a;
    }
  // weighted fit (extension): weight 1 / sigma^2 of each substamp pixel, the
  // chi^2 noise model of calcSigs; every product of the normal equations
  // becomes a * (b * w_k) with b the later factor as written below
  const bool wfit = o.p.fitWeighted != 0;
  double* om = wfit ? &S.omega[(size_t)s * g.wCols] : nullptr;
  if(wfit) {
    const double invGain = o.p.gain > 0.0 ? 1.0 / o.p.gain : 1.0;
    const double rn2x2 = 2.0 * o.p.readNoise * o.p.readNoise;
    for(int p = 0; p < g.wCols; p++) {
      double v = 0.0;
      if(live) {
        const size_t id = (size_t)(ssx + p % fSS - hSS) + (size_t)(ssy + p / fSS - hSS) * w;
        const double var = (std::fabs(I[id]) + std::fabs(O[id])) * invGain + rn2x2;
        v = var > 0.0 ? 1.0 / var : 0.0;
      }
      om[p] = v;
    }
  }
  for(int i = 0; i < g.qCount; i++)
    for(int j = 0; j < g.qCount; j++) {
      double q0 = 0.0;
      if(i > 0 && j > 0 && j <= i)
        for(int k = 0; k < fSS * fSS; k++)
          q0 += wfit ? W[(size_t)(i - 1) * g.wCols + k] * (W[(size_t)(j - 1) * g.wCols + k] * om[k])
                     : W[(size_t)(i - 1) * g.wCols + k] * W[(size_t)(j - 1) * g.wCols + k];
      Q[(size_t)i * g.qCount + j] = q0;
    }
  for(int i = 0; i < g.bCount; i++) {
    double p0 = 0.0;
    if(live && i > 0)
      for(int x = -hSS; x <= hSS; x++)
        for(int y = -hSS; y <= hSS; y++) {
          int k = x + hSS + fSS * (y + hSS);
          const double ov = O[(size_t)(x + ssx) + (size_t)(y + ssy) * w];
          p0 += W[(size_t)(i - 1) * g.wCols + k] * (wfit ? ov * om[k] : ov);
        }
    B[i] = p0;
  }
}

// ------------------------------------------------------------------ LU ---
// NR ludcmp/lubksb.  `gpuForm` selects the OpenCL form (cl_kern/bach.cl:1-127:
// no zero-row check, vv = 1/big even when big = 0) versus the CPU form
// (src/bachUtil.cpp:319-411: returns 1 before decomposing on a zero row).
// Both are 1-based on an (n+1)x(n+1) row-major matrix.
int ludcmp(double* a, int n, int* index, bool gpuForm) {
  const int ld = n + 1;
  std::vector<double> vv(n + 1, 0.0);
  for(int i = 1; i <= n; i++) {
    double big = 0.0;
    for(int j = 1; j <= n; j++) {
      double t = std::fabs(a[i * ld + j]);
      if(t > big) big = t;
    }
    if(!gpuForm && big == 0.0) return 1;
    vv[i] = 1.0 / big;
  }
  int maxI = 0;
  for(int j = 1; j <= n; j++) {
    for(int i = 1; i < j; i++) {
      double sum = a[i * ld + j];
      for(int k = 1; k < i; k++) sum -= a[i * ld + k] * a[k * ld + j];
      a[i * ld + j] = sum;
    }
    double big = 0.0;
    for(int i = j; i <= n; i++) {
      double sum = a[i * ld + j];
      for(int k = 1; k < j; k++) sum -= a[i * ld + k] * a[k * ld + j];
      a[i * ld + j] = sum;
      double dum = vv[i] * std::fabs(sum);
      if(dum >= big) {
        big = dum;
        maxI = i;
      }
    }
    if(j != maxI) {
      // the GPU form swaps columns 1..n, the CPU form 1..n as well
      for(int k = 1; k <= n; k++) std::swap(a[maxI * ld + k], a[j * ld + k]);
      vv[maxI] = vv[j];
    }
    index[j] = maxI;
    if(a[j * ld + j] == 0.0) a[j * ld + j] = 1.0e-20;
    if(j != n) {
      double dum = 1.0 / a[j * ld + j];
      for(int i = j + 1; i <= n; i++) a[i * ld + j] *= dum;
    }
  }
  return 0;
}

void lubksb(const double* a, int n, const int* index, double* b) {
  const int ld = n + 1;
  int ii = 0;
  for(int i = 1; i <= n; i++) {
    int ip = index[i];
    double sum = b[ip];
    b[ip] = b[i];
    if(ii != 0) {
      for(int j = ii; j <= i - 1; j++) sum -= a[i * ld + j] * b[j];
    } else if(sum != 0.0) {
      ii = i;
    }
    b[i] = sum;
  }
  for(int i = n; i >= 1; i--) {
    double sum = b[i];
    for(int j = i + 1; j <= n; j++) sum -= a[i * ld + j] * b[j];
    b[i] = sum / a[i * ld + i];
  }
}

// ------------------------------------------------------ global system ----
// Spatial weights: createMatrixWeights (cl_kern/cd.cl:152-180) / the weight
// loop of CPU createMatrix (src/cdkscUtil.cpp:331-342).  Both evaluate the
// float-rounded normalised coordinate and products of powers.
void stampWeights(const xbo_handle& o, const StampSet& S, const std::vector<int>& ids,
                  std::vector<double>& wts) {
  const int nC2 = o.g.nComp2;
  wts.assign(ids.size() * nC2, 0.0);
  for(size_t t = 0; t < ids.size(); t++) {
    int s = ids[t];
    if(S.cur[s] >= S.count[s]) continue;
    const SubSt& ss = S.subs[(size_t)s * o.g.maxSS + S.cur[s]];
    double fx = floatNorm(ss.x, o.w), fy = floatNorm(ss.y, o.h);
    for(int k = 0; k < nC2; k++) wts[t * nC2 + k] = ipow(fx, o.kpX[k]) * ipow(fy, o.kpY[k]);
  }
}

// createMatrix: cl_kern/cd.cl:182-295 (cd) and src/cdkscUtil.cpp:307-402
// (ksc) produce the same entries in the same per-entry order (stamps in
// ascending order, one contribution per stamp per entry; exhausted stamps
// contribute exact zeros on the GPU and are skipped on the CPU).  Returns
// the (matSize+1)^2 row-major matrix.
void createMatrix(const xbo_handle& o, const StampSet& S, const std::vector<int>& ids,
                  const std::vector<double>& wts, std::vector<double>& M) {
  const Geo& g = o.g;
  const int ld = g.matSize + 1, nC2 = g.nComp2, nComp = g.nComp;
  const int nT = (int)ids.size(), pix = g.fSS * g.fSS;
  M.assign((size_t)ld * ld, 0.0);
  // per-stamp dot products that the reference recomputes per entry
  std::vector<double> pKB((size_t)nT * g.nComp1 * g.nBG, 0.0);  // W[i1]·W[bg]
  std::vector<double> p0B((size_t)nT * g.nBG, 0.0);             // W[0]·W[bg]
  std::vector<double> pBB((size_t)nT * g.nBG * g.nBG, 0.0);     // W[bg]·W[bg']
  std::vector<uint8_t> live(nT);
#pragma omp parallel for schedule(dynamic)
  for(int t = 0; t < nT; t++) {
    int s = ids[t];
    live[t] = S.cur[s] < S.count[s];
    const double* W = &S.W[(size_t)s * g.wRows * g.wCols];
    const double* om = S.omega.empty() ? nullptr : &S.omega[(size_t)s * g.wCols];
    // a * b, or a * (b * w_k) in the weighted fit
    auto dot = [&](const double* a, const double* b) {
      double p = 0.0;
      for(int k = 0; k < pix; k++) p += om ? a[k] * (b[k] * om[k]) : a[k] * b[k];
      return p;
    };
    for(int ib = 0; ib < g.nBG; ib++) {
      const double* wb = W + (size_t)(g.nComp1 + ib + 1) * g.wCols;
      for(int i1 = 1; i1 <= g.nComp1; i1++)
        pKB[((size_t)t * g.nComp1 + (i1 - 1)) * g.nBG + ib] = dot(W + (size_t)i1 * g.wCols, wb);
      p0B[(size_t)t * g.nBG + ib] = dot(W, wb);
      for(int jb = 0; jb <= ib; jb++)
        pBB[((size_t)t * g.nBG + ib) * g.nBG + jb] = dot(wb, W + (size_t)(g.nComp1 + jb + 1) * g.wCols);
    }
  }
  // entries of the lower triangle (row >= col >= 1), each summed over stamps
#pragma omp parallel for schedule(dynamic)
  for(int row = 1; row < ld; row++) {
    for(int col = 1; col <= row; col++) {
      double m0 = 0.0;
      for(int t = 0; t < nT; t++) {
        int s = ids[t];
        const double* Q = &S.Q[(size_t)s * g.qCount * g.qCount];
        const double* wt = &wts[(size_t)t * nC2];
        if(row == 1 && col == 1) {
          m0 += Q[1 * g.qCount + 1];
        } else if(row > nComp + 1 && col > nComp + 1) {
          int ib = row - (nComp + 2), jb = col - (nComp + 2);
          m0 += pBB[((size_t)t * g.nBG + ib) * g.nBG + jb];
        } else if(col == 1 && row > nComp + 1) {
          m0 += p0B[(size_t)t * g.nBG + (row - (nComp + 2))];
        } else if(row > nComp + 1 && col >= 2) {
          int ib = row - (nComp + 2);
          int i1 = (col - 2) / nC2 + 1, i2 = (col - 2) % nC2;
          m0 += pKB[((size_t)t * g.nComp1 + (i1 - 1)) * g.nBG + ib] * wt[i2];
        } else if(col == 1 && row >= 2) {
          int i = row - 2, i1 = i / nC2, i2 = i - i1 * nC2;
          m0 += wt[i2] * Q[(i1 + 2) * g.qCount + 1];
        } else {
          int i = row - 2, j = col - 2;
          int i1 = i / nC2, i2 = i - i1 * nC2, j1 = j / nC2, j2 = j - j1 * nC2;
          m0 += wt[i2] * wt[j2] * Q[(i1 + 2) * g.qCount + (j1 + 2)];
        }
        (void)live;
      }
      M[(size_t)row * ld + col] = m0;
    }
  }
  for(int row = 1; row < ld; row++)
    for(int col = 1; col < row; col++) M[(size_t)col * ld + row] = M[(size_t)row * ld + col];
}

// createScProd.  gpuForm: cl_kern/cd.cl:297-352 (row-major background
// projection on the FP64 image).  CPU form: src/cdkscUtil.cpp:429-475
// (column-major projection on float-rounded pixels, Image::operator[] of
// include/datatypeUtil.h:158; exhausted stamps skipped).
void createScProd(const xbo_handle& o, const StampSet& S, const std::vector<int>& ids,
                  const std::vector<double>& wts, const std::vector<double>& img,
                  bool gpuForm, std::vector<double>& res) {
  const Geo& g = o.g;
  const int nC2 = g.nComp2, hSS = g.hSS, fSS = g.fSS, w = o.w;
  res.assign(g.nSol, 0.0);
  const int nT = (int)ids.size();
  std::vector<double> bgP((size_t)nT * g.nBG, 0.0);
#pragma omp parallel for schedule(dynamic)
  for(int t = 0; t < nT; t++) {
    int s = ids[t];
    if(S.cur[s] >= S.count[s]) continue;
    const SubSt& ss = S.subs[(size_t)s * g.maxSS + S.cur[s]];
    const double* W = &S.W[(size_t)s * g.wRows * g.wCols];
    const double* om = S.omega.empty() ? nullptr : &S.omega[(size_t)s * g.wCols];
    for(int b = 0; b < g.nBG; b++) {
      const double* wb = W + (size_t)(g.nComp1 + b + 1) * g.wCols;
      double q = 0.0;
      if(gpuForm) {
        for(int y = -hSS; y <= hSS; y++)
          for(int x = -hSS; x <= hSS; x++) {
            int index = x + hSS + fSS * (y + hSS);
            const double v = img[(size_t)(x + ss.x) + (size_t)(y + ss.y) * w];
            q += wb[index] * (om ? v * om[index] : v);
          }
      } else {
        for(int x = -hSS; x <= hSS; x++)
          for(int y = -hSS; y <= hSS; y++) {
            int index = x + hSS + fSS * (y + hSS);
            const double v = (double)(float)img[(size_t)(x + ss.x) + (size_t)(y + ss.y) * w];
            q += wb[index] * (om ? v * om[index] : v);
          }
      }
      bgP[(size_t)t * g.nBG + b] = q;
    }
  }
  for(int t = 0; t < nT; t++) {
    int s = ids[t];
    if(S.cur[s] >= S.count[s]) continue;  // contributes zeros on the GPU form
    const double* B = &S.B[(size_t)s * g.bCount];
    const double* wt = &wts[(size_t)t * nC2];
    res[1] += B[1];
    for(int i = 1; i <= g.nComp1; i++)
      for(int j = 0; j < nC2; j++) res[(i - 1) * nC2 + j + 2] += B[i + 1] * wt[j];
    for(int b = 0; b < g.nBG; b++) res[g.nComp + b + 2] += bgP[(size_t)t * g.nBG + b];
  }
}

// Kernel coefficients at (xf, yf): makeKernelCoeffs (cl_kern/cd.cl:354-383)
// and the CPU makeKernel (src/bachUtil.cpp:508-526), same operation order.
void kernelCoeffs(const xbo_handle& o, const std::vector<double>& sol, double xf,
                  double yf, std::vector<double>& c) {
  const int nPSF = o.g.nPSF, ko = o.p.kernelOrder;
  c.assign(nPSF, 0.0);
  int k = 2;
  for(int i = 1; i < nPSF; i++) {
    double aX = 1.0;
    for(int ix = 0; ix <= ko; ix++) {
      double aY = 1.0;
      for(int iy = 0; iy <= ko - ix; iy++) {
        c[i] += sol[k++] * aX * aY;
        aY *= yf;
      }
      aX *= xf;
    }
  }
  c[0] = sol[1];
}

// Kernel image at pixel (x, y).  treeSum: the GPU makeKernel + sumKernel
// (cd.cl:385-442, 32-wide partial sums); otherwise the sequential CPU sum
// (bachUtil.cpp:532-538).
double makeKernel(const xbo_handle& o, const std::vector<double>& sol, int x, int y,
                  bool treeSum, double* kern) {
  double hx = 0.5 * o.w, hy = 0.5 * o.h;
  double xf = (x - hx) / hx, yf = (y - hy) / hy;
  std::vector<double> c;
  kernelCoeffs(o, sol, xf, yf, c);
  const int nk = o.g.fK * o.g.fK;
  std::vector<double> tmp;
  if(!kern) {
    tmp.resize(nk);
    kern = tmp.data();
  }
  for(int i = 0; i < nk; i++) {
    double k0 = 0.0;
    for(int p = 0; p < o.g.nPSF; p++) k0 += c[p] * o.vec[(size_t)p * nk + i];
    kern[i] = k0;
  }
  if(!treeSum) {
    double s = 0.0;
    for(int i = 0; i < nk; i++) s += kern[i];
    return s;
  }
  std::vector<double> cur(kern, kern + nk), nxt;
  int count = nk;
  while(count > 1) {
    int groups = (count + 31) / 32;
    nxt.assign(groups, 0.0);
    for(int gi = 0; gi < groups; gi++) {
      double s = 0.0;
      int lc = std::min(32, count - gi * 32);
      for(int l = 0; l < lc; l++) s += cur[gi * 32 + l];
      nxt[gi] = s;
    }
    cur.swap(nxt);
    count = groups;
  }
  return cur[0];
}

// getBackground: cl_kern/cd.cl:444-467 (double normalisation).
double getBackground(const xbo_handle& o, int x, int y, const std::vector<double>& sol) {
  double xf = (x - 0.5 * o.w) / (0.5 * o.w);
  double yf = (y - 0.5 * o.h) / (0.5 * o.h);
  double bg = 0.0;
  int k = o.g.nComp + 2;  // nBgComp + 1 with nBgComp = nComp1*nComp2 + 1
  double ax = 1.0;
  for(int i = 0; i <= o.p.backgroundOrder; i++) {
    double ay = 1.0;
    for(int j = 0; j <= o.p.backgroundOrder - i; j++) {
      bg += sol[k++] * ax * ay;
      ay *= yf;
    }
    ax *= xf;
  }
  return bg;
}

// calcSigs: src/cdkscUtil.cpp:477-583 -> calcSigBg (cd.cl:469-487), makeModel
// (:489-531, FP32 model), calcSig (:533-598), reduceSig (:600-655).  Returns
// one chi^2 per listed stamp (-1 when no pixel counts or chi^2 >= 1e10).
// `T` supplies the |t| of the denominator, `Simg` the data modelled.  The
// denominator (|t| + |s|) of cd.cl:578 becomes (|t| + |s|) * (1 / gain) +
// 2 readNoise^2 with the noise-model extension of xb_params (the same value
// for the defaults, gain 1 and no read noise).
void calcSigs(xbo_handle& o, const StampSet& S, const std::vector<int>& ids,
              const std::vector<double>& sol, const std::vector<double>& T,
              const std::vector<double>& Simg, std::vector<double>& sig) {
  const Geo& g = o.g;
  const double invGain = o.p.gain > 0.0 ? 1.0 / o.p.gain : 1.0;
  const double rn2x2 = 2.0 * o.p.readNoise * o.p.readNoise;
  const int nT = (int)ids.size(), fSS = g.fSS, pix = fSS * fSS, w = o.w;
  const int reduceCount = (pix + 31) / 32;
  sig.assign(nT, 0.0);
#pragma omp parallel for schedule(dynamic)
  for(int t = 0; t < nT; t++) {
    int s = ids[t];
    bool live = S.cur[s] < S.count[s];
    int ssx = 0, ssy = 0;
    double bg = 0.0;
    std::vector<float> model(pix, 0.0f);
    if(live) {
      const SubSt& ss = S.subs[(size_t)s * g.maxSS + S.cur[s]];
      ssx = ss.x;
      ssy = ss.y;
      bg = getBackground(o, ssx, ssy, sol);
      const double* W = &S.W[(size_t)s * g.wRows * g.wCols];
      double xf = (ssx - w * 0.5) / (w * 0.5);
      double yf = (ssy - o.h * 0.5) / (o.h * 0.5);
      std::vector<double> coeff(g.nPSF, 0.0);
      {
        int k = 2;
        for(int i = 1; i < g.nPSF; i++) {
          double c = 0.0, ax = 1.0;
          for(int x = 0; x <= o.p.kernelOrder; x++) {
            double ay = 1.0;
            for(int y = 0; y <= o.p.kernelOrder - x; y++) {
              c += sol[k++] * ax * ay;
              ay *= yf;
            }
            ax *= xf;
          }
          coeff[i] = c;
        }
      }
      for(int j = 0; j < pix; j++) {
        float m0 = (float)(sol[1] * W[j]);
        for(int i = 1; i < g.nPSF; i++)
          m0 = (float)((double)m0 + coeff[i] * W[(size_t)i * g.wCols + j]);
        model[j] = m0;
      }
    }
    // calcSig: 32-wide groups over gi in [0, reduceCount*32)
    std::vector<double> partial(reduceCount);
    std::vector<int> pcount(reduceCount);
    for(int grp = 0; grp < reduceCount; grp++) {
      double local[32];
      int lc = 0;
      for(int l = 0; l < 32; l++) {
        int gi = grp * 32 + l;
        int gx = gi % fSS, gy = gi / fSS;
        double s0 = 0.0;
        if(live && gx < fSS && gy < fSS) {
          int absX = gx - fSS / 2 + ssx, absY = gy - fSS / 2 + ssy;
          size_t ai = (size_t)absX + (size_t)absY * w;
          double tD = model[gx + gy * fSS];
          double sD = Simg[ai];
          double diff = tD - sD + bg;
          if((o.mask[ai] & BAD_INPUT) == 0 && std::fabs(sD) > 1e-10) {
            if(std::isnan(tD) || std::isnan(sD)) {
#pragma omp atomic
              o.mask[ai] |= NAN_PIXEL;
            } else {
              lc++;
              s0 = diff * diff / ((std::fabs(T[ai]) + std::fabs(sD)) * invGain + rn2x2);
            }
          }
        }
        local[l] = s0;
      }
      double sum = 0.0;
      for(int l = 0; l < 32; l++) sum += local[l];
      partial[grp] = sum;
      pcount[grp] = lc;
    }
    // reduceSig levels
    int count = reduceCount;
    bool first = true;
    double result = 0.0;
    while(count > 1 || first) {
      int next = (count + 31) / 32;
      std::vector<double> np(next);
      std::vector<int> nc(next);
      for(int gi = 0; gi < next; gi++) {
        double sum = 0.0;
        int c = 0;
        int lc = std::min(32, count - gi * 32);
        for(int l = 0; l < lc; l++) {
          sum += partial[gi * 32 + l];
          c += pcount[gi * 32 + l];
        }
        if(next == 1) {
          if(c == 0) sum = -1.0;
          else {
            sum /= c;
            if(sum >= 1e10) sum = -1.0;
          }
          result = sum;
        }
        np[gi] = sum;
        nc[gi] = c;
      }
      partial.swap(np);
      pcount.swap(nc);
      count = next;
      first = false;
    }
    sig[t] = result;
  }
}

// ------------------------------------------------------------- testFit ---
// src/cdkscUtil.cpp:4-266 for stamp set `si` convolving image I = img[ii]
// and projecting on O = img[1-ii].
double testFit(xbo_handle& o, int si, int ii) {
  StampSet& S = o.set[si];
  const Geo& g = o.g;
  const std::vector<double>& I = o.img[ii];
  const std::vector<double>& O = o.img[1 - ii];
  const int n = S.n, qc = g.qCount;
  const std::string sfx = std::to_string(si);
  // createTestVec/createTestMat + GPU ludcmp/lubksb (matrixSize = nPSF+2)
  std::vector<double> ks(n, 0.0);
#pragma omp parallel for schedule(dynamic)
  for(int s = 0; s < n; s++) {
    std::vector<double> M((size_t)qc * qc), v(qc);
    std::vector<int> idx(qc, 0);
    const double* Q = &S.Q[(size_t)s * qc * qc];
    const double* B = &S.B[(size_t)s * g.bCount];
    for(int i = 0; i < qc; i++) {
      v[i] = i > 0 ? B[i] : 0.0;
      for(int j = 0; j < qc; j++)
        M[(size_t)i * qc + j] =
            (i > 0 && j > 0) ? Q[(size_t)std::max(i, j) * qc + std::min(i, j)] : 0.0;
    }
    ludcmp(M.data(), qc - 1, idx.data(), true);
    lubksb(M.data(), qc - 1, idx.data(), v.data());
    ks[s] = v[1];
  }
  o.put("kernel_sums" + sfx, ks);
  double kMean = 0.0, kStd = 0.0;
  sigmaClip(ks.data(), n, &kMean, &kStd, 10, o.p.sigClipAlpha);
  std::vector<int> test;
  for(int s = 0; s < n; s++)
    if(std::fabs((ks[s] - kMean) / kStd) < o.p.sigKernFit) test.push_back(s);
  o.put("cd_test" + sfx, test);
  o.scalars["cd_kmean" + sfx] = kMean;
  o.scalars["cd_kstd" + sfx] = kStd;
  if(test.empty()) return 666;
  std::vector<double> wts, M, sol;
  stampWeights(o, S, test, wts);
  createMatrix(o, S, test, wts, M);
  o.put("cd_matrix" + sfx, M);
  createScProd(o, S, test, wts, O, true, sol);
  std::vector<int> idx(g.nSol + 1, 0);
  if(ludcmp(M.data(), g.matSize, idx.data(), false) != 0) o.singular = 1;
  lubksb(M.data(), g.matSize, idx.data(), sol.data());
  o.put("cd_solution" + sfx, sol);
  double kernelMean = makeKernel(o, sol, 0, 0, true, nullptr);
  o.scalars["cd_kernel_mean" + sfx] = kernelMean;
  std::vector<double> sig;
  calcSigs(o, S, test, sol, I, O, sig);
  o.put("cd_sig" + sfx, sig);
  std::vector<double> clean;
  for(double v : sig)
    if(v >= 0.0) clean.push_back(v);
  if(clean.empty()) return 666;
  double mMean = 0.0, mStd = 0.0;
  sigmaClip(clean.data(), (int)clean.size(), &mMean, &mStd, 10, o.p.sigClipAlpha);
  return mMean / kernelMean;
}

// -------------------------------------------------------------- fitKernel -
// src/cdkscUtil.cpp:585-802 on the chosen stamp set.
void fitKernel(xbo_handle& o) {
  StampSet& S = o.set[o.chosen];
  const Geo& g = o.g;
  const std::vector<double>& I = o.img[o.chosen];
  const std::vector<double>& O = o.img[1 - o.chosen];
  std::vector<int> all(S.n);
  for(int s = 0; s < S.n; s++) all[s] = s;
  std::vector<int> rejects;  // (iteration, pass, stamp)
  int iteration = 0;
  bool check = false;
  do {
    std::vector<double> wts, M, sol;
    stampWeights(o, S, all, wts);
    createMatrix(o, S, all, wts, M);
    if(iteration == 0) o.put("ksc_matrix0", M);
    createScProd(o, S, all, wts, O, false, sol);
    std::vector<int> idx(g.nSol + 1, 0);
    if(ludcmp(M.data(), g.matSize, idx.data(), false) != 0) o.singular = 1;
    lubksb(M.data(), g.matSize, idx.data(), sol.data());
    o.solution = sol;
    // checkFitSolution (:686-770)
    std::vector<double> sig;
    calcSigs(o, S, all, sol, I, O, sig);
    std::vector<double> chi2;
    std::vector<int> inv(S.n, 0);
    check = false;
    for(int s = 0; s < S.n; s++) {
      if(S.cur[s] < S.count[s]) {
        if(sig[s] == -1.0) {
          S.cur[s]++;
          inv[s] = 1;
        } else {
          chi2.push_back(sig[s]);
        }
      }
    }
#pragma omp parallel for schedule(dynamic)
    for(int s = 0; s < S.n; s++)
      if(inv[s]) fillStamp(o, S, s, I, O);
    for(int s = 0; s < S.n; s++)
      if(inv[s]) {
        check = true;
        rejects.insert(rejects.end(), {iteration, 0, s});
      }
    double mean = 0.0, sd = 0.0;
    sigmaClip(chi2.data(), (int)chi2.size(), &mean, &sd, 10, o.p.sigClipAlpha);
    for(int s = 0; s < S.n; s++) {
      inv[s] = 0;
      if(S.cur[s] < S.count[s]) {
        if((sig[s] - mean) > o.p.sigKernFit * sd) {
          S.cur[s]++;
          inv[s] = 1;
        }
      }
    }
#pragma omp parallel for schedule(dynamic)
    for(int s = 0; s < S.n; s++)
      if(inv[s]) fillStamp(o, S, s, I, O);
    for(int s = 0; s < S.n; s++)
      if(inv[s]) {
        check = true;
        rejects.insert(rejects.end(), {iteration, 1, s});
      }
    o.put("ksc_sig_last", sig);
    iteration++;
  } while(check);
  o.scalars["ksc_iterations"] = iteration;
  o.put("ksc_rejects", rejects);
  o.put("cur", S.cur);
  o.put("solution", o.solution);
}

// ------------------------------------------------------ per-pixel conv ---
// Extension (xb_params.convPerPixel; the reference evaluates the kernel once
// per fK x fK block, src/bach.cpp:339-350).  The kernel at pixel (x, y) is
// sum_t P_t Kt[t], P_t = xf^i yf^j of the pixel (x power outer) and
// Kt[t] = sol[1] vec_0 [t = 0] + sum_{n>=1} sol[2 + (n-1) nC2 + t] vec_n (FMA
// chain over n); the convolved value is sum_t P_t (Kt[t] * I)(x, y), each
// convolution an FMA chain over the window (rows, then columns), combined by
// an FMA chain over t.  Pixels with a bad input in the window evaluate their
// kernel tap by tap (FMA chain over t) for the 0.99 |kernel| rule of
// conv.cl:70-100.
void convPerPixel(xbo_handle& o, const std::vector<uint16_t>& cmask, double invKernMult) {
  const Geo& g = o.g;
  const int w = o.w, h = o.h, fK = g.fK, hK = g.hK, nk = fK * fK, nC2 = g.nComp2;
  const int kOrder = o.p.kernelOrder;
  const std::vector<double>& I = o.img[o.chosen];
  const std::vector<double>& sol = o.solution;
  std::vector<double> Kt((size_t)nC2 * nk);
  for(int t = 0; t < nC2; t++)
    for(int p = 0; p < nk; p++) {
      double k0 = t == 0 ? sol[1] * o.vec[p] : 0.0;
      for(int n = 1; n < g.nPSF; n++)
        k0 = std::fma(sol[2 + (size_t)(n - 1) * nC2 + t], o.vec[(size_t)n * nk + p], k0);
      Kt[(size_t)t * nk + p] = k0;
    }
  const double hx = 0.5 * w, hy = 0.5 * h;
#pragma omp parallel for schedule(static)
  for(int y = hK; y < h - hK; y++) {
    std::vector<double> P(nC2);
    for(int x = hK; x < w - hK; x++) {
      const size_t id = (size_t)x + (size_t)y * w;
      const double xf = (x - hx) / hx, yf = (y - hy) / hy;
      double ax = 1.0;
      int t = 0;
      for(int i = 0; i <= kOrder; i++) {
        double ay = 1.0;
        for(int j = 0; j <= kOrder - i; j++) {
          P[t++] = ax * ay;
          ay *= yf;
        }
        ax *= xf;
      }
      double acc = 0.0;
      for(t = 0; t < nC2; t++) {
        const double* kk = &Kt[(size_t)t * nk];
        double ct = 0.0;
        for(int jj = 0; jj < fK; jj++)
          for(int ii = 0; ii < fK; ii++)
            ct = std::fma(kk[(2 * hK - ii) + (2 * hK - jj) * fK],
                          I[(size_t)(x - hK + ii) + (size_t)(y - hK + jj) * w], ct);
        acc = std::fma(P[t], ct, acc);
      }
      bool anyBad = false;
      for(int jj = 0; jj < fK && !anyBad; jj++)
        for(int ii = 0; ii < fK; ii++)
          anyBad = anyBad || (cmask[(size_t)(x - hK + ii) + (size_t)(y - hK + jj) * w] & BAD_INPUT);
      acc += getBackground(o, x, y, sol);
      acc *= invKernMult;
      o.conv[id] = acc;
      uint16_t nm = cmask[id];
      if(cmask[id] & BAD_INPUT) nm |= BAD_OUTPUT;
      if(anyBad) {
        double aks = 0.0, uks = 0.0;
        for(int jj = 0; jj < fK; jj++)
          for(int ii = 0; ii < fK; ii++) {
            const int tap = (2 * hK - ii) + (2 * hK - jj) * fK;
            double kv = 0.0;
            for(t = 0; t < nC2; t++) kv = std::fma(P[t], Kt[(size_t)t * nk + tap], kv);
            aks += std::fabs(kv);
            if(!(cmask[(size_t)(x - hK + ii) + (size_t)(y - hK + jj) * w] & BAD_INPUT))
              uks += std::fabs(kv);
          }
        if((uks / aks) < (double)0.99f) nm |= BAD_OUTPUT | BAD_CONV;
        else nm |= OK_CONV;
      }
      o.mask[id] = nm;
    }
  }
  for(int y = 0; y < h; y++)
    for(int x = 0; x < w; x++)
      if(!(x >= hK && x < w - hK && y >= hK && y < h - hK)) {
        const size_t id = (size_t)x + (size_t)y * w;
        o.conv[id] = 1e-30;
        if(!o.inMask.empty() && o.inMask[id]) o.mask[id] |= INPUT_MASK | BAD_INPUT | BAD_OUTPUT;
      }
}

// ---------------------------------------------------------- conv + sub ---
// conv: src/bach.cpp:325-413, createConvMask (cl_kern/conv.cl:15-29), conv
// (:31-97), maskAfterConv (:99-113).  sub: src/bach.cpp:415-440 ->
// cl_kern/sub.cl:15-32.
void convSub(xbo_handle& o) {
  const Geo& g = o.g;
  const int w = o.w, h = o.h, fK = g.fK, hK = g.hK, nk = fK * fK;
  const std::vector<double>& I = o.img[o.chosen];
  const std::vector<double>& O = o.img[1 - o.chosen];
  const bool scaleConv = (o.p.normalizeTemplate && o.convTemplate) ||
                         (!o.p.normalizeTemplate && !o.convTemplate);
  const int xSteps = (int)std::ceil(w / (double)fK);
  const int ySteps = (int)std::ceil(h / (double)fK);
  std::vector<double> table((size_t)xSteps * ySteps * nk);
#pragma omp parallel for schedule(dynamic)
  for(int ys = 0; ys < ySteps; ys++)
    for(int xs = 0; xs < xSteps; xs++)
      makeKernel(o, o.solution, xs * fK + hK + hK, ys * fK + hK + hK, false,
                 &table[((size_t)ys * xSteps + xs) * nk]);
  o.kernSum = makeKernel(o, o.solution, w / 2, h / 2, false, nullptr);
  const double invKernSum = 1.0 / o.kernSum;
  const double invKernMult = scaleConv ? invKernSum : 1.0;
  std::vector<uint16_t> cmask((size_t)w * h);
  for(size_t id = 0; id < cmask.size(); id++) {
    double t = I[id];
    uint16_t m = 0;
    if(t == 0.0) m |= BAD_INPUT | BAD_PIX_VAL;
    if(t >= o.p.threshHigh) m |= BAD_INPUT | SAT_PIXEL;
    if(t <= o.p.threshLow) m |= BAD_INPUT | LOW_PIXEL;
    if(!o.inMask.empty() && o.inMask[id]) m |= INPUT_MASK | BAD_INPUT;  // input mask
    cmask[id] = m;
  }
  o.conv.assign((size_t)w * h, 0.0);
  if(o.p.convPerPixel) {
    convPerPixel(o, cmask, invKernMult);
  } else
#pragma omp parallel for schedule(static)
  for(int y = 0; y < h; y++)
    for(int x = 0; x < w; x++) {
      size_t id = (size_t)x + (size_t)y * w;
      if(x >= hK && x < w - hK && y >= hK && y < h - hK) {
        int xS = (x - hK) / fK, yS = (y - hK) / fK;
        const double* kern = &table[((size_t)xS + (size_t)yS * xSteps) * nk];
        double acc = 0.0, aks = 0.0, uks = 0.0;
        int maskAcc = 0;
        for(int j = y - hK; j <= y + hK; j++) {
          int jk = y - j + hK;
          for(int i = x - hK; i <= x + hK; i++) {
            int ik = x - i + hK;
            double kk = kern[ik + jk * fK];
            size_t ii = (size_t)i + (size_t)w * j;
            acc += kk * I[ii];
            maskAcc |= cmask[ii];
            aks += std::fabs(kk);
            if((cmask[ii] & BAD_INPUT) == 0) uks += std::fabs(kk);
          }
        }
        acc += getBackground(o, x, y, o.solution);
        acc *= invKernMult;
        o.conv[id] = acc;
        uint16_t nm = cmask[id];
        if(cmask[id] & BAD_INPUT) nm |= BAD_OUTPUT;
        if(maskAcc != 0) {
          if((uks / aks) < (double)0.99f) nm |= BAD_OUTPUT | BAD_CONV;
          else nm |= OK_CONV;
        }
        o.mask[id] = nm;
      } else {
        o.conv[id] = 1e-30;
        if(!o.inMask.empty() && o.inMask[id]) o.mask[id] |= INPUT_MASK | BAD_INPUT | BAD_OUTPUT;
      }
    }
  for(size_t id = 0; id < cmask.size(); id++) {
    double t = O[id];
    uint16_t m = 0;
    if(t == 0.0) m |= BAD_OUTPUT | BAD_INPUT | BAD_PIX_VAL;
    if(t >= o.p.threshHigh) m |= BAD_OUTPUT | BAD_INPUT | SAT_PIXEL;
    if(t <= o.p.threshLow) m |= BAD_OUTPUT | BAD_INPUT | LOW_PIXEL;
    o.mask[id] |= m;
  }
  const double convFactor = scaleConv ? o.kernSum : 1.0;
  const double finalFactor = scaleConv ? -(1.0 / o.kernSum) : 1.0;
  o.diff.assign((size_t)w * h, 1e-30);
#pragma omp parallel for schedule(static)
  for(int y = 0; y < h; y++)
    for(int x = 0; x < w; x++) {
      size_t id = (size_t)x + (size_t)y * w;
      if(x >= hK && x < w - hK && y >= hK && y < h - hK &&
         (o.mask[id] & BAD_OUTPUT) == 0)
        o.diff[id] = (o.conv[id] * convFactor - O[id]) * finalFactor;
    }
}

// ------------------------------------------------------------------- sss --
// src/bach.cpp:44-170.
int sssPass(xbo_handle& o, AllStamps& st, int passIdx) {
  const int w = o.w, h = o.h;
  st.n = o.stampsx * o.stampsy;
  st.cx.assign(st.n, 0);
  st.cy.assign(st.n, 0);
  st.sx.assign(st.n, 0);
  st.sy.assign(st.n, 0);
  // createStampBounds: cl_kern/sss.cl:19-38
  for(int id = 0; id < st.n; id++) {
    int sxI = id % o.stampsx, syI = id / o.stampsx;
    int startX = sxI * w / o.stampsx, startY = syI * h / o.stampsy;
    int stopX = std::min(startX + o.fStampWidth, w);
    int stopY = std::min(startY + o.fStampWidth, h);
    st.cx[id] = startX;
    st.cy[id] = startY;
    st.sx[id] = stopX - startX;
    st.sy[id] = stopY - startY;
  }
  std::vector<double> sky[2], fwhm[2];
  for(int im = 0; im < 2; im++) {  // identifySStamps: calcStats T then S
    int rc = calcStats(o, st, im, sky[im], fwhm[im]);
    if(rc != XB_OK) return rc;
  }
  const int maxSS = o.g.maxSS;
  for(int im = 0; im < 2; im++) {  // findSStamps T then S
    uint16_t badMask = (uint16_t)(ALL & ~OK_CONV);
    uint16_t badPixelMask, skipMask;
    if(im == 0) {
      badMask &= (uint16_t)~(BAD_PIXEL_S | SKIP_S);
      badPixelMask = BAD_PIXEL_T;
      skipMask = SKIP_T;
    } else {
      badMask &= (uint16_t)~(BAD_PIXEL_T | SKIP_T);
      badPixelMask = BAD_PIXEL_S;
      skipMask = SKIP_S;
    }
    std::vector<SubSt> subs((size_t)st.n * maxSS);
    std::vector<int> cnt(st.n);
#pragma omp parallel for schedule(dynamic)
    for(int s = 0; s < st.n; s++)
      findSubStampsOne(o, st, im, s, sky[im][s], fwhm[im][s], badMask,
                       badPixelMask, skipMask, &subs[(size_t)s * maxSS], &cnt[s]);
    // removeEmptyStamps (src/sssUtil.cpp:106-197): ascending original index
    StampSet& S = o.set[im];
    S = StampSet{};
    for(int s = 0; s < st.n; s++) {
      if(cnt[s] <= 0) continue;
      S.orig.push_back(s);
      S.cx.push_back(st.cx[s]);
      S.cy.push_back(st.cy[s]);
      S.sx.push_back(st.sx[s]);
      S.sy.push_back(st.sy[s]);
      S.sky.push_back(sky[im][s]);
      S.fwhm.push_back(fwhm[im][s]);
      S.count.push_back(cnt[s]);
      S.cur.push_back(0);
      for(int k = 0; k < maxSS; k++)
        S.subs.push_back(k < cnt[s] ? subs[(size_t)s * maxSS + k] : SubSt{});
    }
    S.n = (int)S.orig.size();
    const std::string sfx = std::to_string(im);
    o.put("sky" + sfx, sky[im]);
    o.put("fwhm" + sfx, fwhm[im]);
    o.put("ss_count_all" + sfx, cnt);
    std::vector<int> xy;
    std::vector<double> vals;
    for(auto& q : subs) {
      xy.push_back(q.x);
      xy.push_back(q.y);
      vals.push_back(q.val);
    }
    o.put("ss_xy_all" + sfx, xy);
    o.put("ss_val_all" + sfx, vals);
  }
  (void)passIdx;
  return XB_OK;
}

int runSss(xbo_handle& o) {
  const int w = o.w, h = o.h;
  int fSW = std::min(w / o.stampsx, h / o.stampsy);
  fSW -= o.g.fK;
  fSW -= fSW % 2 == 0 ? 1 : 0;
  if(fSW < o.g.fSS) {
    fSW = o.g.fSS + o.g.fK;
    fSW -= fSW % 2 == 0 ? 1 : 0;
    o.stampsx = w / fSW;
    o.stampsy = h / fSW;
  }
  o.fStampWidth = fSW;
  if(o.stampsx <= 0 || o.stampsy <= 0) return XB_ERR_ARG;
  AllStamps st;
  int rc = sssPass(o, st, 0);
  if(rc != XB_OK) return rc;
  int oldCount = o.stampsx * o.stampsy;
  double fT = (double)o.set[0].n / oldCount, fS = (double)o.set[1].n / oldCount;
  o.scalars["sss_retry"] = 0;
  if(fT < 0.1 || fS < 0.1) {
    o.scalars["sss_retry"] = 1;
    o.p.threshLow *= 0.5;
    for(auto& m : o.mask) m &= (uint16_t)~(SKIP_S | SKIP_T);  // resetSkipMask
    rc = sssPass(o, st, 1);
    o.p.threshLow /= 0.5;
    if(rc != XB_OK) return rc;
  }
  if(o.set[0].n == 0 && o.set[1].n == 0) return XB_ERR_NO_SUBSTAMPS;
  return XB_OK;
}

void allocW(xbo_handle& o, StampSet& S) {
  const Geo& g = o.g;
  S.W.assign((size_t)S.n * g.wRows * g.wCols, 0.0);
  S.Q.assign((size_t)S.n * g.qCount * g.qCount, 0.0);
  S.B.assign((size_t)S.n * g.bCount, 0.0);
  S.omega.assign(o.p.fitWeighted ? (size_t)S.n * g.wCols : 0, 0.0);
}

void snapshotSets(xbo_handle& o) {
  for(int im = 0; im < 2; im++) {
    const StampSet& S = o.set[im];
    const std::string sfx = std::to_string(im);
    std::vector<int> xy;
    std::vector<double> vals;
    for(auto& q : S.subs) {
      xy.push_back(q.x);
      xy.push_back(q.y);
      vals.push_back(q.val);
    }
    o.put("stamp_index" + sfx, S.orig);
    o.put("ss_count" + sfx, S.count);
    o.put("ss_xy" + sfx, xy);
    o.put("ss_val" + sfx, vals);
    o.scalars["nstamps" + sfx] = S.n;
  }
}

}  // namespace

// ================================================================ C API ===
extern "C" {

xbo_handle* xbo_run(const xb_params* p, const double* T, const double* S,
                    int w, int h, int nthreads, int keep_w, int* status) {
  return xbo_run_masked(p, T, S, nullptr, w, h, nthreads, keep_w, status);
}

xbo_handle* xbo_run_masked(const xb_params* p, const double* T, const double* S,
                           const uint8_t* inMask, int w, int h, int nthreads, int keep_w,
                           int* status) {
  auto* o = new xbo_handle();
  if(inMask) o->inMask.assign(inMask, inMask + (size_t)w * h);
#ifdef _OPENMP
  if(nthreads > 0) omp_set_num_threads(nthreads);
  o->scalars["threads"] = nthreads > 0 ? nthreads : omp_get_max_threads();
#else
  (void)nthreads;
  o->scalars["threads"] = 1;
#endif
  o->p = *p;
  o->w = w;
  o->h = h;
  o->keepW = keep_w != 0;
  Geo& g = o->g;
  g.hSS = p->hSStampWidth;
  g.fSS = 2 * g.hSS + 1;
  g.hK = p->hKernelWidth;
  g.fK = 2 * g.hK + 1;
  g.nPSF = xb_params_npsf(p);
  g.nComp1 = g.nPSF - 1;
  g.nComp2 = triNum(p->kernelOrder + 1);
  g.nComp = g.nComp1 * g.nComp2;
  g.nBG = triNum(p->backgroundOrder + 1);
  g.matSize = g.nComp + g.nBG + 1;
  g.nSol = g.nPSF * g.nComp2 + g.nBG + 1;
  g.wRows = g.nPSF + g.nBG;
  g.wCols = g.fSS * g.fSS;
  g.qCount = g.nPSF + 2;
  g.bCount = g.nPSF + 2;
  g.maxSS = 2 * p->maxKSStamps;
  auto fail = [&](int rc) {
    o->status = rc;
    if(status) *status = rc;
    return o;
  };
  if(w <= 0 || h <= 0 || p->stampsx <= 0 || p->stampsy <= 0 || g.nPSF <= 0)
    return fail(XB_ERR_ARG);
  o->img[0].assign(T, T + (size_t)w * h);
  o->img[1].assign(S, S + (size_t)w * h);
  o->stampsx = p->stampsx;
  o->stampsy = p->stampsy;
  auto t0 = std::chrono::steady_clock::now();
  maskInput(*o);
  o->put("mask_init", o->mask);
  o->scalars["ms_ini"] = msSince(t0);
  t0 = std::chrono::steady_clock::now();
  int rc = runSss(*o);
  o->scalars["ms_sss"] = msSince(t0);
  o->scalars["stampsx"] = o->stampsx;
  o->scalars["stampsy"] = o->stampsy;
  o->scalars["fStampWidth"] = o->fStampWidth;
  if(rc != XB_OK) return fail(rc);
  snapshotSets(*o);
  o->put("mask_sss", o->mask);
  t0 = std::chrono::steady_clock::now();
  buildBasis(*o);
  o->put("basis", o->vec);
  for(int im = 0; im < 2; im++) {
    allocW(*o, o->set[im]);
    StampSet& Sset = o->set[im];
#pragma omp parallel for schedule(dynamic)
    for(int s = 0; s < Sset.n; s++) fillStamp(*o, Sset, s, o->img[im], o->img[1 - im]);
    o->put("Q" + std::to_string(im), Sset.Q);
    o->put("B" + std::to_string(im), Sset.B);
    if(o->keepW) o->put("W" + std::to_string(im), Sset.W);
  }
  o->scalars["ms_cmv"] = msSince(t0);
  t0 = std::chrono::steady_clock::now();
  double tMerit = testFit(*o, 0, 0);
  double sMerit = testFit(*o, 1, 1);
  o->scalars["merit0"] = tMerit;
  o->scalars["merit1"] = sMerit;
  o->convTemplate = sMerit > tMerit ? 1 : 0;
  o->chosen = o->convTemplate ? 0 : 1;
  o->scalars["convTemplate"] = o->convTemplate;
  o->scalars["ms_cd"] = msSince(t0);
  t0 = std::chrono::steady_clock::now();
  fitKernel(*o);
  o->scalars["ms_ksc"] = msSince(t0);
  t0 = std::chrono::steady_clock::now();
  convSub(*o);
  o->scalars["ms_conv_sub"] = msSince(t0);
  o->scalars["kernSum"] = o->kernSum;
  o->scalars["singular"] = o->singular;
  o->put("conv", o->conv);
  o->put("diff", o->diff);
  o->put("mask", o->mask);
  if(status) *status = XB_OK;
  return o;
}

int xbo_get_array(const xbo_handle* h, const char* name, void* out, size_t cap,
                  size_t* nbytes) {
  auto it = h->arrays.find(name);
  if(it == h->arrays.end()) return XB_ERR_ARG;
  if(nbytes) *nbytes = it->second.size();
  if(out) std::memcpy(out, it->second.data(), std::min(cap, it->second.size()));
  return XB_OK;
}

int xbo_get_scalar(const xbo_handle* h, const char* name, double* out) {
  auto it = h->scalars.find(name);
  if(it == h->scalars.end()) {
    if(std::string(name) == "status") {
      *out = h->status;
      return XB_OK;
    }
    return XB_ERR_ARG;
  }
  *out = it->second;
  return XB_OK;
}

void xbo_free(xbo_handle* h) { delete h; }

int xbo_stamp_stats(const double* img, uint16_t* mask, int w, int h, const int* geom,
                    int n, int fStampWidth, double sigClipAlpha, double iqRange, double* sky,
                    double* fwhm) {
  xbo_handle o;
  xb_params_default(&o.p);
  o.p.sigClipAlpha = sigClipAlpha;
  o.p.iqRange = iqRange;
  o.w = w;
  o.h = h;
  o.fStampWidth = fStampWidth;
  o.img[0].assign(img, img + (size_t)w * h);
  o.mask.assign(mask, mask + (size_t)w * h);
  AllStamps st;
  st.n = n;
  for(int i = 0; i < n; i++) {
    st.cx.push_back(geom[4 * i]);
    st.cy.push_back(geom[4 * i + 1]);
    st.sx.push_back(geom[4 * i + 2]);
    st.sy.push_back(geom[4 * i + 3]);
  }
  std::vector<double> sk, fw;
  const int rc = calcStats(o, st, 0, sk, fw);
  if(rc != XB_OK) return rc;
  std::copy(sk.begin(), sk.end(), sky);
  std::copy(fw.begin(), fw.end(), fwhm);
  std::copy(o.mask.begin(), o.mask.end(), mask);
  return XB_OK;
}

void xbo_sigma_clip(const double* data, int n, int maxIter, double alpha,
                    double* mean, double* stdDev) {
  sigmaClip(data, n, mean, stdDev, maxIter, alpha);
}

void xbo_ran1_seq(int idum, int n, double* out) {
  Ran1 r(idum);
  for(int i = 0; i < n; i++) out[i] = r.next();
}

int xbo_lu_solve(double* a, int n, double* rhs) {
  std::vector<int> idx(n + 1, 0);
  int rc = ludcmp(a, n, idx.data(), false);
  lubksb(a, n, idx.data(), rhs);
  return rc;
}

// The oracle carries its own copies of the two parameter helpers so that it
// links without the product library.
void xb_params_default(xb_params* p) {
  std::memset(p, 0, sizeof(*p));
  p->stampsx = 10;
  p->stampsy = 10;
  p->threshLow = 0.0;
  p->threshHigh = 25000.0;
  p->threshKernFit = 20.0;
  p->sigKernFit = 2.0;
  p->sigClipAlpha = 3.0;
  p->iqRange = 1.35;
  p->maxKSStamps = 3;
  p->hSStampWidth = 15;
  p->hKernelWidth = 10;
  p->inSpreadMaskFactor = 1.0;
  p->normalizeTemplate = 1;
  p->backgroundOrder = 1;
  p->kernelOrder = 2;
  p->nGauss = 3;
  p->dg[0] = 6;
  p->dg[1] = 4;
  p->dg[2] = 2;
  p->bg[0] = (float)(1.0 / (2.0 * 0.7 * 0.7));
  p->bg[1] = (float)(1.0 / (2.0 * 1.5 * 1.5));
  p->bg[2] = (float)(1.0 / (2.0 * 3.0 * 3.0));
  p->mode = XB_MODE_PLAIN;
  p->verbose = 0;
}

int xb_params_npsf(const xb_params* p) {
  int n = 0;
  for(int i = 0; i < p->nGauss && i < XB_MAX_GAUSS; i++)
    n += (p->dg[i] + 1) * (p->dg[i] + 2) / 2;
  return n;
}

}  // extern "C"
