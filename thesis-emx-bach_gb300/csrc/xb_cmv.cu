// xb_cmv.cu — the cmv stage (src/bach.cpp:172-268, src/cmvUtil.cpp):
// Gaussian-basis convolutions of every current substamp (W), the per-stamp
// Gram matrix Q and the projection B.
//
// Plain mode keeps the reference's precision choices: the Y pass
// accumulates in FP32 over FP64 products (cl_kern/cmv.cl:70-106), the X pass
// in FP64 (:108-135), Q and B are FP64 dot products in the reference's
// summation order (createQ :195-215 ascending pixel index, createB :217-248
// column-major).  Basis functions sharing a bit-identical Y filter share one
// Y pass.

#include <algorithm>

#include "xb_internal.h"

namespace xb {

namespace {

constexpr int FILL_THREADS = 256;

// (x - (w * 0.5f)) / (w * 0.5f) evaluated in float (cl_kern/cmv.cl:180).
__device__ __forceinline__ double floatNorm(int x, int w) {
  float hw = (float)w * 0.5f;
  float r = ((float)x - hw) / hw;
  return (double)r;
}
__device__ __forceinline__ double ipow(double x, int n) {
  double r = 1.0;
  for(int i = 0; i < n; i++) r *= x;
  return r;
}

// Y then X pass for one (stamp, Y-filter group).
template <class T>
__global__ void __launch_bounds__(FILL_THREADS)
    k_fill_w(const T* __restrict__ img, int w, int h, const int* __restrict__ list,
             const int* __restrict__ count, const int* __restrict__ cur,
             const int2* __restrict__ ssxy, int maxSS, const double* __restrict__ fX,
             const double* __restrict__ fY, const int* __restrict__ gStart,
             const int* __restrict__ gMembers, int hSS, int hK, int wRows,
             double* __restrict__ W) {
  extern __shared__ unsigned char fill_s[];
  const int s = list[blockIdx.x], gi = blockIdx.y, tid = threadIdx.x;
  const int fK = 2 * hK + 1, fSS = 2 * hSS + 1, wCols = fSS * fSS;
  const int xHalf = hSS + hK, tw = 2 * xHalf + 1, th = fSS;
  const int m0 = gStart[gi], m1 = gStart[gi + 1];
  double* Ws = W + (size_t)s * wRows * wCols;
  const bool live = cur[s] < count[s];
  if(!live) {
    for(int m = m0; m < m1; m++) {
      const int n = gMembers[m];
      for(int p = tid; p < wCols; p += FILL_THREADS) Ws[(size_t)n * wCols + p] = 0.0;
    }
    return;
  }
  const int2 c = ssxy[(size_t)s * maxSS + cur[s]];
  float* win = (float*)fill_s;                 // tw x tw, rows y, cols x
  float* tmp = win + tw * tw;                  // th x tw
  const int off = tw * tw + th * tw;
  double* fy = (double*)(win + off + (off & 1));  // 8-byte aligned
  double* fx = fy + fK;
  const int n0 = gMembers[m0];
  for(int i = tid; i < fK; i += FILL_THREADS) fy[i] = fY[(size_t)n0 * fK + i];
  // input window: x in [ssx - xHalf, ssx + xHalf], y in [ssy - xHalf, ssy + xHalf]
  for(int i = tid; i < tw * tw; i += FILL_THREADS) {
    int lx = i % tw, ly = i / tw;
    // substamp centres keep hSS+hK from the frame edge (the border mask of
    // maskInput); the clamp only guards the address
    int gx = min(max(c.x - xHalf + lx, 0), w - 1);
    int gy = min(max(c.y - xHalf + ly, 0), h - 1);
    win[i] = (float)img[(size_t)gx + (size_t)gy * w];
  }
  __syncthreads();
  // Y pass (cmv.cl:70-106): v accumulates in float, products in double
  for(int p = tid; p < th * tw; p += FILL_THREADS) {
    const int row = p / tw, col = p % tw;
    float v = 0.0f;
    for(int y = -hK; y <= hK; y++)
      v = (float)((double)v + (double)win[(row + hK + y) * tw + col] * fy[hK - y]);
    tmp[p] = v;
  }
  __syncthreads();
  for(int m = m0; m < m1; m++) {
    const int n = gMembers[m];
    for(int i = tid; i < fK; i += FILL_THREADS) fx[i] = fX[(size_t)n * fK + i];
    __syncthreads();
    // X pass (cmv.cl:108-135)
    for(int p = tid; p < wCols; p += FILL_THREADS) {
      const int row = p / fSS, ii = p % fSS;
      double w0 = 0.0;
      for(int x = -hK; x <= hK; x++) w0 += (double)tmp[row * tw + ii + x + hK] * fx[hK - x];
      Ws[(size_t)n * wCols + p] = w0;
    }
    __syncthreads();
  }
}

// convStampOdd (cmv.cl:137-154) and convStampBg (:156-193).
__global__ void __launch_bounds__(FILL_THREADS)
    k_fill_finish(const int* __restrict__ list, const int* __restrict__ count,
                  const int* __restrict__ cur, const int2* __restrict__ ssxy, int maxSS,
                  const int* __restrict__ kx, const int* __restrict__ ky, int nPSF,
                  const int2* __restrict__ bgXY, int nBG, int hSS, int w, int h,
                  int wRows, double* __restrict__ W) {
  const int s = list[blockIdx.x], tid = threadIdx.x;
  const int fSS = 2 * hSS + 1, wCols = fSS * fSS;
  double* Ws = W + (size_t)s * wRows * wCols;
  const bool live = cur[s] < count[s];
  for(int n = 1; n < nPSF; n++) {
    if(kx[n] % 2 != 0 || ky[n] % 2 != 0) continue;
    for(int p = tid; p < wCols; p += FILL_THREADS) Ws[(size_t)n * wCols + p] -= Ws[p];
  }
  int2 c = make_int2(0, 0);
  if(live) c = ssxy[(size_t)s * maxSS + cur[s]];
  for(int b = 0; b < nBG; b++)
    for(int p = tid; p < wCols; p += FILL_THREADS) {
      double a = 0.0;
      if(live) {
        int x = c.x - hSS + p % fSS, y = c.y - hSS + p / fSS;
        double xf = floatNorm(x, w), yf = floatNorm(y, h);
        a = ipow(xf, bgXY[b].x) * ipow(yf, bgXY[b].y);
      }
      Ws[(size_t)(nPSF + b) * wCols + p] = a;
    }
}

// createQ (cmv.cl:195-215) and createB (:217-248) for one stamp per CTA.
// Q: each thread owns up to GQ_E lower-triangle entries and accumulates them
// over K in ascending order while W tiles stream through shared memory.
constexpr int GQ_KT = 32, GQ_E = 8;
template <class T>
__global__ void __launch_bounds__(FILL_THREADS)
    k_gram_qb(const T* __restrict__ other, const T* __restrict__ conv, int w, int h,
              const int* __restrict__ list,
              const int* __restrict__ count, const int* __restrict__ cur,
              const int2* __restrict__ ssxy, int maxSS, int hSS, int wRows, int qCount,
              const double* __restrict__ W, double* __restrict__ Q, double* __restrict__ B,
              double invGain, double rn2x2, double* __restrict__ omega) {
  extern __shared__ double gq_s[];
  const int s = list[blockIdx.x], tid = threadIdx.x;
  const int fSS = 2 * hSS + 1, wCols = fSS * fSS;
  const int R = qCount - 1;                 // W rows 0..R-1 enter Q
  const int nEnt = R * (R + 1) / 2;
  const double* Ws = W + (size_t)s * wRows * wCols;
  double* Qs = Q + (size_t)s * qCount * qCount;
  double* Bs = B + (size_t)s * qCount;
  double* tile = gq_s;                      // R x (GQ_KT + 1)
  double* sub = gq_s + R * (GQ_KT + 1);     // fSS * fSS image values
  double* om = sub + wCols;                 // fSS * fSS pixel weights (weighted fit)
  const bool live = cur[s] < count[s];
  if(omega) {
    // weights of the current substamp's pixels (exhausted stamps: zero)
    const int2 c = live ? ssxy[(size_t)s * maxSS + cur[s]] : make_int2(0, 0);
    for(int i = tid; i < wCols; i += FILL_THREADS) {
      double v = 0.0;
      if(live) {
        const int gx = min(max(i % fSS - hSS + c.x, 0), w - 1);
        const int gy = min(max(i / fSS - hSS + c.y, 0), h - 1);
        const size_t id = (size_t)gx + (size_t)gy * w;
        v = fitWeight((double)conv[id], (double)other[id], invGain, rn2x2);
      }
      om[i] = v;
      omega[(size_t)s * wCols + i] = v;
    }
  }
  int ei[GQ_E], ej[GQ_E];
  double acc[GQ_E];
#pragma unroll
  for(int e = 0; e < GQ_E; e++) {
    int idx = tid + e * FILL_THREADS;
    acc[e] = 0.0;
    ei[e] = -1;
    ej[e] = 0;
    if(idx < nEnt) {
      // idx -> (i, j), i >= j, row-major lower triangle
      int i = (int)((sqrt(8.0 * idx + 1.0) - 1.0) * 0.5);
      while((i + 1) * (i + 2) / 2 <= idx) i++;
      while(i * (i + 1) / 2 > idx) i--;
      ei[e] = i;
      ej[e] = idx - i * (i + 1) / 2;
    }
  }
  for(int k0 = 0; k0 < wCols; k0 += GQ_KT) {
    const int kt = min(GQ_KT, wCols - k0);
    for(int i = tid; i < R * GQ_KT; i += FILL_THREADS) {
      int r = i / GQ_KT, kk = i % GQ_KT;
      tile[r * (GQ_KT + 1) + kk] = kk < kt ? Ws[(size_t)r * wCols + k0 + kk] : 0.0;
    }
    __syncthreads();
#pragma unroll
    for(int e = 0; e < GQ_E; e++) {
      if(ei[e] < 0) continue;
      const double* a = tile + ei[e] * (GQ_KT + 1);
      const double* b = tile + ej[e] * (GQ_KT + 1);
      double q = acc[e];
      if(omega) {
        for(int kk = 0; kk < kt; kk++) q += a[kk] * (b[kk] * om[k0 + kk]);
      } else {
        for(int kk = 0; kk < kt; kk++) q += a[kk] * b[kk];
      }
      acc[e] = q;
    }
    __syncthreads();
  }
  // Q buffer: entry (i+1, j+1) for the triangle, zero elsewhere
  for(int i = tid; i < qCount * qCount; i += FILL_THREADS) Qs[i] = 0.0;
  __syncthreads();
#pragma unroll
  for(int e = 0; e < GQ_E; e++)
    if(ei[e] >= 0) Qs[(size_t)(ei[e] + 1) * qCount + (ej[e] + 1)] = acc[e];
  // B: W[i-1] . other image, x outer / y inner (column-major)
  if(live) {
    const int2 c = ssxy[(size_t)s * maxSS + cur[s]];
    for(int i = tid; i < wCols; i += FILL_THREADS) {
      int x = i % fSS - hSS, y = i / fSS - hSS;
      int gx = min(max(x + c.x, 0), w - 1), gy = min(max(y + c.y, 0), h - 1);
      sub[i] = (double)other[(size_t)gx + (size_t)gy * w];
    }
  }
  __syncthreads();
  for(int i = tid; i < qCount; i += FILL_THREADS) {
    double p0 = 0.0;
    if(live && i > 0) {
      const double* wr = Ws + (size_t)(i - 1) * wCols;
      for(int x = 0; x < fSS; x++)
        for(int y = 0; y < fSS; y++) {
          int k = x + fSS * y;
          p0 += omega ? wr[k] * (sub[k] * om[k]) : wr[k] * sub[k];
        }
    }
    Bs[i] = p0;
  }
}

}  // namespace

// Refill W, Q and B of the listed stamps of set `si`, convolving image
// `imgConv` and projecting on the other image (fillStamps,
// src/cmvUtil.cpp:37-187).
void fillStamps(xb_ctx* c, int si, const int* dList, int nList, int imgConv, const int* liveN) {
  if(nList <= 0) return;
  if(mixedMode(c)) {
    fillStampsMixed(c, si, dList, nList, imgConv, liveN);
    return;
  }
  if(liveN) throw XbError{XB_ERR_STATE, "device-counted fills are a mixed-mode path"};
  const Geo& g = c->g;
  StampSetDev& S = c->set[si];
  const int nGroups = (int)c->basis.yGroupStart.size() - 1;
  const int tw = 2 * (g.hSS + g.hK) + 1, th = g.fSS;
  size_t smemFill = (size_t)(tw * tw + th * tw + 2) * sizeof(float) + 2 * g.fK * sizeof(double);
  dim3 grid(nList, nGroups);
  double* W = (double*)S.W;
  { KT_SCOPE(c, "fill_w");
  if(c->imgIsF64)
    k_fill_w<double><<<grid, FILL_THREADS, smemFill, c->stream>>>(
        (const double*)c->img[imgConv], c->w, c->h, dList, S.count, S.cur, S.ssxy, g.maxSS, c->dFX,
        c->dFY, c->dYGroupStart, c->dYGroupMembers, g.hSS, g.hK, g.wRows, W);
  else
    k_fill_w<float><<<grid, FILL_THREADS, smemFill, c->stream>>>(
        (const float*)c->img[imgConv], c->w, c->h, dList, S.count, S.cur, S.ssxy, g.maxSS, c->dFX,
        c->dFY, c->dYGroupStart, c->dYGroupMembers, g.hSS, g.hK, g.wRows, W);
  XB_LAUNCHED(c);
  }
  int2* bgXY = buf<int2>(c, "bgXY", g.nBG);
  { KT_SCOPE(c, "fill_finish");
  k_fill_finish<<<nList, FILL_THREADS, 0, c->stream>>>(dList, S.count, S.cur, S.ssxy, g.maxSS,
                                                       c->dKx, c->dKy, g.nPSF, bgXY, g.nBG,
                                                       g.hSS, c->w, c->h, g.wRows, W);
  XB_LAUNCHED(c);
  }
  size_t smemGram = ((size_t)(g.qCount - 1) * (GQ_KT + 1) + 2 * (size_t)g.wCols) * sizeof(double);
  const double invGain = noiseInvGain(c->p), rn2x2 = noiseRn2x2(c->p);
  double* omega = c->p.fitWeighted ? S.omega : nullptr;
  const int other = 1 - imgConv;
  { KT_SCOPE(c, "gram_qb");
  if(c->imgIsF64)
    k_gram_qb<double><<<nList, FILL_THREADS, smemGram, c->stream>>>(
        (const double*)c->img[other], (const double*)c->img[imgConv], c->w, c->h, dList, S.count,
        S.cur, S.ssxy, g.maxSS, g.hSS, g.wRows, g.qCount, W, S.Q, S.B, invGain, rn2x2, omega);
  else
    k_gram_qb<float><<<nList, FILL_THREADS, smemGram, c->stream>>>(
        (const float*)c->img[other], (const float*)c->img[imgConv], c->w, c->h, dList, S.count,
        S.cur, S.ssxy, g.maxSS, g.hSS, g.wRows, g.qCount, W, S.Q, S.B, invGain, rn2x2, omega);
  XB_LAUNCHED(c);
  }
}

void stageCmv(xb_ctx* c) {
  const Geo& g = c->g;
  if((g.qCount - 1) * (g.qCount) / 2 > GQ_E * FILL_THREADS)
    throw XbError{XB_ERR_UNSUPPORTED, "too many basis functions for the Gram kernel"};
  // basis tables (host-built once per context) and background exponents
  std::vector<int2> bg(g.nBG);
  for(int b = 0; b < g.nBG; b++) bg[b] = make_int2(c->basis.bgX[b], c->basis.bgY[b]);
  toDevice(c, buf<int2>(c, "bgXY", g.nBG), bg);
  for(int si = 0; si < 2; si++) {
    StampSetDev& S = c->set[si];
    const std::string sfx = std::to_string(si);
    if(mixedMode(c)) {
      S.Wf = buf<float>(c, "Wf" + sfx, (size_t)std::max(S.n, 1) * g.wRows * mixedLd(g));
      S.Wlo = buf<float>(c, "Wlo" + sfx, (size_t)std::max(S.n, 1) * g.wRows * mixedLd(g));
      S.dots = buf<double>(c, "dots" + sfx, (size_t)std::max(S.n, 1) * mixedDotStride(g));
    } else {
      S.W = buf<double>(c, "W" + sfx, (size_t)std::max(S.n, 1) * g.wRows * g.wCols);
      S.omega = c->p.fitWeighted ? buf<double>(c, "omega" + sfx, (size_t)std::max(S.n, 1) * g.wCols)
                                 : nullptr;
    }
    S.Q = buf<double>(c, "Q" + sfx, (size_t)std::max(S.n, 1) * g.qCount * g.qCount);
    S.B = buf<double>(c, "B" + sfx, (size_t)std::max(S.n, 1) * g.bCount);
    std::vector<int> all(S.n);
    for(int s = 0; s < S.n; s++) all[s] = s;
    int* dList = buf<int>(c, "fillList" + sfx, std::max(S.n, 1));
    toDevice(c, dList, all);
    fillStamps(c, si, dList, S.n, si, S.dN);
  }
  if(c->trace) {
    for(int si = 0; si < 2; si++) {
      const StampSetDev& S = c->set[si];
      const std::string sfx = std::to_string(si);
      c->put("Q" + sfx, toHost(c, S.Q, (size_t)S.n * g.qCount * g.qCount));
      c->put("B" + sfx, toHost(c, S.B, (size_t)S.n * g.bCount));
      if(mixedMode(c)) {
        c->put("Wf" + sfx, toHost(c, S.Wf, (size_t)S.n * g.wRows * mixedLd(g)));
        c->put("Wlo" + sfx, toHost(c, S.Wlo, (size_t)S.n * g.wRows * mixedLd(g)));
      }
      else
        c->put("W" + sfx, toHost(c, (const double*)S.W, (size_t)S.n * g.wRows * g.wCols));
    }
  }
}

}  // namespace xb
