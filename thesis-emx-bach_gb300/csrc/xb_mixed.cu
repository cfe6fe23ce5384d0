// xb_mixed.cu — the mixed-precision (chosen) path, XB_MODE_MIXED.
//
// Same stages, same decisions logic, different arithmetic:
//   * basis convolutions of the substamps in FP32 FMA, W kept in FP32;
//   * one Gram matrix per stamp of the W rows plus the projected image row
//     (FP32 accumulation), scattered into Q, B and the dot products the
//     global normal matrix needs (createQ/createB/createMatrix terms);
//   * the global system in FP64: LU with fused multiply-adds on a 16-CTA
//     thread-block cluster, triangular solves by column sweeps, and one
//     iterative-refinement step with an FP64 residual;
//   * the chi^2 model in FP32 (the reference already stores it in FP32,
//     cl_kern/cd.cl:489-531);
//   * the full-frame convolution in FP32: 4, 6 or 8 kernel blocks per CTA,
//     a 7 x 3 pixel tile per thread held in registers.
// Statistics, substamp search and the per-stamp test fits are shared with the
// plain path.

#include <cooperative_groups.h>

#include <algorithm>
#include <atomic>
#include <climits>

#include "xb_df.cuh"
#include "xb_device.cuh"
#include "xb_internal.h"

namespace cg = cooperative_groups;

namespace xb {

namespace {

constexpr int MX_THREADS = 256;

using df::dfAccum;
using df::dfNorm;
using df::dfSub;
using df::floatNormF;
using df::refStepY;
using df::splitF64;

// One CTA per (stamp, group of basis functions sharing a Y filter).
template <class T>
__global__ void __launch_bounds__(MX_THREADS)
    k_fill_w_f32(const T* __restrict__ img, int w, int h, const int* __restrict__ list,
                 const int* __restrict__ liveN, const int* __restrict__ count, const int* __restrict__ cur,
                 const int2* __restrict__ ssxy, int maxSS, const double* __restrict__ fX,
                 const double* __restrict__ fY, const int* __restrict__ gStart,
                 const int* __restrict__ gMembers, int hSS, int hK, int wRows, int ldW,
                 float* __restrict__ W, float* __restrict__ Wlo) {
  extern __shared__ float fw_s[];
  if(liveN && (int)blockIdx.x >= *liveN) return;
  const int s = list[blockIdx.x], gi = blockIdx.y, tid = threadIdx.x;
  const int fK = 2 * hK + 1, fSS = 2 * hSS + 1, wCols = fSS * fSS;
  const int xHalf = hSS + hK, tw = 2 * xHalf + 1, th = fSS;
  const int m0 = gStart[gi], m1 = gStart[gi + 1];
  float* Ws = W + (size_t)s * wRows * ldW;
  float* Wl = Wlo + (size_t)s * wRows * ldW;
  const bool live = cur[s] < count[s];
  if(!live) {
    for(int m = m0; m < m1; m++)
      for(int p = tid; p < ldW; p += MX_THREADS) {
        Ws[(size_t)gMembers[m] * ldW + p] = 0.f;
        Wl[(size_t)gMembers[m] * ldW + p] = 0.f;
      }
    return;
  }
  const int2 c = ssxy[(size_t)s * maxSS + cur[s]];
  float* win = fw_s;              // tw * tw
  float* tmp = win + tw * tw;     // th * tw
  float* fyh = tmp + th * tw;     // fK
  float* fyl = fyh + fK;          // fK
  float* fxh = fyl + fK;          // fK
  float* fxl = fxh + fK;          // fK
  const int n0 = gMembers[m0];
  for(int i = tid; i < fK; i += MX_THREADS) splitF64(fY[(size_t)n0 * fK + i], fyh[i], fyl[i]);
  for(int i = tid; i < tw * tw; i += MX_THREADS) {
    int gx = min(max(c.x - xHalf + i % tw, 0), w - 1);
    int gy = min(max(c.y - xHalf + i / tw, 0), h - 1);
    win[i] = (float)img[(size_t)gx + (size_t)gy * w];
  }
  __syncthreads();
  for(int p = tid; p < th * tw; p += MX_THREADS) {
    const int row = p / tw, col = p % tw;
    float v = 0.f;
#pragma unroll 7
    for(int y = -hK; y <= hK; y++) v = refStepY(v, win[(row + hK + y) * tw + col], fyh[hK - y], fyl[hK - y]);
    tmp[p] = v;
  }
  for(int m = m0; m < m1; m++) {
    const int n = gMembers[m];
    __syncthreads();
    for(int i = tid; i < fK; i += MX_THREADS) splitF64(fX[(size_t)n * fK + i], fxh[i], fxl[i]);
    __syncthreads();
    for(int p = tid; p < ldW; p += MX_THREADS) {
      float hi = 0.f, lo = 0.f;
      if(p < wCols) {
        const int row = p / fSS, ii = p % fSS;
        float sh = 0.f, sl = 0.f;
#pragma unroll 7
        for(int x = -hK; x <= hK; x++) dfAccum(sh, sl, tmp[row * tw + ii + x + hK], fxh[hK - x], fxl[hK - x]);
        dfNorm(sh, sl, hi, lo);
      }
      Ws[(size_t)n * ldW + p] = hi;
      Wl[(size_t)n * ldW + p] = lo;
    }
  }
}

// convStampOdd and convStampBg on the hi + lo pair; pads the background rows.
__global__ void __launch_bounds__(MX_THREADS)
    k_fill_finish_f32(const int* __restrict__ list, const int* __restrict__ liveN,
                      const int* __restrict__ count,
                      const int* __restrict__ cur, const int2* __restrict__ ssxy, int maxSS,
                      const int* __restrict__ kx, const int* __restrict__ ky, int nPSF,
                      const int2* __restrict__ bgXY, int nBG, int hSS, int w, int h, int wRows,
                      int ldW, float* __restrict__ W, float* __restrict__ Wlo) {
  if(liveN && (int)blockIdx.x >= *liveN) return;
  const int s = list[blockIdx.x], tid = threadIdx.x;
  const int fSS = 2 * hSS + 1, wCols = fSS * fSS;
  float* Ws = W + (size_t)s * wRows * ldW;
  float* Wl = Wlo + (size_t)s * wRows * ldW;
  const bool live = cur[s] < count[s];
  // W[n] -= W[0] for the even/even rows: each thread takes its pixels
  // through all such rows (independent loads in flight, not one pass per row)
  __shared__ short evenRows[MAX_NPSF];
  __shared__ int nEven;
  if(tid == 0) {
    int m = 0;
    for(int n = 1; n < nPSF; n++)
      if(kx[n] % 2 == 0 && ky[n] % 2 == 0) evenRows[m++] = (short)n;
    nEven = m;
  }
  __syncthreads();
  const int ne = nEven;
  for(int p = tid; p < wCols; p += MX_THREADS) {
    const float bh = Ws[p], bl = Wl[p];
#pragma unroll 4
    for(int e = 0; e < ne; e++) {
      const size_t i = (size_t)evenRows[e] * ldW + p;
      float hi, lo;
      dfSub(Ws[i], Wl[i], bh, bl, hi, lo);
      Ws[i] = hi;
      Wl[i] = lo;
    }
  }
  int2 c = make_int2(0, 0);
  if(live) c = ssxy[(size_t)s * maxSS + cur[s]];
  for(int b = 0; b < nBG; b++)
    for(int p = tid; p < ldW; p += MX_THREADS) {
      double a = 0.0;
      if(live && p < wCols) {
        // the reference's form: float-normalised coordinates, FP64 powers
        const double xf = (double)floatNormF(c.x - hSS + p % fSS, w);
        const double yf = (double)floatNormF(c.y - hSS + p / fSS, h);
        double ax = 1.0, ay = 1.0;
        for(int i = 0; i < bgXY[b].x; i++) ax *= xf;
        for(int i = 0; i < bgXY[b].y; i++) ay *= yf;
        a = ax * ay;
      }
      float hi, lo;
      splitF64(a, hi, lo);
      Ws[(size_t)(nPSF + b) * ldW + p] = hi;
      Wl[(size_t)(nPSF + b) * ldW + p] = lo;
    }
}

// ------------------------------------------------------------------ Gram ---
// G = X X^T with X = [W rows; image row] over the substamp pixels, on the
// CUDA cores in FP64 (the weighted fit and shapes beyond the tensor-core
// kernel).  Each W element hi + lo is exact in FP64; the normal matrices are
// ill-conditioned (cond ~1e14), and an FP32 accumulation moves the fitted
// kernel sum by up to 9 %.  Each stamp's lower triangle is split over
// gridDim.y CTAs; k_gram_scatter then fills Q (createQ), B (createB) and the
// global-matrix dot table.
constexpr int GM_KT = 32, GM_SPLIT = 6;
template <class T>
__global__ void __launch_bounds__(MX_THREADS)
    k_gram_mixed(const T* __restrict__ other, const T* __restrict__ conv, int w, int h,
                 const int* __restrict__ list,
                 const int* __restrict__ liveN, const int* __restrict__ count, const int* __restrict__ cur,
                 const int2* __restrict__ ssxy, int maxSS, int hSS, int wRows, int ldW,
                 const float* __restrict__ W, const float* __restrict__ Wlo,
                 double* __restrict__ Gout, int weighted, double invGain, double rn2x2) {
  extern __shared__ double gm_s[];
  __shared__ double omT[GM_KT];  // pixel weights of the tile (weighted fit)
  if(liveN && (int)blockIdx.x >= *liveN) return;
  const int t = blockIdx.x, s = list[t], tid = threadIdx.x;
  const int fSS = 2 * hSS + 1, wCols = fSS * fSS, R = wRows + 1;
  const int nEnt = R * (R + 1) / 2;
  const int per = (nEnt + gridDim.y - 1) / gridDim.y, e0 = blockIdx.y * per;
  double* tile = gm_s;  // R x (GM_KT + 1)
  const float* Ws = W + (size_t)s * wRows * ldW;
  const float* Wl = Wlo + (size_t)s * wRows * ldW;
  const bool live = cur[s] < count[s];
  int2 c = make_int2(0, 0);
  if(live) c = ssxy[(size_t)s * maxSS + cur[s]];
  int ei = -1, ej = 0;
  const int idx = e0 + tid;
  if(tid < per && idx < nEnt) {
    int i = (int)((sqrtf(8.f * idx + 1.f) - 1.f) * 0.5f);
    while((i + 1) * (i + 2) / 2 <= idx) i++;
    while(i * (i + 1) / 2 > idx) i--;
    ei = i;
    ej = idx - i * (i + 1) / 2;
  }
  double acc = 0.0;
  for(int k0 = 0; k0 < wCols; k0 += GM_KT) {
    const int kt = min(GM_KT, wCols - k0);
    for(int i = tid; i < R * GM_KT; i += MX_THREADS) {
      const int r = i / GM_KT, kk = i % GM_KT;
      double v = 0.0;
      if(kk < kt) {
        if(r < wRows) {
          v = (double)Ws[(size_t)r * ldW + k0 + kk] + (double)Wl[(size_t)r * ldW + k0 + kk];
        } else if(live) {
          const int k = k0 + kk;
          const int gx = min(max(c.x - hSS + k % fSS, 0), w - 1);
          const int gy = min(max(c.y - hSS + k / fSS, 0), h - 1);
          v = (double)(float)other[(size_t)gx + (size_t)gy * w];
        }
      }
      tile[r * (GM_KT + 1) + kk] = v;
    }
    if(weighted && tid < GM_KT) {
      double v = 0.0;
      if(tid < kt && live) {
        const int k = k0 + tid;
        const int gx = min(max(c.x - hSS + k % fSS, 0), w - 1);
        const int gy = min(max(c.y - hSS + k / fSS, 0), h - 1);
        const size_t id = (size_t)gx + (size_t)gy * w;
        v = fitWeight((double)conv[id], (double)other[id], invGain, rn2x2);
      }
      omT[tid] = v;
    }
    __syncthreads();
    if(ei >= 0) {
      const double* a = tile + ei * (GM_KT + 1);
      const double* b = tile + ej * (GM_KT + 1);
      if(weighted) {
        for(int kk = 0; kk < kt; kk++) acc = fma(a[kk], b[kk] * omT[kk], acc);
      } else {
        for(int kk = 0; kk < kt; kk++) acc = fma(a[kk], b[kk], acc);
      }
    }
    __syncthreads();
  }
  if(ei >= 0) {
    double* G = Gout + (size_t)t * R * R;
    G[ei * R + ej] = acc;
    G[ej * R + ei] = acc;
  }
}

__global__ void __launch_bounds__(MX_THREADS)
    k_gram_scatter(const int* __restrict__ list, const int* __restrict__ liveN,
                   const int* __restrict__ count,
                   const int* __restrict__ cur, int wRows, int nPSF, int nBG, int qc,
                   const double* __restrict__ Gin, double* __restrict__ Q,
                   double* __restrict__ B, double* __restrict__ dots, int stride) {
  if(liveN && (int)blockIdx.x >= *liveN) return;
  const int t = blockIdx.x, s = list[t], tid = threadIdx.x, R = wRows + 1;
  const double* G = Gin + (size_t)t * R * R;
  const bool live = cur[s] < count[s];
  double* Qs = Q + (size_t)s * qc * qc;
  for(int i = tid; i < qc * qc; i += MX_THREADS) {
    const int a = i / qc, b = i % qc;
    Qs[i] = (a > 0 && b > 0 && b <= a) ? G[(a - 1) * R + (b - 1)] : 0.0;
  }
  for(int i = tid; i < qc; i += MX_THREADS)
    B[(size_t)s * qc + i] = (i > 0 && live) ? G[wRows * R + (i - 1)] : 0.0;
  double* d = dots + (size_t)s * stride;
  const int nC1 = nPSF - 1, nKB = nC1 * nBG;
  for(int i = tid; i < stride; i += MX_THREADS) {
    double v = 0.0;
    if(i < nKB) {
      v = G[(nPSF + i % nBG) * R + (1 + i / nBG)];
    } else if(i < nKB + nBG) {
      v = G[(nPSF + (i - nKB)) * R + 0];
    } else if(i < nKB + nBG + nBG * nBG) {
      const int e = i - nKB - nBG, ib = e / nBG, jb = e % nBG;
      v = jb <= ib ? G[(nPSF + ib) * R + (nPSF + jb)] : 0.0;
    } else {
      const int ib = (i - nKB - nBG - nBG * nBG) % nBG;  // both RHS forms
      v = live ? G[wRows * R + (nPSF + ib)] : 0.0;
    }
    d[i] = v;
  }
}

// ---------------------------------------------------- chi^2, FP32 model ---
template <class T>
__global__ void __launch_bounds__(MX_THREADS)
    k_sigs_f32(const int* __restrict__ list, const int* __restrict__ liveN,
               const int* __restrict__ count,
               const int* __restrict__ cur, const int2* __restrict__ ssxy, int maxSS,
               const float* __restrict__ W, int wRows, int ldW, int hSS, int nPSF, int kOrder,
               int bgOrder, int nComp, const double* __restrict__ sol, const T* __restrict__ tImg,
               const T* __restrict__ sImg, uint16_t* __restrict__ mask, int w, int h,
               float invGain, float rn2x2, double* __restrict__ sig) {
  __shared__ double coeff[MAX_NPSF];
  __shared__ float cHi[MAX_NPSF], cLo[MAX_NPSF];
  __shared__ double sBg;
  __shared__ double rs[MX_THREADS / 32];
  __shared__ int rc[MX_THREADS / 32];
  if(liveN && (int)blockIdx.x >= *liveN) return;
  const int t = blockIdx.x, s = list[t], tid = threadIdx.x;
  const int fSS = 2 * hSS + 1, pix = fSS * fSS;
  const bool live = cur[s] < count[s];
  int2 c = make_int2(0, 0);
  if(live) c = ssxy[(size_t)s * maxSS + cur[s]];
  if(live) {
    const double xf = (c.x - w * 0.5) / (w * 0.5), yf = (c.y - h * 0.5) / (h * 0.5);
    const int nC2 = (kOrder + 1) * (kOrder + 2) / 2;
    for(int i = tid; i < nPSF; i += MX_THREADS) {
      double cc = 0.0;
      if(i == 0) {
        cc = sol[1];
      } else {
        int k = 2 + (i - 1) * nC2;
        double ax = 1.0;
        for(int x = 0; x <= kOrder; x++) {
          double ay = 1.0;
          for(int y = 0; y <= kOrder - x; y++) {
            cc = fma(sol[k++], ax * ay, cc);
            ay *= yf;
          }
          ax *= xf;
        }
      }
      coeff[i] = cc;
      const float hi = (float)cc;
      cHi[i] = hi;
      cLo[i] = (float)(cc - (double)hi);
    }
    if(tid == 0) {
      double bg = 0.0, ax = 1.0;
      int k = nComp + 2;
      for(int i = 0; i <= bgOrder; i++) {
        double ay = 1.0;
        for(int j = 0; j <= bgOrder - i; j++) {
          bg = fma(sol[k++], ax * ay, bg);
          ay *= yf;
        }
        ax *= xf;
      }
      sBg = bg;
    }
  }
  __syncthreads();
  // The coefficients of an ill-conditioned fit cancel strongly, so the model
  // keeps about 48 bits: each coefficient is hi + lo in FP32, every product
  // with the (FP32) basis value is split exactly by an FMA, and the sum runs
  // in double-float (two-sum with a running error term), all on the FP32
  // pipe.  The model is then stored in FP32 as the reference does, and the
  // chi^2 terms (which only rank stamps against each other) are FP32.
  const float* Ws = W + (size_t)s * wRows * ldW;
  double acc = 0.0;
  int cnt = 0;
  if(live) {
    const float bgF = (float)sBg;
    float part = 0.f;
    // four consecutive pixels per thread, read as float4 (ldW is a multiple
    // of 4 and covers pix rounded up), rows unrolled so that several loads
    // are in flight; each pixel's sum runs over the rows in order
    for(int j0 = 4 * tid; j0 < pix; j0 += 4 * MX_THREADS) {
      float sh[4] = {0.f, 0.f, 0.f, 0.f}, sl[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll 7
      for(int i = 0; i < nPSF; i++) {
        const float4 w4 = *(const float4*)(Ws + (size_t)i * ldW + j0);
        const float wq[4] = {w4.x, w4.y, w4.z, w4.w};
        const float ch = cHi[i], cl = cLo[i];
#pragma unroll
        for(int q = 0; q < 4; q++) {
          const float wv = wq[q];
          const float ph = ch * wv;
          const float pe = fmaf(ch, wv, -ph) + cl * wv;  // exact low part + lo term
          const float ts = sh[q] + ph;                   // two-sum of sh and ph
          const float bp = ts - sh[q];
          const float er = (sh[q] - (ts - bp)) + (ph - bp);
          sh[q] = ts;
          sl[q] += er + pe;
        }
      }
#pragma unroll
      for(int q = 0; q < 4; q++) {
      const int j = j0 + q;
      if(j >= pix) break;
      const float m0 = (float)((double)sh[q] + (double)sl[q]);
      const int ax = j % fSS - fSS / 2 + c.x, ay = j / fSS - fSS / 2 + c.y;
      const size_t ai = (size_t)min(max(ax, 0), w - 1) + (size_t)min(max(ay, 0), h - 1) * w;
      const float sF = (float)sImg[ai];
      if((mask[ai] & BAD_INPUT) == 0 && fabsf(sF) > __double2float_rd(1e-10)) {
        if(isnan(m0) || isnan(sF)) {
          maskOr(mask, ai, NAN_PIXEL);
        } else {
          const float d = (m0 - sF) + bgF;
          part += d * d / ((fabsf((float)tImg[ai]) + fabsf(sF)) * invGain + rn2x2);
          cnt++;
        }
      }
      }
    }
    acc = (double)part;
  }
#pragma unroll
  for(int o = 16; o > 0; o >>= 1) {
    acc += __shfl_down_sync(0xffffffffu, acc, o);
    cnt += __shfl_down_sync(0xffffffffu, cnt, o);
  }
  if((tid & 31) == 0) {
    rs[tid >> 5] = acc;
    rc[tid >> 5] = cnt;
  }
  __syncthreads();
  if(tid == 0) {
    double a = 0.0;
    int n = 0;
    for(int i = 0; i < MX_THREADS / 32; i++) {
      a += rs[i];
      n += rc[i];
    }
    double r = -1.0;
    if(n > 0) {
      r = a / n;
      if(r >= 1e10) r = -1.0;
    }
    sig[t] = r;
  }
}

// ------------------------------------------------- global LU, FP64 + FMA ---
// Same distribution as the plain kernel (columns cyclic over the cluster's
// shared memories); pivots compared on the bit patterns of the non-negative
// doubles, trailing updates with fused multiply-adds.
template <int CL>
__global__ void __launch_bounds__(256)
    k_global_lu_fast(const double* __restrict__ M, double* __restrict__ F, int n,
                     int* __restrict__ idxOut, int* __restrict__ singular,
                     const int* __restrict__ gate) {
  if(gate != nullptr && !(gate[0] & 1)) return;  // the LDL^T factorisation succeeded
  extern __shared__ double gl_s[];
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank(), tid = threadIdx.x, nt = blockDim.x;
  const int ld = n + 1, ncol = (n + CL - 1) / CL;
  double* col = gl_s;
  double* vv = col + (size_t)ncol * ld;
  double* bc = vv + ld;
  double* L = bc + 2 * (ld + 1);
  __shared__ unsigned long long rv[8];
  __shared__ int ri[8];
  __shared__ int sP, sMaxI, sSing;
  if(tid == 0) sSing = 0;
  __syncthreads();
  for(int i = 1 + tid; i <= n; i += nt) {
    double big = 0.0;
    for(int j = 1; j <= n; j++) big = fmax(big, fabs(M[(size_t)i * ld + j]));
    if(big == 0.0) sSing = 1;
    vv[i] = 1.0 / big;
  }
  __syncthreads();
  if(sSing) {
    if(rank == 0 && tid == 0) *singular = 1;
    if(rank == 0) {
      for(int i = tid; i <= n; i += nt) idxOut[i] = 0;
      for(size_t q = tid; q < (size_t)ld * ld; q += nt) F[q] = M[q];  // left as it was
    }
    cluster.sync();
    return;
  }
  for(int lc = 0; lc < ncol; lc++) {
    const int j = lc * CL + rank + 1;
    for(int i = tid; i <= n; i += nt) col[(size_t)lc * ld + i] = j <= n ? M[(size_t)i * ld + j] : 0.0;
  }
  if(tid == 0) sMaxI = 0;
  __syncthreads();
  cluster.sync();
  for(int j = 1; j <= n; j++) {
    const int owner = (j - 1) % CL, lcj = (j - 1) / CL;
    double* myBc = bc + (j & 1) * (ld + 1);
    if(rank == owner) {
      double* cj = col + (size_t)lcj * ld;
      unsigned long long bv = 0;
      int bi = -1;
      for(int i = j + tid; i <= n; i += nt) {
        const double dum = vv[i] * fabs(cj[i]);
        if(!isnan(dum)) {
          const unsigned long long u = (unsigned long long)__double_as_longlong(dum);
          if(bi < 0 || u > bv || (u == bv && i > bi)) {
            bv = u;
            bi = i;
          }
        }
      }
#pragma unroll
      for(int o = 16; o > 0; o >>= 1) {
        unsigned long long ov = __shfl_down_sync(0xffffffffu, bv, o);
        int oi = __shfl_down_sync(0xffffffffu, bi, o);
        if(oi >= 0 && (bi < 0 || ov > bv || (ov == bv && oi > bi))) {
          bv = ov;
          bi = oi;
        }
      }
      if((tid & 31) == 0) {
        rv[tid >> 5] = bv;
        ri[tid >> 5] = bi;
      }
      __syncthreads();
      if(tid == 0) {
        unsigned long long v = rv[0];
        int i0 = ri[0];
        for(int q = 1; q < nt / 32; q++)
          if(ri[q] >= 0 && (i0 < 0 || rv[q] > v || (rv[q] == v && ri[q] > i0))) {
            v = rv[q];
            i0 = ri[q];
          }
        const int p = i0 >= 0 ? i0 : sMaxI;
        if(p != j) {
          double t = cj[p];
          cj[p] = cj[j];
          cj[j] = t;
        }
        if(cj[j] == 0.0) cj[j] = 1.0e-20;
        myBc[0] = (double)p;
      }
      __syncthreads();
      const double piv = cj[j];
      for(int i = j + 1 + tid; i <= n; i += nt) {
        const double l = cj[i] / piv;
        cj[i] = l;
        myBc[i] = l;
      }
    }
    cluster.sync();
    const double* src = cluster.map_shared_rank(myBc, owner);
    if(tid == 0) {
      sP = (int)src[0];
      sMaxI = sP;
    }
    for(int i = j + 1 + tid; i <= n; i += nt) L[i] = src[i];
    __syncthreads();
    const int p = sP;
    if(rank == 0 && tid == 0) idxOut[j] = p;
    if(p != j) {
      for(int lc = tid; lc < ncol; lc += nt) {
        if(rank == owner && lc == lcj) continue;
        double* cc = col + (size_t)lc * ld;
        double t = cc[p];
        cc[p] = cc[j];
        cc[j] = t;
      }
      if(tid == 0) vv[p] = vv[j];
    }
    __syncthreads();
    const int lcStart = (j - rank + CL - 1) / CL;
    const int nLoc = ncol - lcStart, m = n - j;
    for(int e = tid; e < nLoc * m; e += nt) {
      const int lc = lcStart + e / m, i = j + 1 + e % m;
      if(lc * CL + rank + 1 > n) continue;
      double* cc = col + (size_t)lc * ld;
      cc[i] = fma(-L[i], cc[j], cc[i]);
    }
    __syncthreads();
  }
  cluster.sync();
  for(int lc = 0; lc < ncol; lc++) {
    const int j = lc * CL + rank + 1;
    if(j > n) break;
    for(int i = tid; i <= n; i += nt) F[(size_t)i * ld + j] = col[(size_t)lc * ld + i];
  }
  if(rank == 0 && tid == 0) idxOut[0] = 0;
}

// Forward/back substitution by column sweeps plus one refinement step with
// the FP64 residual r = b - A x of the original matrix A.  One CTA.
__device__ void sweepSolve(const double* __restrict__ LU, int n, const int* piv, double* x,
                           const double* invU) {
  const int tid = threadIdx.x, nt = blockDim.x, ld = n + 1;
  __syncthreads();
  if(tid == 0)
    for(int i = 1; i <= n; i++) {
      const int ip = piv[i];
      const double t = x[ip];
      x[ip] = x[i];
      x[i] = t;
    }
  __syncthreads();
  for(int j = 1; j < n; j++) {
    const double xj = x[j];
    for(int i = j + 1 + tid; i <= n; i += nt) x[i] = fma(-LU[(size_t)i * ld + j], xj, x[i]);
    __syncthreads();
  }
  for(int j = n; j >= 1; j--) {
    const double xj = x[j] * invU[j];
    for(int i = 1 + tid; i < j; i += nt) x[i] = fma(-LU[(size_t)i * ld + j], xj, x[i]);
    __syncthreads();
    if(tid == 0) x[j] = xj;
    __syncthreads();
  }
}

__global__ void __launch_bounds__(1024)
    k_solve_refine(const double* __restrict__ LU, const double* __restrict__ A, int n,
                   const int* __restrict__ piv, double* __restrict__ b,
                   const int* __restrict__ gate) {
  if(gate != nullptr && !(gate[0] & 1)) return;  // solved from the LDL^T factors
  extern __shared__ double sv_s[];
  const int tid = threadIdx.x, nt = blockDim.x, ld = n + 1;
  double* x = sv_s;          // n + 1
  double* bb = x + ld;       // n + 1
  double* invU = bb + ld;    // n + 1
  double* d = invU + ld;     // n + 1
  int* p = (int*)(d + ld);   // n + 1
  for(int i = tid; i <= n; i += nt) {
    bb[i] = b[i];
    x[i] = b[i];
    p[i] = piv[i];
    invU[i] = i > 0 ? 1.0 / LU[(size_t)i * ld + i] : 0.0;
  }
  sweepSolve(LU, n, p, x, invU);
  // r = b - A x, one warp per row
  const int lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
  for(int i = 1 + warp; i <= n; i += nw) {
    double a = 0.0;
    for(int j = 1 + lane; j <= n; j += 32) a = fma(A[(size_t)i * ld + j], x[j], a);
#pragma unroll
    for(int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
    if(lane == 0) d[i] = bb[i] - a;
  }
  if(tid == 0) d[0] = 0.0;
  sweepSolve(LU, n, p, d, invU);
  for(int i = 1 + tid; i <= n; i += nt) b[i] = x[i] + d[i];
}

// -------------------------------------------------- conv + sub in FP32 ----
// BX kernel blocks (BX*21 columns) x one block row (21 rows) per CTA; each
// thread produces a 7 x 3 pixel tile of one block: every image row it loads
// into registers (27 values) feeds its three output rows through three
// kernel rows (broadcast float4 reads), 441 FMAs per 27 + 18 shared loads.
// BX (4, 6 or 8) is chosen by the autotuner; the three give identical
// images.
struct ConvArgsF {
  int w, h, hK, fK, nPSF, kOrder, bgOrder, nComp, scaleConv;
  float tH, tL;
  int xSteps;  // kernel blocks per row (block-centre table of k_conv_sub_f32)
};

// Normalised centres of the fK x fK kernel blocks, xf of the xSteps block
// columns then yf of the block rows: (centre - w/2) / (w/2) in FP64, the
// coordinates of the spatial kernel terms (conv(), src/bach.cpp:339-350).
__global__ void k_block_centres(int w, int h, int fK, int xSteps, int ySteps,
                                double* __restrict__ xy) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int hK = fK / 2;
  if(i < xSteps) {
    const double hx = 0.5 * w;
    xy[i] = (i * fK + 2 * hK - hx) / hx;
  } else if(i < xSteps + ySteps) {
    const double hy = 0.5 * h;
    xy[i] = ((i - xSteps) * fK + 2 * hK - hy) / hy;
  }
}

__device__ __forceinline__ uint16_t convMaskF(float t, float tH, float tL) {
  uint16_t m = 0;
  if(t == 0.f) m |= BAD_INPUT | BAD_PIX_VAL;
  if(t >= tH) m |= BAD_INPUT | SAT_PIXEL;
  if(t <= tL) m |= BAD_INPUT | LOW_PIXEL;
  return m;
}
__device__ __forceinline__ uint16_t afterMaskF(float t, float tH, float tL) {
  uint16_t m = 0;
  if(t == 0.f) m |= BAD_OUTPUT | BAD_INPUT | BAD_PIX_VAL;
  if(t >= tH) m |= BAD_OUTPUT | BAD_INPUT | SAT_PIXEL;
  if(t <= tL) m |= BAD_OUTPUT | BAD_INPUT | LOW_PIXEL;
  return m;
}

// Shared-memory layout of k_conv_sub_f32 for BX blocks per CTA.  The tile
// row stride S is padded so that the window loads of a warp (lanes ordered
// block, column group, row group) fall in 32 distinct banks.
template <int FK, int BX>
struct ConvTileF {
  static constexpr int HK = FK / 2, NK = FK * FK, PX = 7, RY = 3;
  static constexpr int TPB = (FK / PX) * (FK / RY);  // threads per kernel block
  static constexpr int NT = BX * TPB;
  static constexpr int TW = BX * FK + 2 * HK, TH = FK + 2 * HK;
  static constexpr int S = TW + (BX == 2 ? 13 : BX == 4 ? 3 : BX == 6 ? 25 : 15);
  static constexpr int NW = (TW + 31) / 32 + 1;  // bad-flag words per tile row (+1: 64-bit reads)
  static constexpr int KS = 24;                  // kernel row stride (float4 reads)
  static constexpr size_t OFF_KERN = ((size_t)TH * S * 4 + 15) / 16 * 16;
  static constexpr size_t OFF_BITS = OFF_KERN + (size_t)BX * FK * KS * 4;
  static constexpr size_t OFF_AKS = OFF_BITS + (size_t)TH * NW * 4;
  static constexpr size_t OFF_FLAG = OFF_AKS + (size_t)(BX + 16) * 4;  // per output pixel
  static constexpr size_t BYTES = OFF_FLAG + (size_t)BX * NK;
  // after the sums the kernel rows hold the CTA's conv sums, row-major
  static_assert((size_t)BX * FK * KS >= (size_t)BX * NK, "staging fits the kernel rows");
};

// Kernel of each of BX blocks at its centre (conv(), src/bach.cpp:339-350)
// from the FP64 spatial-term images Kt[t] (t over xf^i yf^j, i outer), one
// tap per thread for all blocks: the terms of each x power collapsed over yf
// (shared by the CTA's blocks) by Horner, then Horner in the block's xf;
// FP64, rounded once to FP32 into rows of KS = 24 floats.
template <int K, int FK, int BX, int NT>
__device__ __forceinline__ void convBlockKernels(const double* __restrict__ Kt,
                                                 const double* __restrict__ xfTab, double yf,
                                                 int xB0, float* kern) {
  constexpr int NK = FK * FK, KS = 24;
  double xfb[BX];
#pragma unroll
  for(int b = 0; b < BX; b++) xfb[b] = xfTab[xB0 + b];
  for(int p = threadIdx.x; p < NK; p += NT) {
    double cx[K + 1];
#pragma unroll
    for(int i = 0; i <= K; i++) {
      const int t0 = i * (K + 1) - i * (i - 1) / 2;  // term of xf^i yf^0
      double s = Kt[(size_t)(t0 + K - i) * NK + p];
#pragma unroll
      for(int j = K - i - 1; j >= 0; j--) s = fma(s, yf, Kt[(size_t)(t0 + j) * NK + p]);
      cx[i] = s;
    }
    const int row = p / FK, col = p - row * FK;
#pragma unroll
    for(int b = 0; b < BX; b++) {
      double k0 = cx[K];
#pragma unroll
      for(int i = K - 1; i >= 0; i--) k0 = fma(k0, xfb[b], cx[i]);
      kern[(b * FK + row) * KS + col] = (float)k0;
    }
  }
}

// The rounding order of each output is the reference's tap order: over
// kernel rows jj, then columns ii, one FP32 FMA per tap.
template <int FK, int BX>
__global__ void __launch_bounds__(BX * 21, BX == 8 ? 2 : 1)
    k_conv_sub_f32(const float* __restrict__ I, const float* __restrict__ O,
                   const double* __restrict__ sol, const double* __restrict__ Kt,
                   const double* __restrict__ blockXY, const double* __restrict__ kernSumPtr,
                   ConvArgsF a,
                   const uint8_t* __restrict__ inMask, uint16_t* __restrict__ mask,
                   float* __restrict__ convF, float* __restrict__ diffF) {
  using L = ConvTileF<FK, BX>;
  static_assert(FK % L::PX == 0 && FK % L::RY == 0 && L::TPB == 21, "tiling");
  constexpr int HK = L::HK, NK = L::NK, S = L::S, TW = L::TW, TH = L::TH, NW = L::NW, KS = L::KS;
  constexpr int NT = L::NT, NFULL = NT / 32;  // full warps (ballots, |k| sums)
  extern __shared__ __align__(16) unsigned char cv_smem[];
  float* tile = (float*)cv_smem;
  float* kern = (float*)(cv_smem + L::OFF_KERN);
  uint32_t* bits = (uint32_t*)(cv_smem + L::OFF_BITS);
  float* aks = (float*)(cv_smem + L::OFF_AKS);
  float* bgc = aks + BX;  // background coefficients (getBackground), FP32
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int xB0 = blockIdx.x * BX, yB = blockIdx.y;
  const int x0 = xB0 * FK, y0 = yB * FK;  // tile origin; block pixels start at +HK
  const int K = a.kOrder;
  for(int i = tid; i < TH * TW; i += NT) {
    const int ly = i / TW, lx = i - ly * TW;
    const int gx = min(x0 + lx, a.w - 1), gy = min(y0 + ly, a.h - 1);
    tile[ly * S + lx] = I[(size_t)gx + (size_t)gy * a.w];
  }
  // kernel of each block (conv(), src/bach.cpp:339-350)
  {
    const double yf = blockXY[a.xSteps + yB];
    switch(K) {
      case 0: convBlockKernels<0, FK, BX, NT>(Kt, blockXY, yf, xB0, kern); break;
      case 1: convBlockKernels<1, FK, BX, NT>(Kt, blockXY, yf, xB0, kern); break;
      case 2: convBlockKernels<2, FK, BX, NT>(Kt, blockXY, yf, xB0, kern); break;
      default: convBlockKernels<3, FK, BX, NT>(Kt, blockXY, yf, xB0, kern); break;
    }
  }
  __syncthreads();
  if(warp < NFULL) {
    // bad-input flags of the tile as bits (word c/32 of a row, bit c%32; the
    // last word of a row is zero), one row per warp at a time
    for(int ly = warp; ly < TH; ly += NFULL) {
      const int gy = min(y0 + ly, a.h - 1);
#pragma unroll
      for(int wc = 0; wc < NW; wc++) {
        const int c = wc * 32 + lane;
        bool bd = false;
        if(c < TW) {
          bd = convMaskF(tile[ly * S + c], a.tH, a.tL) & BAD_INPUT;
          if(inMask) bd |= inMask[(size_t)min(x0 + c, a.w - 1) + (size_t)gy * a.w] != 0;
        }
        const unsigned m = __ballot_sync(0xffffffffu, bd);
        if(lane == 0) bits[ly * NW + wc] = m;
      }
    }
    // sum of |k| of each block: lane-strided partial sums, then a butterfly
    for(int b = warp; b < BX; b += NFULL) {
      float s = 0.f;
      for(int p = lane; p < NK; p += 32) s += fabsf(kern[(b * FK + p / FK) * KS + p % FK]);
#pragma unroll
      for(int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      if(lane == 0) aks[b] = s;
    }
  }
  const int nBgC = (a.bgOrder + 1) * (a.bgOrder + 2) / 2;
  if(tid < nBgC) bgc[tid] = (float)sol[a.nComp + 2 + tid];
  __syncthreads();
  // thread -> (block b, column group k, row group g): 7 columns x 3 rows
  const int b = tid / L::TPB, r = tid - b * L::TPB, kq = r / 7, g = r - kq * 7;
  const int ly0 = L::RY * g, lx0 = b * FK + L::PX * kq;
  const float* kb = kern + b * FK * KS;
  float acc[3][7];
#pragma unroll
  for(int o = 0; o < 3; o++)
#pragma unroll
    for(int q = 0; q < 7; q++) acc[o][q] = 0.f;
  // tile row ly0 + R feeds output row ly0 + o through kernel row jj = R - o
  for(int R = 0; R < FK + 2; R++) {
    float win[27];
    const float* trow = tile + (ly0 + R) * S + lx0;
#pragma unroll
    for(int q = 0; q < 27; q++) win[q] = trow[q];
#pragma unroll
    for(int o = 0; o < 3; o++) {
      const int jj = R - o;
      if(jj < 0 || jj >= FK) continue;
      const float4* kr4 = (const float4*)(kb + (FK - 1 - jj) * KS);
      float kf[24];
#pragma unroll
      for(int m = 0; m < 6; m++) {
        const float4 v = kr4[m];
        kf[4 * m] = v.x;
        kf[4 * m + 1] = v.y;
        kf[4 * m + 2] = v.z;
        kf[4 * m + 3] = v.w;
      }
#pragma unroll
      for(int ii = 0; ii < FK; ii++) {
        const float kk = kf[FK - 1 - ii];
#pragma unroll
        for(int q = 0; q < 7; q++) acc[o][q] = fmaf(kk, win[q + ii], acc[o][q]);
      }
    }
  }
  // Pixels whose window holds a bad one: the sum of |k| over the good
  // pixels is the kernel's |k| sum less that over the bad pixels, which are
  // few (saturated cores); each bad pixel's |k| is added, in row then column
  // order, to every output pixel of this thread whose window covers it.
  constexpr unsigned long long WIN = (1ull << FK) - 1, COLS = (1ull << 27) - 1;
  unsigned long long orw[3] = {0ull, 0ull, 0ull};
  float badSum[3][7];
#pragma unroll
  for(int o = 0; o < 3; o++)
#pragma unroll
    for(int q = 0; q < 7; q++) badSum[o][q] = 0.f;
  for(int R = 0; R < FK + 2; R++) {
    const uint32_t* br = bits + (ly0 + R) * NW + (lx0 >> 5);
    unsigned long long wb =
        (((unsigned long long)br[0] | ((unsigned long long)br[1] << 32)) >> (lx0 & 31)) & COLS;
    if(wb == 0ull) continue;
#pragma unroll
    for(int o = 0; o < 3; o++)
      if(R - o >= 0 && R - o < FK) orw[o] |= wb;
    while(wb != 0ull) {
      const int cI = __ffsll((long long)wb) - 1;  // window column of a bad pixel
      wb &= wb - 1ull;
#pragma unroll
      for(int o = 0; o < 3; o++) {
        const int jj = R - o;
        if(jj < 0 || jj >= FK) continue;
        const float* krow = kb + (FK - 1 - jj) * KS + (FK - 1);
#pragma unroll
        for(int q = 0; q < 7; q++) {
          const int ii = cI - q;
          if(ii >= 0 && ii < FK) badSum[o][q] += fabsf(krow[-ii]);
        }
      }
    }
  }
  __syncthreads();  // every thread is done with the kernel rows
  float* sv = kern;  // conv sums of the CTA's pixels, row-major (FK rows x BX*FK)
  unsigned char* cflag = cv_smem + L::OFF_FLAG;  // 0: window clean, 1: OK_CONV, 2: BAD_CONV
  constexpr int RW = BX * FK;
#pragma unroll
  for(int o = 0; o < 3; o++)
#pragma unroll
    for(int q = 0; q < 7; q++) {
      const int e = (ly0 + o) * RW + lx0 + q;
      sv[e] = acc[o][q];
      unsigned char f = 0;
      if(((orw[o] >> q) & WIN) != 0ull) f = ((aks[b] - badSum[o][q]) / aks[b]) < 0.99f ? 2 : 1;
      cflag[e] = f;
    }
  __syncthreads();
  // one output column per thread, consecutive x across the CTA: coalesced
  // reads of the other image and writes of mask, conv and difference
  const float hxF = 0.5f * (float)a.w, hyF = 0.5f * (float)a.h;
  const float ihxF = 1.f / hxF, ihyF = 1.f / hyF;
  const float kernSum = (float)*kernSumPtr;
  const float invKernMult = a.scaleConv ? 1.f / kernSum : 1.f;
  const float convFactor = a.scaleConv ? kernSum : 1.f;
  const float finalFactor = a.scaleConv ? -(1.f / kernSum) : 1.f;
  static_assert(NT == RW, "one output column per thread");
  const int x = x0 + HK + tid;
  if(x >= a.w - HK) return;
  // background polynomial (getBackground, cd.cl:444-467) in FP32: the terms
  // are O(1e3) ADU, so FP32 rounding moves a pixel by ~1e-4 ADU
  const float bxf = ((float)x - hxF) * ihxF;
  for(int ly = 0; ly < FK; ly++) {
    const int y = y0 + HK + ly;
    if(y >= a.h - HK) break;
    const int e = ly * RW + tid;
    const float byf = ((float)y - hyF) * ihyF;
    float bgv = 0.f, ax = 1.f;
    int k = 0;
    for(int i = 0; i <= a.bgOrder; i++) {
      float ay = 1.f;
      for(int j = 0; j <= a.bgOrder - i; j++) {
        bgv = fmaf(bgc[k++], ax * ay, bgv);
        ay *= byf;
      }
      ax *= bxf;
    }
    const float v = (sv[e] + bgv) * invKernMult;
    const size_t id = (size_t)x + (size_t)y * a.w;
    const float tc = tile[(ly + HK) * S + tid + HK];
    uint16_t cm = convMaskF(tc, a.tH, a.tL);
    if(inMask && inMask[id]) cm |= INPUT_MASK | BAD_INPUT;
    uint16_t nm = cm;
    if(cm & BAD_INPUT) nm |= BAD_OUTPUT;
    const unsigned char f = cflag[e];
    if(f == 2) nm |= BAD_OUTPUT | BAD_CONV;
    else if(f == 1) nm |= OK_CONV;
    const float ov = O[id];
    nm |= afterMaskF(ov, a.tH, a.tL);
    mask[id] = nm;
    convF[id] = v;
    diffF[id] = (nm & BAD_OUTPUT) ? 1e-30f : (v * convFactor - ov) * finalFactor;
  }
}

// Per-pixel kernel in FP32 (option convPerPixel; the FP64 statement is
// k_conv_sub_pp_f64).  The kernel at pixel (x, y) is written as the block
// kernel plus corrections, k(x, y) = k(xc, yc) + sum_{t>=1} dP_t Kt[t] with
// dP_t = P_t(x, y) - P_t(xc, yc): the block kernel is evaluated in FP64 and
// rounded once (as k_conv_sub_f32 does), and the FP32 rounding of the
// term images only scales the small dP_t (|dP| <= ~fK / frame size), so
// fits whose spatial terms cancel keep the block kernel's accuracy.  Seven
// pixels of one row per thread, the window in registers, one pass over the
// tile per term.
template <int FK, int CV_BX>
__global__ void __launch_bounds__(CV_BX * FK * (FK / 7))
    k_conv_sub_pp_f32(const float* __restrict__ I, const float* __restrict__ O,
                      const double* __restrict__ sol, const double* __restrict__ Kt,
                      const double* __restrict__ kernSumPtr, ConvArgsF a,
                      const uint8_t* __restrict__ inMask, uint16_t* __restrict__ mask,
                      float* __restrict__ convF, float* __restrict__ diffF) {
  constexpr int HK = FK / 2, NK = FK * FK, PX = 7, TPR = FK / PX;
  constexpr int TH = FK + 2 * HK, TW = CV_BX * FK + 2 * HK;
  constexpr int MAXT = (MAX_KORDER + 1) * (MAX_KORDER + 2) / 2;
  __shared__ float tile[TH][TW + 1];
  __shared__ unsigned char bad[TH][TW + 1];
  __shared__ unsigned char rowBad[TH][CV_BX * FK];
  __shared__ float kern[CV_BX][NK];
  __shared__ double poly[CV_BX][MAXT];
  __shared__ float bgc[16];
  extern __shared__ float ktf[];  // nC2 * NK, term 0 unused
  const int tid = threadIdx.x, nthr = blockDim.x;
  const int xB0 = blockIdx.x * CV_BX, yB = blockIdx.y;
  const int x0 = xB0 * FK, y0 = yB * FK;
  const int nC2 = (a.kOrder + 1) * (a.kOrder + 2) / 2;
  const double hx = 0.5 * a.w, hy = 0.5 * a.h;
  if(tid < CV_BX) {
    // spatial terms at the block centre (conv(), src/bach.cpp:339-350)
    const double xf = ((xB0 + tid) * FK + 2 * HK - hx) / hx, yf = (yB * FK + 2 * HK - hy) / hy;
    double ax = 1.0;
    int t = 0;
    for(int i = 0; i <= a.kOrder; i++) {
      double ay = 1.0;
      for(int j = 0; j <= a.kOrder - i; j++) {
        poly[tid][t++] = ax * ay;
        ay *= yf;
      }
      ax *= xf;
    }
  }
  for(int e = tid; e < nC2 * NK; e += nthr) ktf[e] = (float)Kt[e];
  for(int i = tid; i < TH * TW; i += nthr) {
    const int ly = i / TW, lx = i % TW;
    const int gx = min(x0 + lx, a.w - 1), gy = min(y0 + ly, a.h - 1);
    const float v = I[(size_t)gx + (size_t)gy * a.w];
    tile[ly][lx] = v;
    bad[ly][lx] = ((convMaskF(v, a.tH, a.tL) & BAD_INPUT) ||
                   (inMask && inMask[(size_t)gx + (size_t)gy * a.w])) ? 1 : 0;
  }
  const int nBgC = (a.bgOrder + 1) * (a.bgOrder + 2) / 2;
  if(tid < nBgC && tid < 16) bgc[tid] = (float)sol[a.nComp + 2 + tid];
  __syncthreads();
  for(int e = tid; e < CV_BX * NK; e += nthr) {
    const int b = e / NK, p = e % NK;
    double k0 = 0.0;
    for(int t = 0; t < nC2; t++) k0 = fma(poly[b][t], Kt[(size_t)t * NK + p], k0);
    kern[b][p] = (float)k0;
  }
  for(int e = tid; e < TH * CV_BX * FK; e += nthr) {
    const int ly = e / (CV_BX * FK), lx = e % (CV_BX * FK);
    unsigned char o = 0;
#pragma unroll
    for(int d = 0; d < FK; d++) o |= bad[ly][lx + d];
    rowBad[ly][lx] = o;
  }
  __syncthreads();
  const float kernSum = (float)*kernSumPtr;
  const float invKernMult = a.scaleConv ? 1.f / kernSum : 1.f;
  const float convFactor = a.scaleConv ? kernSum : 1.f;
  const float finalFactor = a.scaleConv ? -(1.f / kernSum) : 1.f;
  const int perBlock = FK * TPR;
  if(tid >= CV_BX * perBlock) return;
  const int b = tid / perBlock, r = tid % perBlock, ly = r / TPR, lx0 = b * FK + (r % TPR) * PX;
  const double yf = ((double)(y0 + HK + ly) - hy) / hy;
  double xf[PX], xp[PX];
  float base[PX], corr[PX];
#pragma unroll
  for(int q = 0; q < PX; q++) {
    xf[q] = ((double)(x0 + HK + lx0 + q) - hx) / hx;
    xp[q] = 1.0;
    corr[q] = 0.f;
  }
  // t = 0 pass: the block kernel
  {
#pragma unroll
    for(int q = 0; q < PX; q++) base[q] = 0.f;
    for(int jj = 0; jj < FK; jj++) {
      float win[PX + FK - 1];
#pragma unroll
      for(int q = 0; q < PX + FK - 1; q++) win[q] = tile[ly + jj][lx0 + q];
      const float* krow = kern[b] + (FK - 1 - jj) * FK;
#pragma unroll
      for(int ii = 0; ii < FK; ii++) {
        const float kk = krow[FK - 1 - ii];
#pragma unroll
        for(int q = 0; q < PX; q++) base[q] = fmaf(kk, win[q + ii], base[q]);
      }
    }
  }
  // t >= 1 passes: the spatial-term images weighted by dP_t
  int t = 0;
  for(int i = 0; i <= a.kOrder; i++) {
    double yp = 1.0;
    for(int j = 0; j <= a.kOrder - i; j++, t++) {
      if(t > 0) {
        const float* kb = ktf + t * NK;
        float ct[PX];
#pragma unroll
        for(int q = 0; q < PX; q++) ct[q] = 0.f;
        for(int jj = 0; jj < FK; jj++) {
          float win[PX + FK - 1];
#pragma unroll
          for(int q = 0; q < PX + FK - 1; q++) win[q] = tile[ly + jj][lx0 + q];
          const float* krow = kb + (FK - 1 - jj) * FK;
#pragma unroll
          for(int ii = 0; ii < FK; ii++) {
            const float kk = krow[FK - 1 - ii];
#pragma unroll
            for(int q = 0; q < PX; q++) ct[q] = fmaf(kk, win[q + ii], ct[q]);
          }
        }
#pragma unroll
        for(int q = 0; q < PX; q++)
          corr[q] = fmaf((float)(xp[q] * yp - poly[b][t]), ct[q], corr[q]);
      }
      yp *= yf;
    }
#pragma unroll
    for(int q = 0; q < PX; q++) xp[q] *= xf[q];
  }
  const float hxF = 0.5f * (float)a.w, hyF = 0.5f * (float)a.h;
  const float ihxF = 1.f / hxF, ihyF = 1.f / hyF;
#pragma unroll
  for(int q = 0; q < PX; q++) {
    const int x = x0 + HK + lx0 + q, y = y0 + HK + ly;
    if(x >= a.w - HK || y >= a.h - HK) continue;
    unsigned char any = 0;
    for(int jj = 0; jj < FK; jj++) any |= rowBad[ly + jj][lx0 + q];
    const float bxf = ((float)x - hxF) * ihxF, byf = ((float)y - hyF) * ihyF;
    float bgv = 0.f, ax = 1.f;
    int k = 0;
    for(int i = 0; i <= a.bgOrder; i++) {
      float ay = 1.f;
      for(int j = 0; j <= a.bgOrder - i; j++) {
        bgv = fmaf(bgc[k++], ax * ay, bgv);
        ay *= byf;
      }
      ax *= bxf;
    }
    const float v = (base[q] + corr[q] + bgv) * invKernMult;
    const size_t id = (size_t)x + (size_t)y * a.w;
    const float tc = tile[ly + HK][lx0 + q + HK];
    uint16_t cm = convMaskF(tc, a.tH, a.tL);
    if(inMask && inMask[id]) cm |= INPUT_MASK | BAD_INPUT;
    uint16_t nm = cm;
    if(cm & BAD_INPUT) nm |= BAD_OUTPUT;
    if(any) {
      // this pixel's kernel tap by tap, for the 0.99 |kernel| rule
      float dP[MAXT];
      {
        double xpw = 1.0;
        int tt = 0;
        for(int i = 0; i <= a.kOrder; i++) {
          double ypw = 1.0;
          for(int j = 0; j <= a.kOrder - i; j++, tt++) {
            dP[tt] = (float)(xpw * ypw - poly[b][tt]);
            ypw *= yf;
          }
          xpw *= xf[q];
        }
      }
      float aks = 0.f, uks = 0.f;
      for(int jj = 0; jj < FK; jj++)
        for(int ii = 0; ii < FK; ii++) {
          const int tap = (FK - 1 - ii) + (FK - 1 - jj) * FK;
          float kv = kern[b][tap];
          for(int tt = 1; tt < nC2; tt++) kv = fmaf(dP[tt], ktf[tt * NK + tap], kv);
          aks += fabsf(kv);
          if(!bad[ly + jj][lx0 + q + ii]) uks += fabsf(kv);
        }
      if((uks / aks) < 0.99f) nm |= BAD_OUTPUT | BAD_CONV;
      else nm |= OK_CONV;
    }
    const float o = O[id];
    nm |= afterMaskF(o, a.tH, a.tL);
    mask[id] = nm;
    convF[id] = v;
    diffF[id] = (nm & BAD_OUTPUT) ? 1e-30f : (v * convFactor - o) * finalFactor;
  }
}

// Kernel images of the spatial terms, FP64: Kt[t] = sum_n sol[2+(n-1)*nC2+t]
// * basis_n (+ sol[1] * basis_0 for the constant term), so that the kernel at
// (xf, yf) is sum_t xf^i yf^j Kt[t] (makeKernelCoeffs + makeKernel,
// cl_kern/cd.cl:354-417, regrouped by spatial term).
__global__ void k_kernel_terms(const double* __restrict__ sol, const double* __restrict__ vec,
                               int nPSF, int nC2, int nk, double* __restrict__ Kt) {
  for(int e = blockIdx.x * blockDim.x + threadIdx.x; e < nC2 * nk; e += gridDim.x * blockDim.x) {
    const int t = e / nk, p = e % nk;
    double k0 = t == 0 ? sol[1] * vec[p] : 0.0;
    for(int n = 1; n < nPSF; n++) k0 = fma(sol[2 + (n - 1) * nC2 + t], vec[(size_t)n * nk + p], k0);
    Kt[e] = k0;
  }
}

__global__ void k_border_f32(const float* __restrict__ O, int w, int h, int hK, float tH, float tL,
                             const uint8_t* __restrict__ inMask, uint16_t* __restrict__ mask, float* __restrict__ convF,
                             float* __restrict__ diffF) {
  const long long n = (long long)w * h;
  for(long long id = (long long)blockIdx.x * blockDim.x + threadIdx.x; id < n;
      id += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(id % w), y = (int)(id / w);
    if(x >= hK && x < w - hK && y >= hK && y < h - hK) continue;
    mask[id] |= afterMaskF(O[id], tH, tL);
    if(inMask && inMask[id]) mask[id] |= INPUT_MASK | BAD_INPUT | BAD_OUTPUT;
    convF[id] = 1e-30f;
    diffF[id] = 1e-30f;
  }
}

// ------------------------------------------------ global matrix and RHS ---
// Every entry of createMatrix / createScProd (cdkscUtil.cpp:307-475) is a sum
// over the fitted stamps of one per-stamp number (a Q entry, a W dot product
// or a B entry) times a spatial factor: a product of two kernel weights, one
// weight, or 1.  The weights are monomials x^a y^b of the substamp position,
// so a product of two is the monomial of the summed exponents.  The sums are
// therefore the products X (rows: per-stamp numbers) x Y (columns: the
// monomials up to twice the kernel order, zero for a stamp without a
// substamp, plus an unmasked 1), computed split over chunks of 32 stamps
// into partials P[split][row][col]; k_mx_scatter adds the splits in order
// and places every matrix and RHS entry.
//   X rows: [Q pairs (qa, qb), 2 <= qa <= nC1+1, 1 <= qb <= qa]
//           [Q(1,1)] [dots entries 0..stride) [B entries 1..nC1+1]
constexpr int MXB_ROWS = 64, MXB_T = 32, MXB_MAXC = 32;

__device__ __forceinline__ int mxPairRow(int qa, int qb) { return (qa - 1) * qa / 2 - 1 + (qb - 1); }

// The spatial factors of the matrix build for the listed stamps: Y[t][c] =
// xf^a yf^b of monomial c at stamp t's substamp (0 for a stamp without one)
// and Y[t][nMono] = 1, split into hi + lo floats; once per build instead of
// once per row block of k_mx_build.
__global__ void k_mx_mono(const int* __restrict__ list, int nList, const int* __restrict__ liveN,
                          const int* __restrict__ count, const int* __restrict__ cur,
                          const int2* __restrict__ ssxy, int maxSS, const int2* __restrict__ monoExp,
                          int nMono, int w, int h, float2* __restrict__ Y) {
  if(liveN) nList = min(nList, *liveN);
  const int NC = nMono + 1;
  for(int e = blockIdx.x * blockDim.x + threadIdx.x; e < nList * NC; e += gridDim.x * blockDim.x) {
    const int t = e / NC, cI = e % NC, st = list[t];
    double v = 0.0;
    if(cI == nMono) {
      v = 1.0;
    } else if(cur[st] < count[st]) {
      const int2 c = ssxy[(size_t)st * maxSS + cur[st]];
      const int2 ex = monoExp[cI];
      v = ipowD(floatNormD(c.x, w), ex.x) * ipowD(floatNormD(c.y, h), ex.y);
    }
    const float hi = (float)v;
    Y[e] = make_float2(hi, (float)(v - (double)hi));
  }
}

__global__ void __launch_bounds__(256)
    k_mx_build(const int* __restrict__ list, int nList, const int* __restrict__ liveN,
               const int* __restrict__ count,
               const int* __restrict__ cur, const int2* __restrict__ ssxy, int maxSS,
               const double* __restrict__ Q, int qc, const double* __restrict__ dots, int stride,
               const double* __restrict__ B, const float2* __restrict__ Ytab, int nMono,
               int nC1, int nRows, double* __restrict__ P) {
  // X and Y as double-float pairs (hi + lo in FP32): the products and sums
  // run on the FP32 pipe with about 48 bits (two-product by FMA, two-sum
  // with a running error term), far below the 2^-36 of the Gram entries
  // they come from; the partial sums are stored in FP64.
  __shared__ float XsH[MXB_ROWS][MXB_T + 1], XsL[MXB_ROWS][MXB_T + 1];
  __shared__ float YsH[MXB_T][MXB_MAXC], YsL[MXB_T][MXB_MAXC];
  __shared__ int sS[MXB_T];
  __shared__ int rowSrc[MXB_ROWS];  // source of each row: type << 24 | offset in the stamp
  if(liveN) nList = min(nList, *liveN);
  const int tid = threadIdx.x, split = blockIdx.y, t0 = split * MXB_T;
  if(t0 >= nList && split > 0) return;  // split 0 writes zeros for an empty list
  const int nt = min(MXB_T, nList - t0), row0 = blockIdx.x * MXB_ROWS, NC = nMono + 1;
  const int nQP = mxPairRow(nC1 + 2, 1);  // Q pairs
  if(tid < MXB_T) sS[tid] = tid < nt ? list[t0 + tid] : -1;
  if(tid >= 64 && tid < 64 + MXB_ROWS) {
    const int r = tid - 64, row = row0 + r;
    int code = -1;
    if(row < nRows) {
      if(row < nQP) {
        int qa = (int)((sqrtf(8.f * (float)(row + 1) + 1.f) - 1.f) * 0.5f) + 1;  // first guess
        while(mxPairRow(qa + 1, 1) <= row) qa++;
        while(qa > 1 && mxPairRow(qa, 1) > row) qa--;
        const int qb = row - mxPairRow(qa, 1) + 1;
        code = qa * qc + qb;
      } else if(row == nQP) {
        code = qc + 1;
      } else if(row < nQP + 1 + stride) {
        code = (1 << 24) | (row - nQP - 1);
      } else {
        code = (2 << 24) | (1 + row - nQP - 1 - stride);
      }
    }
    rowSrc[r] = code;
  }
  __syncthreads();
  for(int e = tid; e < MXB_T * NC; e += 256) {
    const int tt = e / NC, cI = e % NC;
    float2 y = make_float2(0.f, 0.f);
    if(sS[tt] >= 0) y = Ytab[(size_t)(t0 + tt) * NC + cI];
    YsH[tt][cI] = y.x;
    YsL[tt][cI] = y.y;
  }
  for(int e = tid; e < MXB_ROWS * MXB_T; e += 256) {
    const int r = e / MXB_T, tt = e % MXB_T, st = sS[tt], code = rowSrc[r];
    double v = 0.0;
    if(st >= 0 && code >= 0) {
      const int type = code >> 24, off = code & 0xFFFFFF;
      v = type == 0 ? Q[(size_t)st * qc * qc + off]
        : type == 1 ? dots[(size_t)st * stride + off]
                    : B[(size_t)st * qc + off];
    }
    const float hi = (float)v;
    XsH[r][tt] = hi;
    XsL[r][tt] = (float)(v - (double)hi);
  }
  __syncthreads();
  const int r = tid >> 2, cg0 = tid & 3;
  float aH[MXB_MAXC / 4], aL[MXB_MAXC / 4];
#pragma unroll
  for(int u = 0; u < MXB_MAXC / 4; u++) aH[u] = aL[u] = 0.f;
  for(int tt = 0; tt < nt; tt++) {
    const float xh = XsH[r][tt], xl = XsL[r][tt];
#pragma unroll
    for(int u = 0; u < MXB_MAXC / 4; u++)
      if(cg0 + 4 * u < NC) {
        const float yh = YsH[tt][cg0 + 4 * u], yl = YsL[tt][cg0 + 4 * u];
        const float ph = xh * yh;
        const float pe = fmaf(xl, yh, fmaf(xh, yl, fmaf(xh, yh, -ph)));
        const float sm = aH[u] + ph, bp = sm - aH[u];
        aL[u] += ((aH[u] - (sm - bp)) + (ph - bp)) + pe;
        aH[u] = sm;
      }
  }
  if(row0 + r < nRows) {
    double* out = P + ((size_t)split * nRows + row0 + r) * NC;
#pragma unroll
    for(int u = 0; u < MXB_MAXC / 4; u++)
      if(cg0 + 4 * u < NC) out[cg0 + 4 * u] = (double)aH[u] + (double)aL[u];
  }
}

// Lower triangle of the global matrix (mirrored), row/column 0 zeroed, and
// the RHS (nSol entries; bgBase selects the background projection form).
__global__ void __launch_bounds__(256)
    k_mx_scatter(const double* __restrict__ P, int nSplit, const int* __restrict__ liveN,
                 int nRows, int nMono, const int2* __restrict__ kp,
                 const int* __restrict__ monoIdx, int monoDim, int nC1, int nC2, int nBG,
                 int stride, int bgBase, int matSize, int nSol, double* __restrict__ M,
                 double* __restrict__ rhs) {
  // live stamps on the device: only their splits hold partial sums
  if(liveN) nSplit = min(nSplit, (*liveN + MXB_T - 1) / MXB_T);
  const int ld = matSize + 1, nComp = nC1 * nC2, NC = nMono + 1;
  const int nQP = mxPairRow(nC1 + 2, 1), dotRow0 = nQP + 1, bRow0 = nQP + 1 + stride;
  const long long nTri = (long long)matSize * (matSize + 1) / 2;
  auto sumP = [&](int xr, int cI) {
    double v = 0.0;
    for(int sp = 0; sp < nSplit; sp++) v += P[((size_t)sp * nRows + xr) * NC + cI];
    return v;
  };
  auto mono = [&](int a, int b) { return monoIdx[a * monoDim + b]; };
  for(long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < nTri + nSol + ld;
      e += (long long)gridDim.x * blockDim.x) {
    if(e < nTri) {
      int r = (int)((sqrt(8.0 * (double)e + 1.0) - 1.0) * 0.5);
      while((long long)(r + 1) * (r + 2) / 2 <= e) r++;
      while((long long)r * (r + 1) / 2 > e) r--;
      const int row = r + 1, col = (int)(e - (long long)r * (r + 1) / 2) + 1;
      double v;
      if(row == 1) {
        v = sumP(nQP, nMono);
      } else if(row <= nComp + 1) {
        const int i = row - 2, i1 = i / nC2, i2 = i % nC2;
        if(col == 1) {
          v = sumP(mxPairRow(i1 + 2, 1), mono(kp[i2].x, kp[i2].y));
        } else {
          const int j = col - 2, j1 = j / nC2, j2 = j % nC2;
          v = sumP(mxPairRow(i1 + 2, j1 + 2), mono(kp[i2].x + kp[j2].x, kp[i2].y + kp[j2].y));
        }
      } else {
        const int ib = row - (nComp + 2);
        if(col == 1) {
          v = sumP(dotRow0 + nC1 * nBG + ib, nMono);
        } else if(col <= nComp + 1) {
          const int i1 = (col - 2) / nC2 + 1, i2 = (col - 2) % nC2;
          v = sumP(dotRow0 + (i1 - 1) * nBG + ib, mono(kp[i2].x, kp[i2].y));
        } else {
          const int jb = col - (nComp + 2);
          v = sumP(dotRow0 + nC1 * nBG + nBG + ib * nBG + jb, nMono);
        }
      }
      M[(size_t)row * ld + col] = v;
      M[(size_t)col * ld + row] = v;
    } else if(e < nTri + nSol) {
      const int id = (int)(e - nTri);
      double v = 0.0;
      if(id == 1) {
        v = sumP(bRow0, mono(0, 0));
      } else if(id >= 2 && id < nComp + 2) {
        const int i = (id - 2) / nC2 + 1, j = (id - 2) % nC2;
        v = sumP(bRow0 + i, mono(kp[j].x, kp[j].y));
      } else if(id >= nComp + 2 && id < nComp + 2 + nBG) {
        v = sumP(dotRow0 + bgBase + (id - (nComp + 2)), mono(0, 0));
      }
      rhs[id] = v;
    } else {
      const int i = (int)(e - nTri - nSol);
      M[i] = 0.0;
      M[(size_t)i * ld] = 0.0;
    }
  }
}

}  // namespace

// ============================================================ host side ===

int mixedLd(const Geo& g) { return (g.wCols + 31) / 32 * 32; }

int mixedDotStride(const Geo& g) { return g.nComp1 * g.nBG + g.nBG + g.nBG * g.nBG + 2 * g.nBG; }

void fillStampsMixed(xb_ctx* c, int si, const int* dList, int nList, int imgConv,
                     const int* liveN) {
  if(nList <= 0) return;
  const Geo& g = c->g;
  StampSetDev& S = c->set[si];
  const int ldW = mixedLd(g);
  const int nGroups = (int)c->basis.yGroupStart.size() - 1;
  const int tw = 2 * (g.hSS + g.hK) + 1, th = g.fSS;
  const size_t smemFill = (size_t)(tw * tw + th * tw + 4 * g.fK) * sizeof(float);
  const int other = 1 - imgConv;
  if(fillGramFits(c)) {
    // one kernel: window by TMA, Y and X passes, W to global, exact Gram
    const int R = g.wRows + 1;
    double* G = buf<double>(c, "gram_scratch", (size_t)nList * R * R);
    {
      KT_SCOPE(c, "fill_gram");
      fillGramLaunch(c, si, dList, nList, imgConv, G, liveN);
    }
    KT_SCOPE(c, "gram_scatter");
    k_gram_scatter<<<nList, MX_THREADS, 0, c->stream>>>(dList, liveN, S.count, S.cur, g.wRows,
                                                        g.nPSF, g.nBG, g.qCount, G, S.Q, S.B,
                                                        S.dots, mixedDotStride(g));
    XB_LAUNCHED(c);
    return;
  }
  {
    KT_SCOPE(c, "fill_w");
    dim3 grid(nList, nGroups);
    if(c->imgIsF64)
      k_fill_w_f32<double><<<grid, MX_THREADS, smemFill, c->stream>>>(
          (const double*)c->img[imgConv], c->w, c->h, dList, liveN, S.count, S.cur, S.ssxy,
          g.maxSS, c->dFX, c->dFY, c->dYGroupStart, c->dYGroupMembers, g.hSS, g.hK, g.wRows, ldW, S.Wf,
          S.Wlo);
    else
      k_fill_w_f32<float><<<grid, MX_THREADS, smemFill, c->stream>>>(
          (const float*)c->img[imgConv], c->w, c->h, dList, liveN, S.count, S.cur, S.ssxy,
          g.maxSS, c->dFX, c->dFY, c->dYGroupStart, c->dYGroupMembers, g.hSS, g.hK, g.wRows, ldW, S.Wf,
          S.Wlo);
    XB_LAUNCHED(c);
  }
  {
    KT_SCOPE(c, "fill_finish");
    k_fill_finish_f32<<<nList, MX_THREADS, 0, c->stream>>>(
        dList, liveN, S.count, S.cur, S.ssxy, g.maxSS, c->dKx, c->dKy, g.nPSF, buf<int2>(c, "bgXY", g.nBG),
        g.nBG, g.hSS, c->w, c->h, g.wRows, ldW, S.Wf, S.Wlo);
    XB_LAUNCHED(c);
  }
  {
    KT_SCOPE(c, "gram");
    const int R = g.wRows + 1;
    const size_t smem = (size_t)R * (GM_KT + 1) * sizeof(double);
    // one Gram entry per thread of the split CTAs
    const int split = std::max(GM_SPLIT, (R * (R + 1) / 2 + MX_THREADS - 1) / MX_THREADS);
    double* G = buf<double>(c, "gram_scratch", (size_t)nList * R * R);
    dim3 grid(nList, split);
    if(!c->p.fitWeighted && gramTensorCores(c, si, dList, nList, other, G, liveN)) {
      // exact tensor-core Gram (xb_gram_tc.cu)
    } else if(c->imgIsF64)
      k_gram_mixed<double><<<grid, MX_THREADS, smem, c->stream>>>(
          (const double*)c->img[other], (const double*)c->img[imgConv], c->w, c->h, dList, liveN,
          S.count, S.cur, S.ssxy, g.maxSS, g.hSS, g.wRows, ldW, S.Wf, S.Wlo, G, c->p.fitWeighted,
          noiseInvGain(c->p), noiseRn2x2(c->p));
    else
      k_gram_mixed<float><<<grid, MX_THREADS, smem, c->stream>>>(
          (const float*)c->img[other], (const float*)c->img[imgConv], c->w, c->h, dList, liveN,
          S.count, S.cur, S.ssxy, g.maxSS, g.hSS, g.wRows, ldW, S.Wf, S.Wlo, G, c->p.fitWeighted,
          noiseInvGain(c->p), noiseRn2x2(c->p));
    XB_LAUNCHED(c);
    k_gram_scatter<<<nList, MX_THREADS, 0, c->stream>>>(dList, liveN, S.count, S.cur, g.wRows,
                                                        g.nPSF, g.nBG, g.qCount, G, S.Q, S.B,
                                                        S.dots, mixedDotStride(g));
    XB_LAUNCHED(c);
  }
}

void sigsMixed(xb_ctx* c, int si, const int* dList, int nList, const double* dSol, int convImg,
               double* dSig, const int* liveN) {
  if(nList <= 0) return;
  const Geo& g = c->g;
  StampSetDev& S = c->set[si];
  const int other = 1 - convImg;
  KT_SCOPE(c, "sigs");
  if(c->imgIsF64)
    k_sigs_f32<double><<<nList, MX_THREADS, 0, c->stream>>>(
        dList, liveN, S.count, S.cur, S.ssxy, g.maxSS, S.Wf, g.wRows, mixedLd(g), g.hSS, g.nPSF,
        c->p.kernelOrder, c->p.backgroundOrder, g.nComp, dSol, (const double*)c->img[convImg],
        (const double*)c->img[other], c->mask, c->w, c->h, (float)noiseInvGain(c->p),
        (float)noiseRn2x2(c->p), dSig);
  else
    k_sigs_f32<float><<<nList, MX_THREADS, 0, c->stream>>>(
        dList, liveN, S.count, S.cur, S.ssxy, g.maxSS, S.Wf, g.wRows, mixedLd(g), g.hSS, g.nPSF,
        c->p.kernelOrder, c->p.backgroundOrder, g.nComp, dSol, (const float*)c->img[convImg],
        (const float*)c->img[other], c->mask, c->w, c->h, (float)noiseInvGain(c->p),
        (float)noiseRn2x2(c->p), dSig);
  XB_LAUNCHED(c);
}

// The pivoted LU and its refined solve, run only when the LDL^T factorisation
// flagged a pivot (status bit 0; both kernels return at once otherwise).  M is
// left intact, the factors go to F, rhs is replaced by the solution.
void luFallbackSolve(xb_ctx* c, const double* M, double* F, int n, double* rhs, int* piv,
                     int* singular, const int* status) {
  const int ld = n + 1;
  static std::atomic<int> clusterSize{0};
  auto launchLu = [&](auto kernel, int CL) -> cudaError_t {
    const int ncol = (n + CL - 1) / CL;
    const size_t smem = ((size_t)ncol * ld + ld + 2 * (ld + 1) + ld) * sizeof(double);
    cudaError_t e = allowMaxDynamicSmem((const void*)kernel, c->device);
    if(e != cudaSuccess) return e;
    if(CL > 8) {
      e = cudaFuncSetAttribute(kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
      if(e != cudaSuccess) return e;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(CL);
    cfg.blockDim = dim3(256);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = c->stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = CL;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, M, F, n, piv, singular, status);
  };
  {
    KT_SCOPE(c, "lu_fallback");
    cudaError_t e = cudaErrorUnknown;
    if(clusterSize.load() != 8) {
      e = launchLu(k_global_lu_fast<16>, 16);
      if(e == cudaSuccess) clusterSize = 16;
      else cudaGetLastError();
    }
    if(e != cudaSuccess) {
      XB_CUDA(launchLu(k_global_lu_fast<8>, 8));
      clusterSize = 8;
    }
    XB_LAUNCHED(c);
    const size_t smem = (size_t)4 * ld * sizeof(double) + (size_t)ld * sizeof(int);
    k_solve_refine<<<1, 1024, smem, c->stream>>>(F, M, n, piv, rhs, status);
    XB_LAUNCHED(c);
  }
}

// Global matrix and RHS of the mixed path for the stamps list[0..nList) of
// set si (weights from the current substamps, W dots per stamp).
void buildSystemMixed(xb_ctx* c, int si, const int* dList, int nList, int bgBase, double* M,
                      double* rhs, const int* liveN) {
  const Geo& g = c->g;
  StampSetDev& S = c->set[si];
  const int K = c->p.kernelOrder, monoDim = 2 * K + 1;
  const int nMono = triNum(2 * K + 1);
  if(nMono + 1 > MXB_MAXC)
    throw XbError{XB_ERR_UNSUPPORTED, "kernel order too high for the mixed build"};
  // monomial exponents, their index table and the kernel powers: fixed by
  // the parameters, uploaded once per context
  int2* dExp = buf<int2>(c, "mx_exp", nMono);
  int* dIdx = buf<int>(c, "mx_idx", (size_t)monoDim * monoDim);
  int2* dKp = buf<int2>(c, "mx_kp", g.nComp2);
  if(!c->mxTables) {
    std::vector<int2> mexp;
    std::vector<int> midx(monoDim * monoDim, 0);
    for(int a = 0; a <= 2 * K; a++)
      for(int b = 0; a + b <= 2 * K; b++) {
        midx[a * monoDim + b] = (int)mexp.size();
        mexp.push_back(make_int2(a, b));
      }
    std::vector<int2> kp(g.nComp2);
    for(int k = 0; k < g.nComp2; k++) kp[k] = make_int2(c->basis.kpX[k], c->basis.kpY[k]);
    toDevice(c, dExp, mexp);
    toDevice(c, dIdx, midx);
    toDevice(c, dKp, kp);
    c->mxTables = 1;
  }
  const int stride = mixedDotStride(g);
  const int nQP = (g.nComp1 + 1) * (g.nComp1 + 2) / 2 - 1;
  const int nRows = nQP + 1 + stride + g.nComp1 + 1;
  const int nSplit = (nList + MXB_T - 1) / MXB_T;
  double* P = buf<double>(c, "mx_partials", (size_t)std::max(nSplit, 1) * nRows * (nMono + 1));
  if(nSplit > 0) {
    KT_SCOPE(c, "mx_build");
    float2* Ytab = buf<float2>(c, "mx_mono", (size_t)nList * (nMono + 1));
    k_mx_mono<<<std::min((nList * (nMono + 1) + 255) / 256, c->smCount * 4), 256, 0, c->stream>>>(
        dList, nList, liveN, S.count, S.cur, S.ssxy, g.maxSS, dExp, nMono, c->w, c->h, Ytab);
    XB_LAUNCHED(c);
    k_mx_build<<<dim3((nRows + MXB_ROWS - 1) / MXB_ROWS, nSplit), 256, 0, c->stream>>>(
        dList, nList, liveN, S.count, S.cur, S.ssxy, g.maxSS, S.Q, g.qCount, S.dots, stride, S.B,
        Ytab, nMono, g.nComp1, nRows, P);
    XB_LAUNCHED(c);
  }
  {
    KT_SCOPE(c, "mx_scatter");
    const long long nTri = (long long)g.matSize * (g.matSize + 1) / 2;
    const long long total = nTri + g.nSol + g.matSize + 1;
    k_mx_scatter<<<(int)std::min<long long>((total + 255) / 256, (long long)c->smCount * 4), 256,
                   0, c->stream>>>(P, nSplit, liveN, nRows, nMono, dKp, dIdx, monoDim, g.nComp1,
                                   g.nComp2, g.nBG, stride, bgBase, g.matSize, g.nSol, M, rhs);
    XB_LAUNCHED(c);
  }
}

void convSubMixed(xb_ctx* c, double* dKernSum) {
  const Geo& g = c->g;
  if(g.fK != 21) throw XbError{XB_ERR_UNSUPPORTED, "mixed conv is built for 21-px kernels"};
  const int I = c->chosen, O = 1 - c->chosen;
  if(c->imgIsF64) throw XbError{XB_ERR_UNSUPPORTED, "mixed mode takes FP32 images"};
  if(c->p.kernelOrder > 3 || c->p.backgroundOrder > 4)
    throw XbError{XB_ERR_UNSUPPORTED, "mixed conv: kernel order <= 3, background order <= 4"};
  const double* Kt = kernelTermsLaunch(c);
  ConvArgsF a{};
  a.w = c->w;
  a.h = c->h;
  a.hK = g.hK;
  a.fK = g.fK;
  a.nPSF = g.nPSF;
  a.kOrder = c->p.kernelOrder;
  a.bgOrder = c->p.backgroundOrder;
  a.nComp = g.nComp;
  a.scaleConv = (c->p.normalizeTemplate && c->convTemplate) || (!c->p.normalizeTemplate && !c->convTemplate);
  a.tH = (float)c->p.threshHigh;
  a.tL = (float)c->p.threshLow;
  const int xSteps = (c->w + g.fK - 1) / g.fK, ySteps = (c->h + g.fK - 1) / g.fK;
  a.xSteps = xSteps;
  double* blockXY = nullptr;
  if(!c->p.convPerPixel) {
    blockXY = buf<double>(c, "conv_block_xy", (size_t)(xSteps + ySteps));
    k_block_centres<<<(xSteps + ySteps + 127) / 128, 128, 0, c->stream>>>(c->w, c->h, g.fK, xSteps,
                                                                        ySteps, blockXY);
    XB_LAUNCHED(c);
  }
  auto launch = [&](int variant) {
    const float *Ii = (const float*)c->img[I], *Oi = (const float*)c->img[O];
    switch(variant) {
      case 0:
        k_conv_sub_f32<21, 4><<<dim3((xSteps + 3) / 4, ySteps), 4 * 21, ConvTileF<21, 4>::BYTES, c->stream>>>(
            Ii, Oi, c->dSol, Kt, blockXY, dKernSum, a, c->inputMask, c->mask, c->convF, c->diffF);
        break;
      case 1:
        k_conv_sub_f32<21, 6><<<dim3((xSteps + 5) / 6, ySteps), 6 * 21, ConvTileF<21, 6>::BYTES, c->stream>>>(
            Ii, Oi, c->dSol, Kt, blockXY, dKernSum, a, c->inputMask, c->mask, c->convF, c->diffF);
        break;
      default:
        k_conv_sub_f32<21, 8><<<dim3((xSteps + 7) / 8, ySteps), 8 * 21, ConvTileF<21, 8>::BYTES, c->stream>>>(
            Ii, Oi, c->dSol, Kt, blockXY, dKernSum, a, c->inputMask, c->mask, c->convF, c->diffF);
        break;
    }
    XB_LAUNCHED(c);
  };
  if(c->p.convPerPixel) {
    const int nC2 = g.nComp2, nk = g.fK * g.fK;
    const size_t smemPP = (size_t)nC2 * nk * sizeof(float);
    int optin = 0;
    XB_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->device));
    if(c->p.kernelOrder > MAX_KORDER || smemPP + 16 * 1024 > (size_t)optin)
      throw XbError{XB_ERR_UNSUPPORTED, "per-pixel kernel: kernel order too large"};
    XB_CUDA(allowMaxDynamicSmem((const void*)k_conv_sub_pp_f32<21, 2>, c->device));
    KT_SCOPE(c, "conv_sub");
    k_conv_sub_pp_f32<21, 2><<<dim3((xSteps + 1) / 2, ySteps), 2 * 63, smemPP, c->stream>>>(
        (const float*)c->img[I], (const float*)c->img[O], c->dSol, Kt, dKernSum, a, c->inputMask,
        c->mask, c->convF, c->diffF);
    XB_LAUNCHED(c);
  } else {
    // blocks per CTA: 4 (default), 6 or 8; the three give identical images
    XB_CUDA(allowMaxDynamicSmem((const void*)k_conv_sub_f32<21, 4>, c->device));
    XB_CUDA(allowMaxDynamicSmem((const void*)k_conv_sub_f32<21, 6>, c->device));
    XB_CUDA(allowMaxDynamicSmem((const void*)k_conv_sub_f32<21, 8>, c->device));
    const int v = tunedVariant(c, "conv_sub_f32", (long long)c->w * 100003LL + c->h, 3, launch);
    KT_SCOPE(c, "conv_sub");
    launch(v);
  }
  const long long n = (long long)c->w * c->h;
  k_border_f32<<<std::min<long long>((n + 255) / 256, c->smCount * 8), 256, 0, c->stream>>>(
      (const float*)c->img[O], c->w, c->h, g.hK, a.tH, a.tL, c->inputMask, c->mask, c->convF, c->diffF);
  XB_LAUNCHED(c);
}

double* kernelTermsLaunch(xb_ctx* c) {
  const Geo& g = c->g;
  const int nk = g.fK * g.fK;
  double* Kt = buf<double>(c, "kernel_terms", (size_t)g.nComp2 * nk);
  k_kernel_terms<<<(g.nComp2 * nk + 255) / 256, 256, 0, c->stream>>>(c->dSol, c->dVec, g.nPSF,
                                                                      g.nComp2, nk, Kt);
  XB_LAUNCHED(c);
  return Kt;
}

}  // namespace xb
