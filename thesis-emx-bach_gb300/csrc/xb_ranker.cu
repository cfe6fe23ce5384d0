// xb_ranker.cu — learned substamp ranking (no counterpart in the reference).
//
// The reference tries each stamp's substamps in order of brightness
// (sss.cl:363-379) and replaces a substamp only after the global fit has
// rejected it (ksc.cl:1-72, cdkscUtil.cpp:686-802), one refit per round of
// rejections.  A small network scores every candidate substamp from
//   * 16 statistics of the template/science windows around it, and
//   * the 2 x 31 x 31 window pair itself (sky-subtracted, peak-normalised),
// and the candidates of each stamp are reordered by score before cmv, so the
// ones the fit would reject are tried last.  The ksc sigma-clip check still
// runs on every pick; the network only changes the order.
//
// Network (2161 parameters, row-major in the order below), computed with
// BF16 weights and FP32 activations and accumulation: the training kernels
// take FP32 master weights (Adam updates those) and round each to BF16 as it
// is loaded, the inference copy in a context is stored as BF16, so both
// evaluate the same BF16-weight network:
//   conv1 2->8, 5x5, stride 2   (31 -> 14), ReLU
//   conv2 8->8, 3x3, stride 2   (14 -> 6),  ReLU
//   conv3 8->8, 3x3, stride 1   (6 -> 4),   ReLU, mean over the 4x4 map -> 8
//   mlp   16->32,                ReLU
//   head  [pool 8, mlp 32] -> 1 logit (accept probability = sigmoid)
// Training: binary cross-entropy with per-sample weights; one CTA computes
// the forward pass, the loss and the gradient of one sample; the gradients
// are summed over the batch in sample order (deterministic) and Adam updates
// the parameters.  Everything runs on the GPU from the C ABI.

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <vector>

#include <cuda_bf16.h>

#include "xb_internal.h"

namespace xb {

namespace {

constexpr int RK_T = 128;  // threads per sample
constexpr int RK_WIN = 31, RK_HWIN = 15, RK_NS = 16, RK_C = 8, RK_H = 32;
constexpr int RK_S1 = 14, RK_S2 = 6, RK_S3 = 4;
constexpr int RK_PIX = 2 * RK_WIN * RK_WIN;
constexpr int O_C1W = 0, O_C1B = O_C1W + RK_C * 2 * 25, O_C2W = O_C1B + RK_C,
              O_C2B = O_C2W + RK_C * RK_C * 9, O_C3W = O_C2B + RK_C,
              O_C3B = O_C3W + RK_C * RK_C * 9, O_M1W = O_C3B + RK_C,
              O_M1B = O_M1W + RK_H * RK_NS, O_HW = O_M1B + RK_H, O_HB = O_HW + RK_C + RK_H,
              RK_NP = O_HB + 1;
static_assert(RK_NP == 2161, "parameter layout");

// A weight as the network uses it: the FP32 master rounded to BF16 (nearest,
// ties to even), or a stored BF16 weight, as a float.
__device__ __forceinline__ float rkWeight(const float* W, int q) {
  return __bfloat162float(__float2bfloat16_rn(W[q]));
}
__device__ __forceinline__ float rkWeight(const __nv_bfloat16* W, int q) { return __bfloat162float(W[q]); }

// Activations of one sample (shared memory).
struct RkAct {
  float in[RK_PIX];
  float a1[RK_C * RK_S1 * RK_S1];  // post-ReLU
  float a2[RK_C * RK_S2 * RK_S2];
  float a3[RK_C * RK_S3 * RK_S3];
  float st[RK_NS];
  float hid[RK_C + RK_H];          // [pool, mlp] (post-ReLU)
  float logit;
};

__device__ float rkForward(const float* __restrict__ W, RkAct& A) {
  const int tid = threadIdx.x;
  for(int o = tid; o < RK_C * RK_S1 * RK_S1; o += RK_T) {
    const int c = o / (RK_S1 * RK_S1), y = (o / RK_S1) % RK_S1, x = o % RK_S1;
    float v = W[O_C1B + c];
    for(int ci = 0; ci < 2; ci++)
      for(int ky = 0; ky < 5; ky++)
        for(int kx = 0; kx < 5; kx++)
          v = fmaf(W[O_C1W + ((c * 2 + ci) * 5 + ky) * 5 + kx],
                   A.in[(ci * RK_WIN + 2 * y + ky) * RK_WIN + 2 * x + kx], v);
    A.a1[o] = fmaxf(v, 0.f);
  }
  __syncthreads();
  for(int o = tid; o < RK_C * RK_S2 * RK_S2; o += RK_T) {
    const int c = o / (RK_S2 * RK_S2), y = (o / RK_S2) % RK_S2, x = o % RK_S2;
    float v = W[O_C2B + c];
    for(int ci = 0; ci < RK_C; ci++)
      for(int ky = 0; ky < 3; ky++)
        for(int kx = 0; kx < 3; kx++)
          v = fmaf(W[O_C2W + ((c * RK_C + ci) * 3 + ky) * 3 + kx],
                   A.a1[(ci * RK_S1 + 2 * y + ky) * RK_S1 + 2 * x + kx], v);
    A.a2[o] = fmaxf(v, 0.f);
  }
  __syncthreads();
  for(int o = tid; o < RK_C * RK_S3 * RK_S3; o += RK_T) {
    const int c = o / (RK_S3 * RK_S3), y = (o / RK_S3) % RK_S3, x = o % RK_S3;
    float v = W[O_C3B + c];
    for(int ci = 0; ci < RK_C; ci++)
      for(int ky = 0; ky < 3; ky++)
        for(int kx = 0; kx < 3; kx++)
          v = fmaf(W[O_C3W + ((c * RK_C + ci) * 3 + ky) * 3 + kx],
                   A.a2[(ci * RK_S2 + y + ky) * RK_S2 + x + kx], v);
    A.a3[o] = fmaxf(v, 0.f);
  }
  for(int j = tid; j < RK_H; j += RK_T) {
    float v = W[O_M1B + j];
    for(int i = 0; i < RK_NS; i++) v = fmaf(W[O_M1W + j * RK_NS + i], A.st[i], v);
    A.hid[RK_C + j] = fmaxf(v, 0.f);
  }
  __syncthreads();
  if(tid < RK_C) {
    float v = 0.f;
    for(int p = 0; p < RK_S3 * RK_S3; p++) v += A.a3[tid * RK_S3 * RK_S3 + p];
    A.hid[tid] = v * (1.f / (RK_S3 * RK_S3));
  }
  __syncthreads();
  if(tid == 0) {
    float z = W[O_HB];
    for(int i = 0; i < RK_C + RK_H; i++) z = fmaf(W[O_HW + i], A.hid[i], z);
    A.logit = z;
  }
  __syncthreads();
  return A.logit;
}

// Gradient of loss = sw * BCE(sigmoid(z), y) with respect to every
// parameter, written to g (RK_NP floats).  Uses the activations of rkForward.
struct RkGrad {
  float dz;
  float dh[RK_C + RK_H];
  float d3[RK_C * RK_S3 * RK_S3];  // dL/d(conv3 pre-activation)
  float d2[RK_C * RK_S2 * RK_S2];  // dL/d(conv2 pre-activation)
  float d1[RK_C * RK_S1 * RK_S1];  // dL/d(conv1 pre-activation)
};

__device__ void rkBackward(const float* __restrict__ W, const RkAct& A, RkGrad& D, float y,
                           float sw, float* __restrict__ g) {
  const int tid = threadIdx.x;
  if(tid == 0) {
    const float p = 1.f / (1.f + expf(-A.logit));
    D.dz = sw * (p - y);
  }
  __syncthreads();
  const float dz = D.dz;
  for(int i = tid; i < RK_C + RK_H; i += RK_T) {
    g[O_HW + i] = dz * A.hid[i];
    D.dh[i] = dz * W[O_HW + i];
  }
  if(tid == 0) g[O_HB] = dz;
  __syncthreads();
  // mlp
  for(int j = tid; j < RK_H; j += RK_T) {
    const float dp = A.hid[RK_C + j] > 0.f ? D.dh[RK_C + j] : 0.f;
    g[O_M1B + j] = dp;
    for(int i = 0; i < RK_NS; i++) g[O_M1W + j * RK_NS + i] = dp * A.st[i];
  }
  // pool -> conv3 pre-activation
  for(int o = tid; o < RK_C * RK_S3 * RK_S3; o += RK_T) {
    const int c = o / (RK_S3 * RK_S3);
    D.d3[o] = A.a3[o] > 0.f ? D.dh[c] * (1.f / (RK_S3 * RK_S3)) : 0.f;
  }
  __syncthreads();
  // conv3 weights / bias
  for(int q = tid; q < RK_C * RK_C * 9 + RK_C; q += RK_T) {
    if(q < RK_C * RK_C * 9) {
      const int c = q / (RK_C * 9), ci = (q / 9) % RK_C, ky = (q / 3) % 3, kx = q % 3;
      float v = 0.f;
      for(int y = 0; y < RK_S3; y++)
        for(int x = 0; x < RK_S3; x++)
          v = fmaf(D.d3[(c * RK_S3 + y) * RK_S3 + x], A.a2[(ci * RK_S2 + y + ky) * RK_S2 + x + kx], v);
      g[O_C3W + q] = v;
    } else {
      const int c = q - RK_C * RK_C * 9;
      float v = 0.f;
      for(int p = 0; p < RK_S3 * RK_S3; p++) v += D.d3[c * RK_S3 * RK_S3 + p];
      g[O_C3B + c] = v;
    }
  }
  // conv2 pre-activation
  for(int o = tid; o < RK_C * RK_S2 * RK_S2; o += RK_T) {
    const int ci = o / (RK_S2 * RK_S2), yy = (o / RK_S2) % RK_S2, xx = o % RK_S2;
    float v = 0.f;
    if(A.a2[o] > 0.f)
      for(int c = 0; c < RK_C; c++)
        for(int ky = 0; ky < 3; ky++)
          for(int kx = 0; kx < 3; kx++) {
            const int y = yy - ky, x = xx - kx;
            if(y < 0 || y >= RK_S3 || x < 0 || x >= RK_S3) continue;
            v = fmaf(D.d3[(c * RK_S3 + y) * RK_S3 + x], W[O_C3W + ((c * RK_C + ci) * 3 + ky) * 3 + kx], v);
          }
    D.d2[o] = v;
  }
  __syncthreads();
  for(int q = tid; q < RK_C * RK_C * 9 + RK_C; q += RK_T) {
    if(q < RK_C * RK_C * 9) {
      const int c = q / (RK_C * 9), ci = (q / 9) % RK_C, ky = (q / 3) % 3, kx = q % 3;
      float v = 0.f;
      for(int y = 0; y < RK_S2; y++)
        for(int x = 0; x < RK_S2; x++)
          v = fmaf(D.d2[(c * RK_S2 + y) * RK_S2 + x],
                   A.a1[(ci * RK_S1 + 2 * y + ky) * RK_S1 + 2 * x + kx], v);
      g[O_C2W + q] = v;
    } else {
      const int c = q - RK_C * RK_C * 9;
      float v = 0.f;
      for(int p = 0; p < RK_S2 * RK_S2; p++) v += D.d2[c * RK_S2 * RK_S2 + p];
      g[O_C2B + c] = v;
    }
  }
  // conv1 pre-activation
  for(int o = tid; o < RK_C * RK_S1 * RK_S1; o += RK_T) {
    const int ci = o / (RK_S1 * RK_S1), yy = (o / RK_S1) % RK_S1, xx = o % RK_S1;
    float v = 0.f;
    if(A.a1[o] > 0.f)
      for(int c = 0; c < RK_C; c++)
        for(int ky = 0; ky < 3; ky++)
          for(int kx = 0; kx < 3; kx++) {
            const int ty = yy - ky, tx = xx - kx;  // = 2y, 2x
            if(ty < 0 || tx < 0 || (ty & 1) || (tx & 1)) continue;
            const int y = ty >> 1, x = tx >> 1;
            if(y >= RK_S2 || x >= RK_S2) continue;
            v = fmaf(D.d2[(c * RK_S2 + y) * RK_S2 + x], W[O_C2W + ((c * RK_C + ci) * 3 + ky) * 3 + kx], v);
          }
    D.d1[o] = v;
  }
  __syncthreads();
  for(int q = tid; q < RK_C * 2 * 25 + RK_C; q += RK_T) {
    if(q < RK_C * 2 * 25) {
      const int c = q / 50, ci = (q / 25) % 2, ky = (q / 5) % 5, kx = q % 5;
      float v = 0.f;
      for(int y = 0; y < RK_S1; y++)
        for(int x = 0; x < RK_S1; x++)
          v = fmaf(D.d1[(c * RK_S1 + y) * RK_S1 + x], A.in[(ci * RK_WIN + 2 * y + ky) * RK_WIN + 2 * x + kx], v);
      g[O_C1W + q] = v;
    } else {
      const int c = q - RK_C * 2 * 25;
      float v = 0.f;
      for(int p = 0; p < RK_S1 * RK_S1; p++) v += D.d1[c * RK_S1 * RK_S1 + p];
      g[O_C1B + c] = v;
    }
  }
}

__device__ __forceinline__ void rkLoad(const float* __restrict__ stats, const float* __restrict__ pix,
                                       int i, RkAct& A) {
  for(int q = threadIdx.x; q < RK_PIX; q += RK_T) A.in[q] = pix[(size_t)i * RK_PIX + q];
  for(int q = threadIdx.x; q < RK_NS; q += RK_T) A.st[q] = stats[(size_t)i * RK_NS + q];
}

// slots (optional): the candidate slots of the stamps, maxSS per stamp; a
// slot that is empty, past nRank in its stamp or in a stamp past *liveN
// gets no score (k_rank_order reads none for it).
template <class WT>
__global__ void __launch_bounds__(RK_T)
    k_rank_forward(const WT* __restrict__ W, const float* __restrict__ stats,
                   const float* __restrict__ pix, int n, float* __restrict__ logit,
                   const int2* __restrict__ slots = nullptr, int maxSS = 1, int nRank = 1,
                   const int* __restrict__ liveN = nullptr) {
  __shared__ float Ws[RK_NP];
  __shared__ RkAct A;
  for(int q = threadIdx.x; q < RK_NP; q += RK_T) Ws[q] = rkWeight(W, q);
  for(int i = blockIdx.x; i < n; i += gridDim.x) {
    if(slots && ((liveN && i / maxSS >= *liveN) || i % maxSS >= nRank || slots[i].x == INT_MAX))
      continue;  // uniform over the CTA
    __syncthreads();
    rkLoad(stats, pix, i, A);
    __syncthreads();
    const float z = rkForward(Ws, A);
    if(threadIdx.x == 0) logit[i] = z;
  }
}

__global__ void __launch_bounds__(RK_T)
    k_rank_grad(const float* __restrict__ W, const float* __restrict__ stats,
                const float* __restrict__ pix, const float* __restrict__ label,
                const float* __restrict__ sweight, int n, float* __restrict__ gPer,
                float* __restrict__ loss) {
  __shared__ float Ws[RK_NP];
  __shared__ RkAct A;
  __shared__ RkGrad D;
  for(int q = threadIdx.x; q < RK_NP; q += RK_T) Ws[q] = rkWeight(W, q);
  for(int i = blockIdx.x; i < n; i += gridDim.x) {
    __syncthreads();
    rkLoad(stats, pix, i, A);
    __syncthreads();
    const float z = rkForward(Ws, A);
    const float y = label[i], sw = sweight ? sweight[i] : 1.f;
    if(threadIdx.x == 0)  // sw * BCE with logits, stable form
      loss[i] = sw * (fmaxf(z, 0.f) - z * y + log1pf(expf(-fabsf(z))));
    rkBackward(Ws, A, D, y, sw, gPer + (size_t)i * RK_NP);
  }
}

// g[p] = (sum over samples in order of gPer[s][p]) * scale
__global__ void k_rank_reduce(const float* __restrict__ gPer, int n, float scale,
                              float* __restrict__ g) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if(p >= RK_NP) return;
  float v = 0.f;
  for(int s = 0; s < n; s++) v += gPer[(size_t)s * RK_NP + p];
  g[p] = v * scale;
}

__global__ void k_rank_adam(float* __restrict__ W, const float* __restrict__ g,
                            float* __restrict__ m, float* __restrict__ v, float lr, float b1,
                            float b2, float eps, float c1, float c2) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if(p >= RK_NP) return;
  const float gp = g[p];
  const float mp = b1 * m[p] + (1.f - b1) * gp;
  const float vp = b2 * v[p] + (1.f - b2) * gp * gp;
  m[p] = mp;
  v[p] = vp;
  W[p] -= lr * (mp / c1) / (sqrtf(vp / c2) + eps);
}

// ---------------------------------------------------------------- features --
// One CTA per candidate (stamp s of the set, slot k): the 16 statistics and
// the normalised window pair.  T = the template, S = the science image.
template <class T>
__global__ void __launch_bounds__(RK_T)
    k_rank_features(const T* __restrict__ imT, const T* __restrict__ imS,
                    const uint16_t* __restrict__ mask, int w, int h, const int* __restrict__ orig,
                    const int2* __restrict__ ssxy, int maxSS, const int2* __restrict__ cand,
                    int nCand, const int* __restrict__ liveN,
                    const double* __restrict__ skyT, const double* __restrict__ sigT,
                    const double* __restrict__ skyS, const double* __restrict__ sigS,
                    float threshHigh, float* __restrict__ stats, float* __restrict__ pix) {
  __shared__ float wt[RK_WIN * RK_WIN], ws[RK_WIN * RK_WIN];
  __shared__ float red[16][RK_T / 32];
  __shared__ float sh[16];
  const int i = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if(i >= nCand) return;
  // candidates from the list, or (no list) slot i % maxSS of stamp i / maxSS,
  // whose features are zero when the slot is empty or the stamp not kept
  int s, k;
  if(cand) {
    s = cand[i].x;
    k = cand[i].y;
  } else {
    s = i / maxSS;
    k = i % maxSS;
    if((liveN && s >= *liveN) || ssxy[(size_t)s * maxSS + k].x == INT_MAX) {
      for(int q = tid; q < RK_NS; q += RK_T) stats[(size_t)i * RK_NS + q] = 0.f;
      for(int q = tid; q < RK_PIX; q += RK_T) pix[(size_t)i * RK_PIX + q] = 0.f;
      return;
    }
  }
  const int o = orig[s];
  const int2 c = ssxy[(size_t)s * maxSS + k];
  int nValid = 0;
  for(int q = 0; q < maxSS; q++) nValid += ssxy[(size_t)s * maxSS + q].x != INT_MAX;
  const float bT = (float)skyT[o], bS = (float)skyS[o];
  const float gT = fmaxf((float)sigT[o], 1e-3f), gS = fmaxf((float)sigS[o], 1e-3f);
  float acc[16];
  for(int q = 0; q < 16; q++) acc[q] = 0.f;
  float mxT = -INFINITY, mxS = -INFINITY, rawMax = -INFINITY;
  for(int p = tid; p < RK_WIN * RK_WIN; p += RK_T) {
    const int dx = p % RK_WIN - RK_HWIN, dy = p / RK_WIN - RK_HWIN;
    const int gx = min(max(c.x + dx, 0), w - 1), gy = min(max(c.y + dy, 0), h - 1);
    const size_t gi = (size_t)gx + (size_t)gy * w;
    const float vT = (float)imT[gi], vS = (float)imS[gi];
    rawMax = fmaxf(rawMax, fmaxf(vT, vS));
    const float a = vT - bT, b = vS - bS;
    wt[p] = a;
    ws[p] = b;
    mxT = fmaxf(mxT, a);
    mxS = fmaxf(mxS, b);
    const float ap = fmaxf(a, 0.f), bp = fmaxf(b, 0.f), r2 = (float)(dx * dx + dy * dy);
    acc[0] += a;                     // flux T
    acc[1] += b;                     // flux S
    acc[2] += (mask[gi] & (BAD_INPUT | BAD_PIXEL_T | BAD_PIXEL_S | NAN_PIXEL)) ? 1.f : 0.f;
    acc[3] += ap;
    acc[4] += ap * r2;
    acc[5] += ap * dx;
    acc[6] += ap * dy;
    acc[7] += bp;
    acc[8] += bp * r2;
    acc[9] += bp * dx;
    acc[10] += bp * dy;
    acc[11] += a * b;
    acc[12] += a * a;
    acc[13] += b * b;
    acc[14] += (a > 20.f * gT) ? 1.f : 0.f;
  }
  // block reductions: sums 0..14 and the T peak into red[]; the S peak and
  // the raw maximum into mx2[]
  for(int q = 0; q < 15; q++) {
    float v = acc[q];
#pragma unroll
    for(int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    if(lane == 0) red[q][warp] = v;
  }
  float m3[3] = {mxT, mxS, rawMax};
  for(int q = 0; q < 3; q++) {
#pragma unroll
    for(int off = 16; off > 0; off >>= 1) m3[q] = fmaxf(m3[q], __shfl_xor_sync(0xffffffffu, m3[q], off));
  }
  __shared__ float mx2[2][RK_T / 32];
  if(lane == 0) {
    red[15][warp] = m3[0];
    mx2[0][warp] = m3[1];
    mx2[1][warp] = m3[2];
  }
  __syncthreads();
  if(tid < 16) {
    float v = tid == 15 ? -INFINITY : 0.f;
    for(int q = 0; q < RK_T / 32; q++) v = tid == 15 ? fmaxf(v, red[15][q]) : v + red[tid][q];
    sh[tid] = v;
  }
  __syncthreads();
  float pS = -INFINITY, rmax = -INFINITY;
  for(int q = 0; q < RK_T / 32; q++) {
    pS = fmaxf(pS, mx2[0][q]);
    rmax = fmaxf(rmax, mx2[1][q]);
  }
  const float pT = sh[15];
  // sharpness: largest excess of a pixel over its 4-neighbour mean (cosmic rays)
  float sharp = 0.f;
  for(int p = tid; p < RK_WIN * RK_WIN; p += RK_T) {
    const int x = p % RK_WIN, y = p / RK_WIN;
    if(x == 0 || y == 0 || x == RK_WIN - 1 || y == RK_WIN - 1) continue;
    const float nT = 0.25f * (wt[p - 1] + wt[p + 1] + wt[p - RK_WIN] + wt[p + RK_WIN]);
    const float nS = 0.25f * (ws[p - 1] + ws[p + 1] + ws[p - RK_WIN] + ws[p + RK_WIN]);
    sharp = fmaxf(sharp, fmaxf((wt[p] - nT) / (fabsf(pT) + gT), (ws[p] - nS) / (fabsf(pS) + gS)));
  }
#pragma unroll
  for(int off = 16; off > 0; off >>= 1) sharp = fmaxf(sharp, __shfl_xor_sync(0xffffffffu, sharp, off));
  __shared__ float shp[RK_T / 32];
  if(lane == 0) shp[warp] = sharp;
  // normalised window pair
  const float nT = 1.f / (fmaxf(pT, 0.f) + gT), nS = 1.f / (fmaxf(pS, 0.f) + gS);
  for(int p = tid; p < RK_WIN * RK_WIN; p += RK_T) {
    pix[(size_t)i * RK_PIX + p] = fminf(fmaxf(wt[p] * nT, -1.f), 2.f);
    pix[(size_t)i * RK_PIX + RK_WIN * RK_WIN + p] = fminf(fmaxf(ws[p] * nS, -1.f), 2.f);
  }
  __syncthreads();
  if(tid == 0) {
    float shv = 0.f;
    for(int q = 0; q < RK_T / 32; q++) shv = fmaxf(shv, shp[q]);
    const float fT = sh[0], fS = sh[1], npx = (float)(RK_WIN * RK_WIN);
    const float momT = sh[4] / fmaxf(sh[3], 1e-20f), momS = sh[8] / fmaxf(sh[7], 1e-20f);
    float* f = stats + (size_t)i * RK_NS;
    f[0] = asinhf(pT / gT) * 0.125f;
    f[1] = asinhf(pS / gS) * 0.125f;
    f[2] = asinhf(fT / (gT * RK_WIN)) * 0.125f;
    f[3] = asinhf(fS / (gS * RK_WIN)) * 0.125f;
    f[4] = sh[2] / npx;
    f[5] = logf((momS + 1.f) / (momT + 1.f));
    f[6] = sh[5] / fmaxf(sh[3], 1e-20f) / RK_HWIN;
    f[7] = sh[6] / fmaxf(sh[3], 1e-20f) / RK_HWIN;
    f[8] = sh[9] / fmaxf(sh[7], 1e-20f) / RK_HWIN;
    f[9] = sh[10] / fmaxf(sh[7], 1e-20f) / RK_HWIN;
    f[10] = sh[11] / sqrtf(fmaxf(sh[12] * sh[13], 1e-30f));
    f[11] = (fS - fT) / (fabsf(fS) + fabsf(fT) + npx * (gT + gS));
    f[12] = (float)k / maxSS;
    f[13] = (float)nValid / maxSS;
    f[14] = rmax / threshHigh;
    f[15] = fminf(shv, 4.f);
  }
}

// The learned order of each kept stamp's candidates (one thread per stamp):
// the valid slots (a prefix of the stamp's maxSS slots) are reordered by
// their scores z, policy 1 moving those below zTau behind the others (each
// group in the reference's order), policy 2 sorting all by descending score
// (ties in the reference's order).
// Reorders the first nRank candidates of every stamp by score (the others
// keep their places after them).
__global__ void k_rank_order(int2* __restrict__ ssxy, double* __restrict__ ssval,
                             const float* __restrict__ z, int nBound,
                             const int* __restrict__ liveN, int maxSS, int nRank, int policy,
                             float zTau) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = liveN ? min(*liveN, nBound) : nBound;
  if(s >= n) return;
  int2 xy[MAX_MAXSS];
  double v[MAX_MAXSS];
  float sc[MAX_MAXSS];
  int order[MAX_MAXSS];
  int cnt = 0;
  for(int k = 0; k < maxSS; k++) {
    xy[k] = ssxy[(size_t)s * maxSS + k];
    v[k] = ssval[(size_t)s * maxSS + k];
    if(xy[k].x != INT_MAX && k < nRank) {
      sc[cnt] = z[(size_t)s * maxSS + k];
      order[cnt++] = k;
    }
  }
  if(policy == 2) {
    for(int a = 1; a < cnt; a++)  // stable insertion sort, descending
      for(int b = a; b > 0 && sc[b - 1] < sc[b]; b--) {
        const float t = sc[b - 1];
        sc[b - 1] = sc[b];
        sc[b] = t;
        const int u = order[b - 1];
        order[b - 1] = order[b];
        order[b] = u;
      }
  } else {
    int tmp[MAX_MAXSS], m = 0;
    for(int a = 0; a < cnt; a++)
      if(sc[a] >= zTau) tmp[m++] = order[a];
    for(int a = 0; a < cnt; a++)
      if(!(sc[a] >= zTau)) tmp[m++] = order[a];
    for(int a = 0; a < cnt; a++) order[a] = tmp[a];
  }
  for(int r = 0; r < cnt; r++) {
    ssxy[(size_t)s * maxSS + r] = xy[order[r]];
    ssval[(size_t)s * maxSS + r] = v[order[r]];
  }
}

}  // namespace

constexpr int kRankParams = RK_NP;

// Candidate list (stamp, slot) of set si: every valid substamp slot.
static int rankCandidates(xb_ctx* c, int si, std::vector<int2>& cand) {
  const Geo& g = c->g;
  StampSetDev& S = c->set[si];
  cand.clear();
  if(S.n <= 0) return 0;
  std::vector<int2> xy = toHost(c, S.ssxy, (size_t)S.n * g.maxSS);
  for(int s = 0; s < S.n; s++)
    for(int k = 0; k < g.maxSS; k++)
      if(xy[(size_t)s * g.maxSS + k].x != INT_MAX) cand.push_back(make_int2(s, k));
  return (int)cand.size();
}

// Features of every candidate of set si into device buffers (stats, pix).
static void rankFeatures(xb_ctx* c, int si, const std::vector<int2>& cand, float* dStats,
                         float* dPix) {
  const Geo& g = c->g;
  StampSetDev& S = c->set[si];
  const int n = (int)cand.size();
  if(n == 0) return;
  int2* dCand = buf<int2>(c, "rank_cand", n);
  toDevice(c, dCand, cand);
  if(c->imgIsF64)
    k_rank_features<double><<<n, RK_T, 0, c->stream>>>(
        (const double*)c->img[0], (const double*)c->img[1], c->mask, c->w, c->h, S.orig, S.ssxy,
        g.maxSS, dCand, n, nullptr, c->skyAll[0], c->fwhmAll[0], c->skyAll[1], c->fwhmAll[1],
        (float)c->p.threshHigh, dStats, dPix);
  else
    k_rank_features<float><<<n, RK_T, 0, c->stream>>>(
        (const float*)c->img[0], (const float*)c->img[1], c->mask, c->w, c->h, S.orig, S.ssxy,
        g.maxSS, dCand, n, nullptr, c->skyAll[0], c->fwhmAll[0], c->skyAll[1], c->fwhmAll[1],
        (float)c->p.threshHigh, dStats, dPix);
  XB_LAUNCHED(c);
}

// Reorders the valid substamp slots of every stamp of both sets; counts are
// unchanged.  Called after sss when a ranker is loaded and the "rank" option
// is on.  rank = 1: candidates whose accept probability is below the
// threshold (option "rank_tau", in thousandths) move behind the others, each
// group keeping the reference's order; rank = 2: all by descending score.
// Everything runs on the device (features of every slot, scores, the
// per-stamp reorder), so a frame graph captures it; S.dN, when set, holds the
// kept count and S.n bounds it.
void rankSubstamps(xb_ctx* c) {
  const float tau = c->rankTau / 1000.f;
  const float zTau = logf(tau / (1.f - tau));  // logit of the threshold
  const Geo& g = c->g;
  for(int si = 0; si < 2; si++) {
    StampSetDev& S = c->set[si];
    if(S.n <= 0) continue;
    const int n = S.n * g.maxSS;
    float* dStats = buf<float>(c, "rank_stats", (size_t)n * RK_NS);
    float* dPix = buf<float>(c, "rank_pix", (size_t)n * RK_PIX);
    float* dLogit = buf<float>(c, "rank_logit", n);
    const int nRank = c->rankCandidates > 0 ? std::min(c->rankCandidates, g.maxSS) : g.maxSS;
    if(c->imgIsF64)
      k_rank_features<double><<<n, RK_T, 0, c->stream>>>(
          (const double*)c->img[0], (const double*)c->img[1], c->mask, c->w, c->h, S.orig,
          S.ssxy, g.maxSS, nullptr, n, S.dN, c->skyAll[0], c->fwhmAll[0], c->skyAll[1],
          c->fwhmAll[1], (float)c->p.threshHigh, dStats, dPix);
    else
      k_rank_features<float><<<n, RK_T, 0, c->stream>>>(
          (const float*)c->img[0], (const float*)c->img[1], c->mask, c->w, c->h, S.orig,
          S.ssxy, g.maxSS, nullptr, n, S.dN, c->skyAll[0], c->fwhmAll[0], c->skyAll[1],
          c->fwhmAll[1], (float)c->p.threshHigh, dStats, dPix);
    XB_LAUNCHED(c);
    {
      KT_SCOPE(c, "rank_score");
      k_rank_forward<__nv_bfloat16><<<std::min(n, c->smCount * 8), RK_T, 0, c->stream>>>(
          (const __nv_bfloat16*)c->rankW, dStats, dPix, n, dLogit, S.ssxy, g.maxSS, nRank, S.dN);
      XB_LAUNCHED(c);
    }
    k_rank_order<<<(S.n + 127) / 128, 128, 0, c->stream>>>(S.ssxy, S.ssval, dLogit, S.n, S.dN,
                                                           g.maxSS, nRank, c->rank, zTau);
    XB_LAUNCHED(c);
  }
}

}  // namespace xb

using namespace xb;

namespace {
template <class F>
int rkGuard(xb_ctx* c, F&& f) {
  try {
    f();
    return XB_OK;
  } catch(const CudaError& e) {
    if(c) c->lastError = std::string(e.where) + ": " + cudaGetErrorString(e.code);
    return XB_ERR_CUDA;
  } catch(const XbError& e) {
    if(c) c->lastError = e.msg;
    return e.code;
  }
}
cudaError_t rkLaunched() { return cudaGetLastError(); }
}  // namespace

extern "C" {

int xb_ranker_param_count(void) { return kRankParams; }

int xb_ranker_set(xb_ctx* c, const float* weights, int n) {
  if(!c) return XB_ERR_ARG;
  return rkGuard(c, [&] {
    if(n != kRankParams || !weights) throw XbError{XB_ERR_ARG, "ranker weights: wrong count"};
    XB_CUDA(cudaSetDevice(c->device));
    // stored as BF16 (nearest, ties to even), the weights the network computes with
    std::vector<uint16_t> wb(kRankParams);
    for(int q = 0; q < kRankParams; q++) {
      uint32_t u;
      memcpy(&u, &weights[q], 4);
      if((u & 0x7F800000u) == 0x7F800000u && (u & 0x7FFFFFu)) wb[q] = (uint16_t)((u >> 16) | 0x40u);
      else wb[q] = (uint16_t)((u + 0x7FFFu + ((u >> 16) & 1u)) >> 16);
    }
    c->rankW = buf<uint16_t>(c, "rank_weights", kRankParams);
    XB_CUDA(cudaMemcpyAsync(c->rankW, wb.data(), sizeof(uint16_t) * kRankParams,
                            cudaMemcpyHostToDevice, c->stream));
    XB_CUDA(cudaStreamSynchronize(c->stream));
  });
}

int xb_ranker_features(xb_ctx* c, int set, float* stats, float* pix, int* stamp, int* slot,
                       int cap, int* nOut) {
  if(!c || set < 0 || set > 1 || !nOut) return XB_ERR_ARG;
  return rkGuard(c, [&] {
    XB_CUDA(cudaSetDevice(c->device));
    if(c->stage < 2) throw XbError{XB_ERR_STATE, "ranker features need sss first"};
    std::vector<int2> cand;
    const int n = rankCandidates(c, set, cand);
    *nOut = n;
    if(!stats && !pix && !stamp && !slot) return;
    if(n > cap) throw XbError{XB_ERR_ARG, "ranker features: capacity too small"};
    float* dStats = buf<float>(c, "rank_stats", (size_t)std::max(n, 1) * RK_NS);
    float* dPix = buf<float>(c, "rank_pix", (size_t)std::max(n, 1) * RK_PIX);
    rankFeatures(c, set, cand, dStats, dPix);
    if(stats)
      XB_CUDA(cudaMemcpyAsync(stats, dStats, sizeof(float) * n * RK_NS, cudaMemcpyDeviceToHost,
                              c->stream));
    if(pix)
      XB_CUDA(cudaMemcpyAsync(pix, dPix, sizeof(float) * (size_t)n * RK_PIX,
                              cudaMemcpyDeviceToHost, c->stream));
    XB_CUDA(cudaStreamSynchronize(c->stream));
    for(int i = 0; i < n; i++) {
      if(stamp) stamp[i] = cand[i].x;
      if(slot) slot[i] = cand[i].y;
    }
  });
}

int xb_ranker_forward(const float* dW, const float* dStats, const float* dPix, int n,
                      float* dLogit, void* stream) {
  if(n < 0 || (n > 0 && (!dW || !dStats || !dPix || !dLogit))) return XB_ERR_ARG;
  if(n == 0) return XB_OK;
  k_rank_forward<float><<<std::min(n, 4096), RK_T, 0, (cudaStream_t)stream>>>(dW, dStats, dPix, n,
                                                                              dLogit);
  return rkLaunched() == cudaSuccess ? XB_OK : XB_ERR_CUDA;
}

int xb_ranker_grad(const float* dW, const float* dStats, const float* dPix, const float* dLabel,
                   const float* dWeight, int n, float* dGradPerSample, float* dGrad,
                   float* dLoss, void* stream) {
  if(n <= 0 || !dW || !dStats || !dPix || !dLabel || !dGradPerSample || !dGrad || !dLoss)
    return XB_ERR_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  k_rank_grad<<<std::min(n, 4096), RK_T, 0, st>>>(dW, dStats, dPix, dLabel, dWeight, n,
                                                  dGradPerSample, dLoss);
  if(rkLaunched() != cudaSuccess) return XB_ERR_CUDA;
  k_rank_reduce<<<(RK_NP + 127) / 128, 128, 0, st>>>(dGradPerSample, n, 1.f / n, dGrad);
  return rkLaunched() == cudaSuccess ? XB_OK : XB_ERR_CUDA;
}

int xb_ranker_adam(float* dW, const float* dGrad, float* dM, float* dV, int step, float lr,
                   void* stream) {
  if(!dW || !dGrad || !dM || !dV || step < 1) return XB_ERR_ARG;
  const float b1 = 0.9f, b2 = 0.999f;
  k_rank_adam<<<(RK_NP + 127) / 128, 128, 0, (cudaStream_t)stream>>>(
      dW, dGrad, dM, dV, lr, b1, b2, 1e-8f, 1.f - powf(b1, (float)step), 1.f - powf(b2, (float)step));
  return rkLaunched() == cudaSuccess ? XB_OK : XB_ERR_CUDA;
}

}  // extern "C"
