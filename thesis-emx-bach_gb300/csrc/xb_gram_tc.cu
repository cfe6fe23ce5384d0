// xb_gram_tc.cu — the per-stamp Gram matrices of the mixed path on the
// tensor cores (tcgen05), exactly, from a W held in global memory (the
// arithmetic, tiling and epilogue are in xb_tc.cuh).  Used for the shapes the
// fused fill + Gram kernel (xb_fill_gram.cu) does not take.

#include "xb_internal.h"
#include "xb_tc.cuh"

namespace xb {

namespace {

constexpr int GT_THREADS = 256;
constexpr int GT_STAGE = tc::RB * tc::KC * 4;          // one FP32 W chunk (16 KB)
constexpr int GT_DYN = 2 * tc::OPBUF + 4 * GT_STAGE;   // operands + hi/lo staging
constexpr size_t GT_SMEM = (size_t)(GT_DYN > tc::EPI_BYTES ? GT_DYN : tc::EPI_BYTES) + 1024;

__device__ __forceinline__ void cpAsync16(uint32_t dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void cpAsyncCommit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cpAsyncWaitOne() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }
__device__ __forceinline__ void cpAsyncWaitAll() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

}  // namespace

// Gout[t] (R x R, row-major, both triangles) for the stamps list[t];
// *timeout gets bit 0 set if a wait ran out of time.
template <class T>
__global__ void __launch_bounds__(GT_THREADS, 1)
    k_gram_tc(const T* __restrict__ other, int w, int h, const int* __restrict__ list,
              const int* __restrict__ liveN, const int* __restrict__ count, const int* __restrict__ cur,
              const int2* __restrict__ ssxy, int maxSS, int hSS, int wRows, int ldW,
              const float* __restrict__ W, const float* __restrict__ Wlo, double* __restrict__ Gout,
              int* __restrict__ timeout) {
  using namespace tc;
  extern __shared__ __align__(1024) unsigned char gt_s[];
  __shared__ float imgRow[64 * KC + 64];
  __shared__ int expo[RB];
  __shared__ unsigned long long bars[2];
  __shared__ uint32_t tmemBase;
  __shared__ int sErr;
  if(liveN && (int)blockIdx.x >= *liveN) return;  // before any barrier or TMEM allocation
  const int t = blockIdx.x, s = list[t], tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int fSS = 2 * hSS + 1, K = fSS * fSS, R = wRows + 1;
  const int nChunk = (K + KC - 1) / KC;
  const float* Ws = W + (size_t)s * wRows * ldW;
  const float* Wl = Wlo + (size_t)s * wRows * ldW;
  const bool live = cur[s] < count[s];
  const unsigned long long deadline = timerNs() + WAIT_NS;
  unsigned char* buf = (unsigned char*)(((uintptr_t)gt_s + 1023) & ~(uintptr_t)1023);

  // the image row of this substamp (the target of createB), zero-padded
  int2 c = make_int2(0, 0);
  if(live) c = ssxy[(size_t)s * maxSS + cur[s]];
  for(int k = tid; k < nChunk * KC; k += GT_THREADS) {
    float v = 0.f;
    if(live && k < K) {
      const int gx = min(max(c.x - hSS + k % fSS, 0), w - 1);
      const int gy = min(max(c.y - hSS + k / fSS, 0), h - 1);
      v = (float)other[(size_t)gx + (size_t)gy * w];
    }
    imgRow[k] = v;
  }
  if(tid == 0) {
    sErr = 0;
    barInit(smemU32(&bars[0]), 1);
    barInit(smemU32(&bars[1]), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if(warp == 0) tmemAlloc512(&tmemBase);
  __syncthreads();
  // per-row exponents: |hi| < 2^e for the whole row
  for(int r = warp; r < RB; r += GT_THREADS / 32) {
    float m = 0.f;
    if(r < R) {
      // four running maxima keep four loads in flight (max is exact in any order)
      const float* src = r < wRows ? Ws + (size_t)r * ldW : imgRow;
      float m1 = 0.f, m2 = 0.f, m3 = 0.f;
      int k = lane;
      for(; k + 96 < K; k += 128) {
        m = fmaxf(m, fabsf(src[k]));
        m1 = fmaxf(m1, fabsf(src[k + 32]));
        m2 = fmaxf(m2, fabsf(src[k + 64]));
        m3 = fmaxf(m3, fabsf(src[k + 96]));
      }
      for(; k < K; k += 32) m = fmaxf(m, fabsf(src[k]));
      m = fmaxf(fmaxf(m, m1), fmaxf(m2, m3));
    }
#pragma unroll
    for(int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if(lane == 0) {
      int e = 0;
      if(m > 0.f) frexpf(m, &e);
      expo[r] = e;
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmemBase;

  // W chunks (hi and lo) arrive one ahead through cp.async into FP32
  // staging buffers behind the operand buffers (the epilogue reuses the area
  // later); columns at or past ldW are not copied (the slicer zeroes k >= K).
  float* stage = (float*)(buf + 2 * OPBUF);
  auto fetch = [&](int ch) {
    float* st = stage + (ch & 1) * (GT_STAGE / 4);
    float* stl = st + 2 * (GT_STAGE / 4);
    for(int u = tid; u < RB * (KC / 4); u += GT_THREADS) {
      const int r = u / (KC / 4), k = ch * KC + (u % (KC / 4)) * 4;
      if(r < wRows && k < ldW) {
        cpAsync16(smemU32(st + r * KC + (k - ch * KC)), Ws + (size_t)r * ldW + k);
        cpAsync16(smemU32(stl + r * KC + (k - ch * KC)), Wl + (size_t)r * ldW + k);
      }
    }
    cpAsyncCommit();
  };
  fetch(0);
  for(int ch = 0; ch < nChunk; ch++) {
    const int b = ch & 1;
    unsigned char* B = buf + b * OPBUF;
    if(ch + 1 < nChunk) {
      fetch(ch + 1);
      cpAsyncWaitOne();
    } else {
      cpAsyncWaitAll();
    }
    if(ch >= 2 && !waitUntil(smemU32(&bars[b]), ((ch - 2) >> 1) & 1, deadline)) sErr = 1;
    __syncthreads();
    const float* stc = stage + (ch & 1) * (GT_STAGE / 4);
    const float* stl = stc + 2 * (GT_STAGE / 4);
    // 16-byte units: (row, 8 consecutive k) -> 5 slice units
    for(int u = tid; u < RB * (KC / 8); u += GT_THREADS) {
      const int r = u % RB, kg = u / RB, k0 = ch * KC + kg * 8;  // rows fastest
      float xh[8], xl[8];
#pragma unroll
      for(int e = 0; e < 8; e++) {
        const int k = k0 + e;
        xh[e] = xl[e] = 0.f;
        if(r < R && k < K) {
          if(r < wRows) {
            xh[e] = stc[r * KC + (k - ch * KC)];
            xl[e] = stl[r * KC + (k - ch * KC)];
          } else {
            xh[e] = imgRow[k];
          }
        }
      }
      uint32_t q[NS][4];
      slice8(xh, xl, r < R ? expo[r] : 0, q);
      storeSlices(B, r, kg, q);
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if(tid == 0) issueChunk(tmem, B, ch == 0, smemU32(&bars[b]));
  }
  // the last commit covers every product issued before it
  {
    const int last = nChunk - 1;
    if(!waitUntil(smemU32(&bars[last & 1]), (last >> 1) & 1, deadline)) {
      sErr = 1;
      // give products still in flight a second bounded chance before TMEM is freed
      waitUntil(smemU32(&bars[last & 1]), (last >> 1) & 1, timerNs() + WAIT_NS);
    }
  }
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  epilogue(tmem, (long long*)buf, expo, R, Gout + (size_t)t * R * R);
  if(tid == 0 && sErr) atomicOr(timeout, 1);
}

template __global__ void k_gram_tc<float>(const float*, int, int, const int*, const int*,
                                          const int*, const int*, const int2*, int, int, int, int,
                                          const float*, const float*, double*, int*);
template __global__ void k_gram_tc<double>(const double*, int, int, const int*, const int*,
                                           const int*, const int*, const int2*, int, int, int,
                                           int, const float*, const float*, double*, int*);

// Launches the tensor-core Gram for nList stamps; false when the shape is
// outside its limits (R > 64 rows), so the caller uses the FP64 kernel.
bool gramTensorCores(xb_ctx* c, int si, const int* dList, int nList, int other, double* G,
                     const int* liveN) {
  const Geo& g = c->g;
  const int R = g.wRows + 1;
  if(c->gramFp64 || R > tc::RB || g.wCols > 1024) return false;
  StampSetDev& S = c->set[si];
  int* err = deviceStatus(c) + 1;  // the context's device-timeout word
  if(c->imgIsF64) {
    XB_CUDA(allowMaxDynamicSmem((const void*)k_gram_tc<double>, c->device));
    k_gram_tc<double><<<nList, GT_THREADS, GT_SMEM, c->stream>>>(
        (const double*)c->img[other], c->w, c->h, dList, liveN, S.count, S.cur, S.ssxy, g.maxSS,
        g.hSS, g.wRows, mixedLd(g), S.Wf, S.Wlo, G, err);
  } else {
    XB_CUDA(allowMaxDynamicSmem((const void*)k_gram_tc<float>, c->device));
    k_gram_tc<float><<<nList, GT_THREADS, GT_SMEM, c->stream>>>(
        (const float*)c->img[other], c->w, c->h, dList, liveN, S.count, S.cur, S.ssxy, g.maxSS,
        g.hSS, g.wRows, mixedLd(g), S.Wf, S.Wlo, G, err);
  }
  XB_LAUNCHED(c);
  return true;
}

}  // namespace xb
