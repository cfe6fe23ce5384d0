// xb_gram_tc.cu — the per-stamp Gram matrices of the mixed path on the
// tensor cores (tcgen05), exactly, from a W held in global memory (the
// arithmetic, tiling and epilogue are in xb_tc.cuh).  Used for the shapes the
// fused fill + Gram kernel (xb_fill_gram.cu) does not take.

#include "xb_internal.h"
#include "xb_tc.cuh"

namespace xb {

namespace {

constexpr int GT_THREADS = 256;
constexpr size_t GT_SMEM =
    (size_t)(tc::CHUNK_SMEM > tc::EPI_BYTES ? tc::CHUNK_SMEM : tc::EPI_BYTES) + 1024;

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
    if(lane == 0) expo[r] = rowExponent(m);
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmemBase;
  const bool ok = gramChunks<GT_THREADS>(Ws, Wl, wRows, ldW, R, K, imgRow, expo, buf, bars, tmem,
                                         deadline);
  epilogue(tmem, (long long*)buf, expo, R, Gout + (size_t)t * R * R);
  if(tid == 0 && !ok) atomicOr(timeout, 1);
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
