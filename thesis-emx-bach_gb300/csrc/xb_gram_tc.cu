// xb_gram_tc.cu — the per-stamp Gram matrices of the mixed path on the
// tensor cores (tcgen05), exactly.
//
// X = [W rows; image row] (R <= 64 rows of FP32 over the K = fSS^2 substamp
// pixels) and G = X X^T feed createQ / createB and the global-matrix dots
// (cl_kern/cmv.cl:195-240, cdkscUtil.cpp:363-392).  The global normal matrix
// built from G has cond ~1e14, so G must carry FP64-level accuracy: rounding
// the products or the sums to FP32 moves the fitted kernel sum by percent.
//
// Exact slicing: row r is scaled by 2^-e_r (e_r = the exponent just above its
// largest |x|) and rounded to a 35-bit fixed-point integer Z, written as five
// signed base-128 digits q_0..q_4 (|q| <= 127, exact in BF16):
//     x ~= 2^e_r * sum_t q_t 2^-7(t+1),   |error| <= 2^(e_r - 36).
// Every slice-pair dot product P_tu[a][b] = sum_k q_{a,t,k} q_{b,u,k} is an
// integer of magnitude <= 961 * 127^2 < 2^24, so the tensor cores' FP32
// accumulation of BF16 products is exact.  Pairs with t + u <= 5 are combined
// exactly in int64 and rounded once:
//     G_ab = 2^(e_a + e_b - 49) * sum_{m<=5} 2^(7(5-m)) sum_{t+u=m} P_tu[a][b].
// The dropped pairs weigh < 2^-42 * K * 2^(e_a + e_b); the rounding of x,
// 2^-36 of the row maximum per element, dominates -- both far under the
// FP32 storage of W itself (2^-24 of every element).
//
// Tiling: one CTA per stamp.  The five slices are stacked as 5 x 64 rows;
// K is staged in chunks of 64 through two shared-memory buffers in the
// no-swizzle K-major layout (8-row x 16-byte core matrices: K-adjacent 128 B
// apart, 8-row groups 1024 B apart).  Per K step of 16 one thread issues
//   D1 (TMEM cols   0..255) += S01 x S0123^T   (M 128, N 256)
//   D2 (TMEM cols 256..319) += S01 x S4^T      (M 128, N 64)
//   D3 (TMEM cols 320..447) += S23 x S23^T     (M 128, N 128)
// which hold every block (t, u), t <= u, t + u <= 5; the blocks with t > u
// are the transposes.  tcgen05.commit on an mbarrier frees a buffer once its
// products are done; all waits are bounded by a global-timer deadline.

#include <cuda_bf16.h>

#include "xb_internal.h"

namespace xb {

namespace {

constexpr int GT_THREADS = 256;
constexpr int GT_RB = 64;          // rows per slice block
constexpr int GT_S = 5;            // slices
constexpr int GT_KC = 64;          // K per chunk
constexpr int GT_ROWS = GT_RB * GT_S;                  // 320
constexpr int GT_BUF = GT_ROWS * GT_KC * 2;            // bytes per buffer (40 KB)
constexpr int GT_SBO = (GT_KC / 8) * 128;              // bytes between 8-row groups
constexpr int GT_P1LD = 256 + 4, GT_P2LD = 64 + 4, GT_P3LD = 128 + 4;  // P3: slice-2 lanes only
constexpr size_t GT_P_BYTES = (size_t)(128 * GT_P1LD + 128 * GT_P2LD + 64 * GT_P3LD) * 4;
constexpr size_t GT_SMEM = (GT_P_BYTES > 2 * (size_t)GT_BUF ? GT_P_BYTES : 2 * (size_t)GT_BUF) + 1024;
constexpr unsigned long long GT_WAIT_NS = 2000000000ull;
constexpr int GT_STAGE = GT_RB * GT_KC * 4;            // one FP32 W chunk (16 KB)
static_assert(2 * GT_BUF + 2 * GT_STAGE <= (int)GT_P_BYTES, "staging fits the epilogue area");

__device__ __forceinline__ uint32_t smemU32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void cpAsync16(uint32_t dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void cpAsyncCommit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cpAsyncWaitOne() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }
__device__ __forceinline__ void cpAsyncWaitAll() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }
__device__ __forceinline__ unsigned long long gtTimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ bool gtTryWait(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}
// false once the deadline has passed
__device__ __forceinline__ bool gtWait(uint32_t bar, uint32_t parity, unsigned long long deadline) {
  while(!gtTryWait(bar, parity))
    if(gtTimer() > deadline) return false;
  return true;
}

// Shared-memory matrix descriptor: no swizzle, K-major core matrices.
__device__ __forceinline__ uint64_t gtDesc(uint32_t addr) {
  uint64_t d = 0;
  d |= (uint64_t)((addr >> 4) & 0x3FFFu);             // start address
  d |= (uint64_t)((128u >> 4) & 0x3FFFu) << 16;       // leading (K) byte offset
  d |= (uint64_t)(((uint32_t)GT_SBO >> 4) & 0x3FFFu) << 32;  // stride (M/N) byte offset
  d |= (uint64_t)1 << 46;                             // descriptor version
  return d;                                           // base offset 0, no swizzle
}
// Instruction descriptor, kind::f16: BF16 A and B (K-major), FP32 D.
__host__ __device__ constexpr uint32_t gtIdesc(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) |
         ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void gtMma(uint32_t dTmem, uint64_t a, uint64_t b, uint32_t idesc,
                                      uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(dTmem),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void gtLd16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,"
      "%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for(int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

}  // namespace

// Gout[t] (R x R, row-major, both triangles) for the stamps list[t];
// *timeout gets bit 0 set if a wait ran out of time.
template <class T>
__global__ void __launch_bounds__(GT_THREADS, 1)
    k_gram_tc(const T* __restrict__ other, int w, int h, const int* __restrict__ list,
              const int* __restrict__ liveN, const int* __restrict__ count, const int* __restrict__ cur,
              const int2* __restrict__ ssxy, int maxSS, int hSS, int wRows, int ldW,
              const float* __restrict__ W, double* __restrict__ Gout, int* __restrict__ timeout) {
  extern __shared__ __align__(1024) unsigned char gt_s[];
  __shared__ float imgRow[64 * GT_KC + 64];
  __shared__ int expo[GT_RB];
  __shared__ unsigned long long bars[2];
  __shared__ uint32_t tmemBase;
  __shared__ int sErr;
  if(liveN && (int)blockIdx.x >= *liveN) return;  // before any barrier or TMEM allocation
  const int t = blockIdx.x, s = list[t], tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int fSS = 2 * hSS + 1, K = fSS * fSS, R = wRows + 1;
  const int nChunk = (K + GT_KC - 1) / GT_KC;
  const float* Ws = W + (size_t)s * wRows * ldW;
  const bool live = cur[s] < count[s];
  const unsigned long long deadline = gtTimer() + GT_WAIT_NS;
  unsigned char* buf = (unsigned char*)(((uintptr_t)gt_s + 1023) & ~(uintptr_t)1023);

  // the image row of this substamp (the target of createB), zero-padded
  int2 c = make_int2(0, 0);
  if(live) c = ssxy[(size_t)s * maxSS + cur[s]];
  for(int k = tid; k < nChunk * GT_KC; k += GT_THREADS) {
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
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smemU32(&bars[0])) : "memory");
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smemU32(&bars[1])) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if(warp == 0) {  // 512 TMEM columns (448 used); this warp also frees them
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(
                     smemU32(&tmemBase))
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  __syncthreads();
  // per-row exponents: |x| < 2^e for the whole row
  for(int r = warp; r < GT_RB; r += GT_THREADS / 32) {
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

  // W chunks arrive one ahead through cp.async into two FP32 staging
  // buffers behind the operand buffers (the epilogue reuses the area later);
  // columns at or past ldW are not copied (the slicer zeroes k >= K).
  float* stage = (float*)(buf + 2 * GT_BUF);
  auto fetch = [&](int ch) {
    float* st = stage + (ch & 1) * (GT_STAGE / 4);
    for(int u = tid; u < GT_RB * (GT_KC / 4); u += GT_THREADS) {
      const int r = u / (GT_KC / 4), k = ch * GT_KC + (u % (GT_KC / 4)) * 4;
      if(r < wRows && k < ldW) cpAsync16(smemU32(st + r * GT_KC + (k - ch * GT_KC)), Ws + (size_t)r * ldW + k);
    }
    cpAsyncCommit();
  };
  fetch(0);
  for(int ch = 0; ch < nChunk; ch++) {
    const int b = ch & 1;
    unsigned char* B = buf + b * GT_BUF;
    if(ch + 1 < nChunk) {
      fetch(ch + 1);
      cpAsyncWaitOne();
    } else {
      cpAsyncWaitAll();
    }
    if(ch >= 2 && !gtWait(smemU32(&bars[b]), ((ch - 2) >> 1) & 1, deadline)) sErr = 1;
    __syncthreads();
    const float* stc = stage + (ch & 1) * (GT_STAGE / 4);
    // 16-byte units: (row, 8 consecutive k) -> 5 slice units
    for(int u = tid; u < GT_RB * (GT_KC / 8); u += GT_THREADS) {
      const int r = u % GT_RB, kg = u / GT_RB, k0 = ch * GT_KC + kg * 8;  // rows fastest
      uint32_t q[GT_S][4];
#pragma unroll
      for(int sl = 0; sl < GT_S; sl++) q[sl][0] = q[sl][1] = q[sl][2] = q[sl][3] = 0u;
      if(r < R) {
        const int er = expo[r];
#pragma unroll
        for(int e = 0; e < 8; e++) {
          const int k = k0 + e;
          float x = 0.f;
          if(k < K) x = r < wRows ? stc[r * GT_KC + (k - ch * GT_KC)] : imgRow[k];
          // |Z| = round(|x| 2^(35 - e_r)) from the float's fields, in integers:
          // x = m 2^(ex - 150) (m with its hidden bit), so Z = m 2^sh.  As
          // |x| <= 2^e_r (1 - 2^-24), |Z| <= 2^35 - 2^11: five digits suffice.
          const uint32_t xb = __float_as_uint(x);
          const int ex = (int)((xb >> 23) & 0xFFu);
          const uint32_t m = (xb & 0x7FFFFFu) | (ex ? 0x800000u : 0u);
          const int sh = (ex ? ex : 1) - 150 + 35 - er;
          unsigned long long mag;
          if(sh >= 0) mag = (unsigned long long)m << sh;
          else if(sh > -40) mag = ((unsigned long long)m + (1ull << (-sh - 1))) >> (-sh);
          else mag = 0;
          const bool neg = (xb >> 31) != 0;
#pragma unroll
          for(int sl = 0; sl < GT_S; sl++) {
            const int dgt = (int)((mag >> (7 * (GT_S - 1 - sl))) & 127u);
            const __nv_bfloat16 hb = __float2bfloat16_rn((float)(neg ? -dgt : dgt));
            const uint32_t bits = (uint32_t)__bfloat16_as_ushort(hb);
            q[sl][e >> 1] |= bits << ((e & 1) * 16);
          }
        }
      }
#pragma unroll
      for(int sl = 0; sl < GT_S; sl++) {
        const int row = sl * GT_RB + r;
        uint4* dst = (uint4*)(B + (row >> 3) * GT_SBO + kg * 128 + (row & 7) * 16);
        *dst = make_uint4(q[sl][0], q[sl][1], q[sl][2], q[sl][3]);
      }
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if(tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t base = smemU32(B);
#pragma unroll
      for(int kk = 0; kk < GT_KC / 16; kk++) {
        const uint32_t ko = kk * 2 * 128;  // two core matrices per K step
        const uint32_t acc = (ch > 0 || kk > 0) ? 1u : 0u;
        const uint64_t s01 = gtDesc(base + ko);
        const uint64_t s23 = gtDesc(base + ko + 2 * (GT_RB / 8) * GT_SBO);
        const uint64_t s4 = gtDesc(base + ko + 4 * (GT_RB / 8) * GT_SBO);
        gtMma(tmem + 0, s01, s01, gtIdesc(128, 256), acc);
        gtMma(tmem + 256, s01, s4, gtIdesc(128, 64), acc);
        gtMma(tmem + 320, s23, s23, gtIdesc(128, 128), acc);
      }
      asm volatile(
          "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
              smemU32(&bars[b]))
          : "memory");
    }
  }
  // the last commit covers every product issued before it
  {
    const int last = nChunk - 1;
    if(!gtWait(smemU32(&bars[last & 1]), (last >> 1) & 1, deadline)) {
      sErr = 1;
      // give products still in flight a second bounded chance before TMEM is freed
      gtWait(smemU32(&bars[last & 1]), (last >> 1) & 1, gtTimer() + GT_WAIT_NS);
    }
  }
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  // TMEM -> shared (the operand buffers are free now)
  float* P1 = (float*)buf;                 // 128 x GT_P1LD
  float* P2 = P1 + 128 * GT_P1LD;          // 128 x GT_P2LD
  float* P3 = P2 + 128 * GT_P2LD;          // 64 x GT_P3LD (slice-2 rows of D3)
  {
    const int q = warp & 3, half = warp >> 2, row = 32 * q + lane;
    const uint32_t lanes = (uint32_t)(32 * q) << 16;
    float v[16];
    for(int c0 = 128 * half; c0 < 128 * half + 128; c0 += 16) {
      gtLd16(tmem + lanes + c0, v);
#pragma unroll
      for(int i = 0; i < 16; i++) P1[row * GT_P1LD + c0 + i] = v[i];
    }
    for(int c0 = 32 * half; c0 < 32 * half + 32; c0 += 16) {
      gtLd16(tmem + lanes + 256 + c0, v);
#pragma unroll
      for(int i = 0; i < 16; i++) P2[row * GT_P2LD + c0 + i] = v[i];
    }
    if(q < 2)
      for(int c0 = 64 * half; c0 < 64 * half + 64; c0 += 16) {
        gtLd16(tmem + lanes + 320 + c0, v);
#pragma unroll
        for(int i = 0; i < 16; i++) P3[row * GT_P3LD + c0 + i] = v[i];
      }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if(warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem) : "memory");
  // P_tu[a][b] for t <= u from the blocks above
  auto pval = [&](int tt, int uu, int a, int bb) -> long long {
    float f;
    if(tt == 2) f = P3[a * GT_P3LD + GT_RB * (uu - 2) + bb];              // (2, 2), (2, 3)
    else if(uu <= 3) f = P1[(GT_RB * tt + a) * GT_P1LD + GT_RB * uu + bb];  // t <= 1
    else f = P2[(GT_RB * tt + a) * GT_P2LD + bb];                         // (0, 4)
    return (long long)__float2ll_rn(f);
  };
  double* G = Gout + (size_t)t * R * R;
  for(int e = tid; e < R * (R + 1) / 2; e += GT_THREADS) {
    int a = (int)((sqrtf(8.f * e + 1.f) - 1.f) * 0.5f);
    while((a + 1) * (a + 2) / 2 <= e) a++;
    while(a * (a + 1) / 2 > e) a--;
    const int bb = e - a * (a + 1) / 2;
    long long acc = 0;
#pragma unroll
    for(int tt = 0; tt < GT_S; tt++)
#pragma unroll
      for(int uu = 0; uu < GT_S; uu++) {
        if(tt + uu > GT_S) continue;
        const long long p = tt <= uu ? pval(tt, uu, a, bb) : pval(uu, tt, bb, a);
        acc += p * (1LL << (7 * (GT_S - tt - uu)));  // |acc| < 2^60
      }
    const int ex = expo[a] + expo[bb] - 49;
    const double g = (double)acc * __longlong_as_double((long long)(1023 + ex) << 52);
    G[a * R + bb] = g;
    G[bb * R + a] = g;
  }
  if(tid == 0 && sErr) atomicOr(timeout, 1);
}

template __global__ void k_gram_tc<float>(const float*, int, int, const int*, const int*,
                                          const int*, const int*, const int2*, int, int, int, int,
                                          const float*, double*, int*);
template __global__ void k_gram_tc<double>(const double*, int, int, const int*, const int*,
                                           const int*, const int*, const int2*, int, int, int,
                                           int, const float*, double*, int*);

// Launches the tensor-core Gram for nList stamps; false when the shape is
// outside its limits (R > 64 rows), so the caller uses the FP64 kernel.
bool gramTensorCores(xb_ctx* c, int si, const int* dList, int nList, int other, double* G,
                     const int* liveN) {
  const Geo& g = c->g;
  const int R = g.wRows + 1;
  if(c->gramFp64 || R > GT_RB || g.wCols > 1024) return false;
  StampSetDev& S = c->set[si];
  int* err = deviceStatus(c) + 1;  // the context's device-timeout word
  if(c->imgIsF64) {
    XB_CUDA(allowMaxDynamicSmem((const void*)k_gram_tc<double>, c->device));
    k_gram_tc<double><<<nList, GT_THREADS, GT_SMEM, c->stream>>>(
        (const double*)c->img[other], c->w, c->h, dList, liveN, S.count, S.cur, S.ssxy, g.maxSS,
        g.hSS, g.wRows, mixedLd(g), S.Wf, G, err);
  } else {
    XB_CUDA(allowMaxDynamicSmem((const void*)k_gram_tc<float>, c->device));
    k_gram_tc<float><<<nList, GT_THREADS, GT_SMEM, c->stream>>>(
        (const float*)c->img[other], c->w, c->h, dList, liveN, S.count, S.cur, S.ssxy, g.maxSS,
        g.hSS, g.wRows, mixedLd(g), S.Wf, G, err);
  }
  XB_LAUNCHED(c);
  return true;
}

}  // namespace xb
