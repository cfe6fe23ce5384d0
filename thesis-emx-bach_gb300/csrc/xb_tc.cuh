// xb_tc.cuh — exact Gram matrices on the tensor cores (tcgen05), shared by
// the Gram kernel that reads W from global memory (xb_gram_tc.cu) and the
// fused fill + Gram kernel (xb_fill_gram.cu).
//
// X = [W rows; image row] (R <= 64 rows over the K = fSS^2 substamp pixels)
// and G = X X^T feed createQ / createB and the global-matrix dots
// (cl_kern/cmv.cl:195-240, cdkscUtil.cpp:363-392).  The global normal matrix
// built from G has cond ~1e14, so G must carry FP64-level accuracy, and it
// must be the Gram matrix of one consistent X: an error E added to the
// normal matrix moves an ill-conditioned fit by ~cond(X^T X) |E|, while the
// same error size in X itself moves it by only ~cond(X) |dX|.
//
// Exact slicing: each element x = hi + lo (two floats, ~48 bits) of row r is
// scaled by 2^-e_r (e_r = the exponent just above the row's largest |hi|) and
// rounded to a 35-bit fixed-point integer Z, written as five signed base-128
// digits q_0..q_4 (|q_0| <= 128, |q_t| <= 80 for t >= 1, exact in BF16;
// slice8 below):
//     x ~= 2^e_r * sum_t q_t 2^-7(t+1),   |error| <= 2^(e_r - 36).
// Every slice-pair dot product P_tu[a][b] = sum_k q_{a,t,k} q_{b,u,k} is an
// integer of magnitude <= 961 * 128^2 < 2^24 (K <= 961: substamps up to
// 31 x 31), so the tensor cores' FP32 accumulation of BF16 products is exact.
// All pairs but (4, 4) are summed exactly in int64 and rounded once:
//     G_ab = 2^(e_a + e_b - 63) * sum_{m<=7} 2^(7(7-m)) sum_{t+u=m} P_tu[a][b],
// i.e. G is the Gram matrix of the rounded X up to the pair (4, 4) (2^-56 of
// the leading pair) and the final FP64 rounding.  (On the reference's own
// test case, whose global system has cond ~6e13, a consistent 35-bit
// rounding moves the difference image by ~1e-5 of the pixel noise; keeping
// only the pairs t + u <= 5, 2^-42 of the leading pair but inconsistent,
// moved it by 2.3e-3.)
//
// Tiling: one CTA per stamp.  The five slices are stacked as 5 x 64 rows;
// K is staged in chunks of 64 through two shared-memory buffers in the
// no-swizzle K-major layout (8-row x 16-byte core matrices: K-adjacent 128 B
// apart, 8-row groups 1024 B apart).  Per K step of 16 one thread issues
//   D1 (TMEM cols   0..255) += S01 x S0123^T   (M 128, N 256)
//   D2 (TMEM cols 256..319) += S01 x S4^T      (M 128, N 64)
//   D3 (TMEM cols 320..511) += S23 x S234^T    (M 128, N 192)
// whose 32 blocks of 64 x 64 hold P_tu for t in {0,1} and every u, and for
// t in {2,3} and u >= 2; the other pairs are their transposes.
// tcgen05.commit on an mbarrier frees a buffer once its products are done;
// every wait is bounded by a global-timer deadline.
#pragma once

#include <stdint.h>

namespace xb {
namespace tc {

constexpr int RB = 64;                        // rows per slice block
constexpr int NS = 5;                         // slices
constexpr int KC = 64;                        // K per chunk
constexpr int ROWS = RB * NS;                 // 320
constexpr int OPBUF = ROWS * KC * 2;          // bytes per operand buffer (40 KB)
constexpr int SBO = (KC / 8) * 128;           // bytes between 8-row groups
constexpr int ELD = RB + 1;                   // int64 row stride of the epilogue sums
constexpr int EPI_BYTES = 4 * RB * ELD * 8;   // the four epilogue sum arrays (130 KB)
constexpr unsigned long long WAIT_NS = 2000000000ull;

__device__ __forceinline__ uint32_t smemU32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ unsigned long long timerNs() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ bool tryWait(uint32_t bar, uint32_t parity) {
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
__device__ __forceinline__ bool waitUntil(uint32_t bar, uint32_t parity, unsigned long long deadline) {
  while(!tryWait(bar, parity))
    if(timerNs() > deadline) return false;
  return true;
}
__device__ __forceinline__ void barInit(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

// Shared-memory matrix descriptor: no swizzle, K-major core matrices.
__device__ __forceinline__ uint64_t sdesc(uint32_t addr) {
  uint64_t d = 0;
  d |= (uint64_t)((addr >> 4) & 0x3FFFu);              // start address
  d |= (uint64_t)((128u >> 4) & 0x3FFFu) << 16;        // leading (K) byte offset
  d |= (uint64_t)(((uint32_t)SBO >> 4) & 0x3FFFu) << 32;  // stride (M/N) byte offset
  d |= (uint64_t)1 << 46;                              // descriptor version
  return d;                                            // base offset 0, no swizzle
}
// Instruction descriptor, kind::f16: BF16 A and B (K-major), FP32 D.
__host__ __device__ constexpr uint32_t idesc(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) |
         ((uint32_t)(M >> 4) << 24);
}
__device__ __forceinline__ void mma(uint32_t dTmem, uint64_t a, uint64_t b, uint32_t id,
                                    uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(dTmem),
      "l"(a), "l"(b), "r"(id), "r"(accumulate)
      : "memory");
}
// 32 lanes x 8 consecutive columns; the caller waits with ldWait()
__device__ __forceinline__ void ld8(uint32_t taddr, float* v) {
  uint32_t r[8];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7])
      : "r"(taddr));
#pragma unroll
  for(int i = 0; i < 8; i++) v[i] = __uint_as_float(r[i]);
}
// 32 lanes x 4 consecutive columns; the caller waits with ldWait()
__device__ __forceinline__ void ld4(uint32_t taddr, float* v) {
  uint32_t r[4];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(taddr));
#pragma unroll
  for(int i = 0; i < 4; i++) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void ldWait() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// 512 TMEM columns (one warp; the same warp frees them)
__device__ __forceinline__ void tmemAlloc512(uint32_t* dst) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(smemU32(dst))
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmemFree512(uint32_t tmem) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem) : "memory");
}

// 2^k as a float, -126 <= k <= 127
__device__ __forceinline__ float pow2f(int k) { return __int_as_float((127 + k) << 23); }
// nearest integer of |x| < 2^22 (ties to even): the sum's spacing is 1
__device__ __forceinline__ float rintSmall(float x) {
  const float big = 12582912.f;  // 1.5 * 2^23
  return (x + big) - big;
}

// The five BF16 digits of 8 consecutive elements (hi[e] + lo[e]) of a row
// with exponent er (|hi| < 2^er on the whole row), as 16-byte core-matrix
// rows q[slice][0..3].  With v = hi 2^(7 - er) (exact, |v| < 128):
//     d0 = rint(v), r = (v - d0) 128, d1 = rint(r), r = (r - d1) 128,
//     d2 = rint(r), r = (r - d2) 128 + lo 2^(28 - er), d3 = rint(r),
//     r = (r - d3) 128, d4 = rint(r),
// every step exact (each remainder is a multiple of ulp(v) below 1) except
// the one addition of lo, which rounds at 2^-46 of the row maximum; so
//     x ~= 2^(er - 35) Z,  Z = sum_t d_t 128^(4 - t),  |x - 2^(er-35) Z| <= 2^(er - 36),
// and |d0| <= 128, |d1|, |d2|, |d4| <= 64, |d3| <= 80.  A digit is an integer
// of at most 8 significant bits, so its BF16 form is the float's upper half.
__device__ __forceinline__ void slice8(const float* hi, const float* lo, int er, uint32_t (&q)[NS][4]) {
  const float s7 = pow2f(7 - er), s28 = pow2f(28 - er);
#pragma unroll
  for(int e = 0; e < 8; e += 2) {
    float d[2][NS];
#pragma unroll
    for(int i = 0; i < 2; i++) {
      const float v = hi[e + i] * s7;
      d[i][0] = rintSmall(v);
      float r = (v - d[i][0]) * 128.f;
      d[i][1] = rintSmall(r);
      r = (r - d[i][1]) * 128.f;
      d[i][2] = rintSmall(r);
      r = (r - d[i][2]) * 128.f + lo[e + i] * s28;
      d[i][3] = rintSmall(r);
      r = (r - d[i][3]) * 128.f;
      d[i][4] = rintSmall(r);
    }
#pragma unroll
    for(int sl = 0; sl < NS; sl++)
      q[sl][e >> 1] = __byte_perm(__float_as_uint(d[0][sl]), __float_as_uint(d[1][sl]), 0x7632);
  }
}
// stores the digits of row r, K group kg (8 elements) into an operand buffer
__device__ __forceinline__ void storeSlices(unsigned char* B, int r, int kg, const uint32_t (&q)[NS][4]) {
#pragma unroll
  for(int sl = 0; sl < NS; sl++) {
    const int row = sl * RB + r;
    uint4* dst = (uint4*)(B + (row >> 3) * SBO + kg * 128 + (row & 7) * 16);
    *dst = make_uint4(q[sl][0], q[sl][1], q[sl][2], q[sl][3]);
  }
}

// One thread: the products of one K chunk of operand buffer B (after
// fence.proxy.async and a barrier), then a commit to the mbarrier bar.
__device__ __forceinline__ void issueChunk(uint32_t tmem, const unsigned char* B, bool first,
                                          uint32_t bar) {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t base = smemU32(B);
#pragma unroll
  for(int kk = 0; kk < KC / 16; kk++) {
    const uint32_t ko = kk * 2 * 128;  // two core matrices per K step
    const uint32_t acc = (!first || kk > 0) ? 1u : 0u;
    const uint64_t s01 = sdesc(base + ko);
    const uint64_t s23 = sdesc(base + ko + 2 * (RB / 8) * SBO);
    const uint64_t s4 = sdesc(base + ko + 4 * (RB / 8) * SBO);
    mma(tmem + 0, s01, s01, idesc(128, 256), acc);    // S01 x S0123
    mma(tmem + 256, s01, s4, idesc(128, 64), acc);    // S01 x S4
    mma(tmem + 320, s23, s23, idesc(128, 192), acc);  // S23 x S234
  }
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
               : "memory");
}

// The row exponent e (|hi| < 2^e on the row) from the row's largest |hi|;
// rows of nothing but zeros (or values below 2^-90) take -90, which keeps
// every scale factor of slice8 a normal float.
__device__ __forceinline__ int rowExponent(float m) {
  int e = 0;
  if(m > 0.f) frexpf(m, &e);
  return e < -90 ? -90 : e;
}

__device__ __forceinline__ void cpAsync16(uint32_t dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void cpAsyncCommit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cpAsyncWaitOne() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }
__device__ __forceinline__ void cpAsyncWaitAll() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

// FP32 W chunk staging: rows padded to KC + 4 floats, so that the slicing
// loop's 16-byte reads of eight consecutive rows fall on distinct banks
constexpr int SKC = KC + 4;
constexpr int STAGE_F = RB * SKC;  // floats of one staging buffer (17 KB)
// shared memory of the K-chunk loop: two operand buffers, then hi and lo
// staging for two chunks (the epilogue reuses the area)
constexpr int CHUNK_SMEM = 2 * OPBUF + 4 * STAGE_F * 4;

// The K-chunk loop of one stamp, run by all NT threads of the CTA: W rows
// r < wRows (hi at Ws, lo at Wl, row stride ldW, K valid columns) and the
// image row imgRow (shared, zero-padded to a whole chunk) as row wRows are
// staged by cp.async one chunk ahead, sliced with the row exponents expo[]
// into the operand buffers at buf (1024-aligned, CHUNK_SMEM bytes), and
// multiplied into TMEM by one thread; bars[0..1] are the operand buffers'
// commit barriers (initialised, count 1).  Returns false, in every thread,
// when a wait of any thread ran out of time (the products in flight were
// then given a second bounded wait).
template <int NT>
__device__ __forceinline__ bool gramChunks(const float* __restrict__ Ws, const float* __restrict__ Wl,
                                           int wRows, int ldW, int R, int K,
                                           const float* imgRow, const int* expo,
                                           unsigned char* buf, unsigned long long* bars,
                                           uint32_t tmem, unsigned long long deadline) {
  const int tid = threadIdx.x;
  const int nChunk = (K + KC - 1) / KC;
  bool ok = true;
  float* stage = (float*)(buf + 2 * OPBUF);
  auto fetch = [&](int ch) {
    float* st = stage + (ch & 1) * STAGE_F;
    float* stl = st + 2 * STAGE_F;
    for(int u = tid; u < RB * (KC / 4); u += NT) {
      const int r = u / (KC / 4), k = ch * KC + (u % (KC / 4)) * 4;
      if(r < wRows && k < ldW) {
        cpAsync16(smemU32(st + r * SKC + (k - ch * KC)), Ws + (size_t)r * ldW + k);
        cpAsync16(smemU32(stl + r * SKC + (k - ch * KC)), Wl + (size_t)r * ldW + k);
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
    if(ch >= 2 && !waitUntil(smemU32(&bars[b]), ((ch - 2) >> 1) & 1, deadline)) ok = false;
    __syncthreads();
    const float* stc = stage + (ch & 1) * STAGE_F;
    const float* stl = stc + 2 * STAGE_F;
    // 16-byte units: (row, 8 consecutive k) -> 5 slice units
    for(int u = tid; u < RB * (KC / 8); u += NT) {
      const int r = u % RB, kg = u / RB, k0 = ch * KC + kg * 8;  // rows fastest
      float xh[8], xl[8];
      if(r < wRows) {
        const float4* ph = (const float4*)(stc + r * SKC + kg * 8);
        const float4* pl = (const float4*)(stl + r * SKC + kg * 8);
        const float4 h0 = ph[0], h1 = ph[1], l0 = pl[0], l1 = pl[1];
        xh[0] = h0.x; xh[1] = h0.y; xh[2] = h0.z; xh[3] = h0.w;
        xh[4] = h1.x; xh[5] = h1.y; xh[6] = h1.z; xh[7] = h1.w;
        xl[0] = l0.x; xl[1] = l0.y; xl[2] = l0.z; xl[3] = l0.w;
        xl[4] = l1.x; xl[5] = l1.y; xl[6] = l1.z; xl[7] = l1.w;
      } else {
#pragma unroll
        for(int e = 0; e < 8; e++) {
          xh[e] = r < R ? imgRow[k0 + e] : 0.f;  // zero-padded past K
          xl[e] = 0.f;
        }
      }
#pragma unroll
      for(int e = 0; e < 8; e++)
        if(k0 + e >= K) xh[e] = xl[e] = 0.f;
      uint32_t q[NS][4];
      slice8(xh, xl, r < R ? expo[r] : 0, q);
      storeSlices(B, r, kg, q);
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if(tid == 0) issueChunk(tmem, B, ch == 0, smemU32(&bars[b]));
  }
  // the last commit covers every product issued before it
  const int last = nChunk - 1;
  if(!waitUntil(smemU32(&bars[last & 1]), (last >> 1) & 1, deadline)) {
    ok = false;
    // give products still in flight a second bounded chance before TMEM is freed
    waitUntil(smemU32(&bars[last & 1]), (last >> 1) & 1, timerNs() + WAIT_NS);
  }
  const int failed = __syncthreads_or(ok ? 0 : 1);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  return failed == 0;
}

// TMEM -> four int64 sum arrays in shared memory (sums: EPI_BYTES, 8-byte
// aligned), then G_ab for a, b < R into G (R x R, both triangles).  All
// threads of the CTA call it (nWarps a multiple of 4), after the last
// commit's wait; it frees the TMEM (warp 0).
//
// For row a and column b the thread holding TMEM lane (t, a) adds to
//   X[a][b]: the pairs (t, u) it holds directly,
//   Y[a][b]: the pairs (u, t) whose value P_ut[b][a] = P_tu[a][b] it holds
//            (u >= 2 for t in {0,1}; u = 4 for t in {2,3}),
// each split into an A half (t + u <= 3, weight 2^(7(3-m))) and a B half
// (m >= 4, weight 2^(7(7-m))); then G_ab = (A 2^28 + B) 2^(e_a + e_b - 63)
// with A = XA[a][b] + YA[b][a], B = XB[a][b] + YB[b][a].  |A|, |B| < 2^48,
// so both convert to FP64 exactly and the sum rounds once.
__device__ __forceinline__ void epilogue(uint32_t tmem, long long* sums, const int* expo, int R,
                                         double* G) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nWarps = blockDim.x >> 5;
  long long* XA = sums;
  long long* XB = XA + RB * ELD;
  long long* YA = XB + RB * ELD;
  long long* YB = YA + RB * ELD;
  const int q = warp & 3, part = warp >> 2, nParts = nWarps >> 2;
  const int a = 32 * (q & 1) + lane;
  const int t1 = q >> 1, t2 = 2 + (q >> 1);
  const uint32_t lanes = (uint32_t)(32 * q) << 16;
  for(int phase = 0; phase < 2; phase++) {
    if(t1 == phase) {
      for(int b0 = 8 * part; b0 < RB; b0 += 8 * nParts) {
        float p1[5][8], p2[3][8];
#pragma unroll
        for(int u = 0; u < 4; u++) ld8(tmem + lanes + 64 * u + b0, p1[u]);
        ld8(tmem + lanes + 256 + b0, p1[4]);
#pragma unroll
        for(int j = 0; j < 3; j++) ld8(tmem + lanes + 320 + 64 * j + b0, p2[j]);
        ldWait();
#pragma unroll
        for(int i = 0; i < 8; i++) {
          long long xa = 0, xb = 0, ya = 0, yb = 0;
#pragma unroll
          for(int u = 0; u < 5; u++) {
            const int m = t1 + u;
            const long long p = (long long)__float2int_rn(p1[u][i]);  // |p| < 2^24: exact
            const long long v = p * (1ll << (m <= 3 ? 7 * (3 - m) : 7 * (7 - m)));
            if(m <= 3) xa += v; else xb += v;
            if(u >= 2) {
              if(m <= 3) ya += v; else yb += v;
            }
          }
#pragma unroll
          for(int j = 0; j < 3; j++) {
            const int m = t2 + 2 + j;  // >= 4
            const long long v = (long long)__float2int_rn(p2[j][i]) * (1ll << (7 * (7 - m)));
            xb += v;
            if(j == 2) yb += v;
          }
          const int idx = a * ELD + b0 + i;
          if(phase == 0) {
            XA[idx] = xa;
            XB[idx] = xb;
            YA[idx] = ya;
            YB[idx] = yb;
          } else {
            XA[idx] += xa;
            XB[idx] += xb;
            YA[idx] += ya;
            YB[idx] += yb;
          }
        }
      }
    }
    __syncthreads();
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if(warp == 0) tmemFree512(tmem);
  for(int e = tid; e < R * (R + 1) / 2; e += blockDim.x) {
    int ra = (int)((sqrtf(8.f * e + 1.f) - 1.f) * 0.5f);
    while((ra + 1) * (ra + 2) / 2 <= e) ra++;
    while(ra * (ra + 1) / 2 > e) ra--;
    const int rb = e - ra * (ra + 1) / 2;
    const long long A = XA[ra * ELD + rb] + YA[rb * ELD + ra];
    const long long B = XB[ra * ELD + rb] + YB[rb * ELD + ra];
    const double v = (double)A * 0x1p28 + (double)B;
    const int ex = expo[ra] + expo[rb] - 63;
    const double g = v * __longlong_as_double((long long)(1023 + ex) << 52);
    G[ra * R + rb] = g;
    G[rb * R + ra] = g;
  }
}

// The K-chunk loop of one stamp without shared-memory staging (for kernels
// that must leave room for a second CTA on the SM): each thread loads its
// 8-element units (row r < R, 8 consecutive k) of the chunk straight from
// global memory (the CTA's own W, just written, so L2) into registers, waits
// until the chunk's operand buffer is free, slices into it, and one thread
// issues the products.  Rows R..63 of both operand buffers are zeroed once.
// Same digits, same products as gramChunks.  Returns false, in every thread,
// when a wait of any thread ran out of time.
//
// stallBar (test option, else null): an initialised mbarrier on which nothing
// ever arrives.  Before the first wait for a commit, every thread waits on it
// with a TEST_STALL_NS bound, which runs out: the CTA records a timeout and
// then waits for the real commit with its full bound, as after a real
// timeout, so the error path runs without a fault and with correct results.
constexpr unsigned long long TEST_STALL_NS = 1000000ull;
template <int NT>
__device__ __forceinline__ bool gramChunksDirect(const float* __restrict__ Ws,
                                                 const float* __restrict__ Wl, int wRows, int ldW,
                                                 int R, int K, const float* imgRow, const int* expo,
                                                 unsigned char* buf, unsigned long long* bars,
                                                 uint32_t tmem, unsigned long long deadline,
                                                 const unsigned long long* stallBar = nullptr) {
  static_assert(2 * NT >= RB * (KC / 8), "two units per thread cover a chunk");
  const int tid = threadIdx.x;
  const int nChunk = (K + KC - 1) / KC, nUnits = R * (KC / 8);
  bool ok = true;
  // rows R..RB-1 stay zero in both buffers
  for(int u = tid; u < 2 * (RB - R) * (KC / 8); u += NT) {
    const int bsel = u / ((RB - R) * (KC / 8)), v = u % ((RB - R) * (KC / 8));
    const uint32_t zero[NS][4] = {};
    storeSlices(buf + bsel * OPBUF, R + v / (KC / 8), v % (KC / 8), zero);
  }
  for(int ch = 0; ch < nChunk; ch++) {
    const int b = ch & 1;
    unsigned char* B = buf + b * OPBUF;
    float xh[2][8], xl[2][8];
#pragma unroll
    for(int i = 0; i < 2; i++) {
      const int u = tid + i * NT;
      const int r = u / (KC / 8), kg = u % (KC / 8), k0 = ch * KC + kg * 8;
#pragma unroll
      for(int e = 0; e < 8; e++) xh[i][e] = xl[i][e] = 0.f;
      if(u < nUnits) {
        if(r < wRows) {
          if(k0 < ldW) {  // ldW is a multiple of 8: a unit is wholly inside or past it
            const float4* ph = (const float4*)(Ws + (size_t)r * ldW + k0);
            const float4* pl = (const float4*)(Wl + (size_t)r * ldW + k0);
            const float4 h0 = ph[0], h1 = ph[1], l0 = pl[0], l1 = pl[1];
            xh[i][0] = h0.x; xh[i][1] = h0.y; xh[i][2] = h0.z; xh[i][3] = h0.w;
            xh[i][4] = h1.x; xh[i][5] = h1.y; xh[i][6] = h1.z; xh[i][7] = h1.w;
            xl[i][0] = l0.x; xl[i][1] = l0.y; xl[i][2] = l0.z; xl[i][3] = l0.w;
            xl[i][4] = l1.x; xl[i][5] = l1.y; xl[i][6] = l1.z; xl[i][7] = l1.w;
          }
        } else {
#pragma unroll
          for(int e = 0; e < 8; e++) xh[i][e] = imgRow[k0 + e];  // zero-padded past K
        }
#pragma unroll
        for(int e = 0; e < 8; e++)
          if(k0 + e >= K) xh[i][e] = xl[i][e] = 0.f;
      }
    }
    if(ch == 2 && stallBar && !waitUntil(smemU32(stallBar), 0, timerNs() + TEST_STALL_NS)) ok = false;
    if(ch >= 2 && !waitUntil(smemU32(&bars[b]), ((ch - 2) >> 1) & 1, deadline)) ok = false;
#pragma unroll
    for(int i = 0; i < 2; i++) {
      const int u = tid + i * NT;
      if(u < nUnits) {
        const int r = u / (KC / 8), kg = u % (KC / 8);
        uint32_t q[NS][4];
        slice8(xh[i], xl[i], expo[r], q);
        storeSlices(B, r, kg, q);
      }
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if(tid == 0) issueChunk(tmem, B, ch == 0, smemU32(&bars[b]));
  }
  const int last = nChunk - 1;
  if(nChunk <= 2 && stallBar && !waitUntil(smemU32(stallBar), 0, timerNs() + TEST_STALL_NS)) ok = false;
  if(!waitUntil(smemU32(&bars[last & 1]), (last >> 1) & 1, deadline)) {
    ok = false;
    waitUntil(smemU32(&bars[last & 1]), (last >> 1) & 1, timerNs() + WAIT_NS);
  }
  const int failed = __syncthreads_or(ok ? 0 : 1);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  return failed == 0;
}

// The epilogue of gramChunksDirect in two int64 arrays (sums: EPI2_BYTES):
// the thread holding (t, a) adds, for each column b, its X parts to SA[a][b]
// / SB[a][b] and its Y parts to SA[b][a] / SB[b][a] with shared-memory
// atomics, so SA[a][b] = XA[a][b] + YA[b][a] = A_ab of epilogue() above and
// likewise SB; every entry of G then follows from its own (a, b), and the
// two triangles agree because A and B are symmetric exact integers.  TMEM
// columns come four at a time.  Frees the TMEM (warp 0).
constexpr int EPI2_BYTES = 2 * RB * ELD * 8;
__device__ __forceinline__ void epilogueAtomic(uint32_t tmem, long long* sums, const int* expo,
                                               int R, double* G) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nWarps = blockDim.x >> 5;
  unsigned long long* SA = (unsigned long long*)sums;
  unsigned long long* SB = SA + RB * ELD;
  for(int i = tid; i < 2 * RB * ELD; i += blockDim.x) SA[i] = 0ull;
  __syncthreads();
  const int q = warp & 3, part = warp >> 2, nParts = nWarps >> 2;
  const int a = 32 * (q & 1) + lane;
  const int t1 = q >> 1, t2 = 2 + (q >> 1);
  const uint32_t lanes = (uint32_t)(32 * q) << 16;
  for(int b0 = 4 * part; b0 < RB; b0 += 4 * nParts) {
    long long xa[4] = {0, 0, 0, 0}, xb[4] = {0, 0, 0, 0}, ya[4] = {0, 0, 0, 0},
              yb[4] = {0, 0, 0, 0};
    {
      float p1[5][4];
#pragma unroll
      for(int u = 0; u < 4; u++) ld4(tmem + lanes + 64 * u + b0, p1[u]);
      ld4(tmem + lanes + 256 + b0, p1[4]);
      ldWait();
#pragma unroll
      for(int i = 0; i < 4; i++)
#pragma unroll
        for(int u = 0; u < 5; u++) {
          const int m = t1 + u;
          const long long p = (long long)__float2int_rn(p1[u][i]);  // |p| < 2^24: exact
          const long long v = p * (1ll << (m <= 3 ? 7 * (3 - m) : 7 * (7 - m)));
          if(m <= 3) xa[i] += v; else xb[i] += v;
          if(u >= 2) {
            if(m <= 3) ya[i] += v; else yb[i] += v;
          }
        }
    }
    {
      float p2[3][4];
#pragma unroll
      for(int j = 0; j < 3; j++) ld4(tmem + lanes + 320 + 64 * j + b0, p2[j]);
      ldWait();
#pragma unroll
      for(int i = 0; i < 4; i++)
#pragma unroll
        for(int j = 0; j < 3; j++) {
          const int m = t2 + 2 + j;  // >= 4
          const long long v = (long long)__float2int_rn(p2[j][i]) * (1ll << (7 * (7 - m)));
          xb[i] += v;
          if(j == 2) yb[i] += v;
        }
    }
#pragma unroll
    for(int i = 0; i < 4; i++) {
      const int bcol = b0 + i;
      atomicAdd(&SA[a * ELD + bcol], (unsigned long long)xa[i]);
      atomicAdd(&SB[a * ELD + bcol], (unsigned long long)xb[i]);
      atomicAdd(&SA[bcol * ELD + a], (unsigned long long)ya[i]);
      atomicAdd(&SB[bcol * ELD + a], (unsigned long long)yb[i]);
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if(warp == 0) tmemFree512(tmem);
  for(int e = tid; e < R * R; e += blockDim.x) {
    const int ra = e / R, rb = e % R;
    const long long A = (long long)SA[ra * ELD + rb];
    const long long B = (long long)SB[ra * ELD + rb];
    const double v = (double)A * 0x1p28 + (double)B;
    const int ex = expo[ra] + expo[rb] - 63;
    G[e] = v * __longlong_as_double((long long)(1023 + ex) << 52);
  }
}

}  // namespace tc
}  // namespace xb
