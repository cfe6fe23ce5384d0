// xb_fill_gram.cu — the mixed path's substamp fill and its exact tensor-core
// Gram matrix in one kernel, one CTA per stamp.
//
// For the common shapes it replaces three launches (k_fill_w_f32 ->
// k_fill_finish_f32 -> k_gram_tc) that passed W through HBM: the separate
// fill wrote W (hi and lo, 412 KB per stamp at 49 basis functions) and the
// Gram read it back after every other stamp's fill had pushed it out of L2.
// Here one CTA runs, for its stamp,
//   1. the 51 x 51 window (substamp + kernel half-width on each side) from
//      the image into shared memory with one TMA tile copy
//      (cp.async.bulk.tensor.2d, completion on an mbarrier) when the window
//      lies inside the frame and the frame's rows are 16-byte multiples, else
//      with clamped loads (the reference clamps at the edge);
//   2. the Y pass of every unique Y filter (convStampY, cl_kern/cmv.cl:70-106)
//      into shared memory, eight output rows per thread from one window
//      column;
//   3. the X pass of every basis function (convStampX, :108-135), eight
//      output pixels per thread from one row, the even/even subtraction
//      (convStampOdd, :137-154) against W[0] kept in shared memory, the
//      background rows (convStampBg, :156-193) and the image row of createB
//      (:218-248); W goes to global memory (hi for the chi^2 of k_sigs_f32, lo
//      as scratch for step 4) while each row's largest |hi| is collected.
//      Steps 2-3 run in passes of at most FG_GP Y filters (the pass holding
//      basis function 0 first; the default basis has 21 distinct Y filters,
//      so 3 passes), so that the Y outputs of one pass fit beside everything
//      else in ~85 KB;
//   4. the exact sliced Gram of xb_tc.cuh: each thread loads its units of the
//      CTA's own W back from L2 chunk by chunk, slices them with the row
//      exponents into BF16 digits, one thread multiplies them by tcgen05.mma
//      into TMEM, and the int64 epilogue (shared-memory atomics) writes G.
// At ~96 KB of shared memory two CTAs share an SM: one's Y/X passes (FP32
// pipe) overlap the other's Gram (tensor pipe, L2, barriers), and other
// kernels of concurrent frames fit beside them.  The arithmetic of steps 2-3
// is that of the separate kernels (xb_df.cuh, same operations in the same
// order) and step 4 forms the same digits and exact sums, so G and W are
// theirs bit for bit (tests/test_gpu_fill_gram.py).
//
// Limits (else the separate kernels run): FP32 images, kernel half-width 10
// (FK = 21 taps), substamps up to 31 x 31, R = basis + background + 1 <= 64
// rows, at most FG_MAXG distinct Y filters, background order <= 2 (its
// values are then exact products of two floats), no weighted fit.
#include <cuda.h>

#include <algorithm>

#include "xb_df.cuh"
#include "xb_internal.h"
#include "xb_tc.cuh"

namespace xb {

namespace {

constexpr int FG_HK = 10;   // the kernel half-width the fused kernel is built for
constexpr int FG_R8 = 8;    // outputs per thread item (rows of the Y pass, pixels of the X pass)
constexpr int FG_GP = 7;    // Y filters per pass
constexpr int FG_MAXPASS = 4;
constexpr int FG_MAXG = FG_MAXPASS * FG_GP;

// Shared-memory layout of the fill (steps 1-3); the Gram (step 4) and the
// epilogue reuse the same area from offset 0.
struct FgLayout {
  int tw, fSS, ldWin, winRows, ldY;
  size_t oWin, oF, oW0, oY, fill, total;
};
__host__ __device__ inline FgLayout fgLayout(int hSS, int hK, int nGroups, int nPSF) {
  FgLayout L;
  L.fSS = 2 * hSS + 1;
  L.tw = L.fSS + 2 * hK;
  L.ldWin = (L.tw + 3 + 3) / 4 * 4;   // TMA box width: 16-byte rows, room for the x offset
  L.winRows = L.tw + FG_R8;           // rows past tw are read only by discarded outputs
  L.ldY = L.tw + FG_R8;               // odd stride: the X items' rows fall on distinct banks
  if(L.ldY % 2 == 0) L.ldY++;
  const int fK = 2 * hK + 1, gp = nGroups < FG_GP ? nGroups : FG_GP;
  auto al = [](size_t v) { return (v + 127) / 128 * 128; };
  L.oWin = 0;
  L.oF = al(L.oWin + (size_t)L.ldWin * L.winRows * 4);
  L.oW0 = al(L.oF + (size_t)2 * (nPSF + nGroups) * fK * 4);
  L.oY = al(L.oW0 + (size_t)2 * L.fSS * L.fSS * 4);
  L.fill = al(L.oY + (size_t)gp * L.fSS * L.ldY * 4);
  size_t m = L.fill;
  if((size_t)2 * tc::OPBUF > m) m = 2 * tc::OPBUF;
  if((size_t)tc::EPI2_BYTES > m) m = tc::EPI2_BYTES;
  L.total = m + 1024;  // 1024-byte alignment of the operand buffers
  return L;
}

struct FillGramArgs {
  const float* conv;   // the image whose substamps are convolved
  const float* other;  // the image of createB's target row
  int w, h;
  const int* list;
  const int* liveN;
  const int* count;
  const int* cur;
  const int2* ssxy;
  int maxSS;
  const float* fSplit;  // the filters as float pairs (xb_ctx::dFSplit)
  const int* kx;
  const int* ky;
  int nPSF, nGroups;
  const int2* bgXY;
  int nBG;
  int hSS, wRows, ldW;
  int useTma;
  int testStall;  // option test_wait_timeout: one bounded wait per CTA runs out (gramChunksDirect)
  // pass plan: pass p holds the Y filters gOrder[gBeg[p] .. gBeg[p+1]) in
  // ytmp slots 0.. (slot[g]) and the X rows rows[rBeg[p] .. rBeg[p+1])
  // (basis function 0 apart: its filter g0 = gOrder[0] runs first alone)
  int nPass;
  int gBeg[FG_MAXPASS + 1], rBeg[FG_MAXPASS + 1];
  unsigned char gOrder[FG_MAXG];
  unsigned char slot[FG_MAXG];
  unsigned char rows[MAX_NPSF];
  unsigned char groupOf[MAX_NPSF];
  float* W;    // [stamp][wRows][ldW] hi
  float* Wlo;  // [stamp][wRows][ldW] lo
  double* G;   // [list entry][R][R]
  int* timeout;
};

// Y pass, 8 consecutive output rows of one window column: v[j] is the
// reference's float accumulation over taps t = 0..FK-1 (window row j + t,
// filter entry FK-1-t), in that order.  The tap loop is not unrolled (eight
// independent chains per tap keep the FP32 pipe busy; small code keeps the
// instruction cache warm); ld is the window's row stride.
template <int FK>
__device__ __forceinline__ void yPass8(const float* wp, int ld, const float* fh, const float* fl,
                                       float (&v)[FG_R8]) {
#pragma unroll
  for(int j = 0; j < FG_R8; j++) v[j] = 0.f;
#pragma unroll 1
  for(int t = 0; t < FK; t++) {
    const float h = fh[FK - 1 - t], l = fl[FK - 1 - t];
    const float* p = wp + t * ld;
#pragma unroll
    for(int j = 0; j < FG_R8; j++) v[j] = df::refStepY(v[j], p[j * ld], h, l);
  }
}
// X pass, 8 consecutive output pixels of one row: the double-float sum over
// taps t = 0..FK-1 (Y-pass value j + t, filter entry FK-1-t), in that order.
template <int FK>
__device__ __forceinline__ void xPass8(const float* yp, const float* fh, const float* fl,
                                       float (&hi)[FG_R8], float (&lo)[FG_R8]) {
  float sh[FG_R8], sl[FG_R8];
#pragma unroll
  for(int j = 0; j < FG_R8; j++) sh[j] = sl[j] = 0.f;
#pragma unroll 1
  for(int t = 0; t < FK; t++) {
    const float h = fh[FK - 1 - t], l = fl[FK - 1 - t];
#pragma unroll
    for(int j = 0; j < FG_R8; j++) df::dfAccum(sh[j], sl[j], yp[t + j], h, l);
  }
#pragma unroll
  for(int j = 0; j < FG_R8; j++) df::dfNorm(sh[j], sl[j], hi[j], lo[j]);
}

__device__ __forceinline__ void maxBits(unsigned* slot, float m) {
  atomicMax(slot, __float_as_uint(m));  // m >= 0: the bit patterns are ordered
}

template <int NT>
__global__ void __launch_bounds__(NT, 2)
    k_fill_gram(const __grid_constant__ CUtensorMap tmap, const __grid_constant__ FillGramArgs a) {
  using namespace tc;
  constexpr int HK = FG_HK, FK = 2 * HK + 1;
  extern __shared__ __align__(1024) unsigned char fg_s[];
  __shared__ float imgRow[1024];  // K <= 961 pixels, padded to whole chunks
  __shared__ int expo[RB];
  __shared__ unsigned rowMax[RB];
  __shared__ unsigned char evenRow[MAX_NPSF];
  __shared__ unsigned long long bars[4];  // two operand buffers, the window copy, the test stall
  __shared__ uint32_t tmemBase;
  if(a.liveN && (int)blockIdx.x >= *a.liveN) return;  // before any barrier or TMEM allocation
  const int t = blockIdx.x, s = a.list[t], tid = threadIdx.x, warp = tid >> 5;
  const int fSS = 2 * a.hSS + 1, K = fSS * fSS, R = a.wRows + 1, nPSF = a.nPSF;
  const int ldW = a.ldW;
  float* Ws = a.W + (size_t)s * a.wRows * ldW;
  float* Wl = a.Wlo + (size_t)s * a.wRows * ldW;
  double* Gs = a.G + (size_t)t * R * R;
  if(!(a.cur[s] < a.count[s])) {
    // no substamp left: W and G are zero (what the separate kernels give)
    for(int i = tid; i < a.wRows * ldW; i += NT) {
      Ws[i] = 0.f;
      Wl[i] = 0.f;
    }
    for(int i = tid; i < R * R; i += NT) Gs[i] = 0.0;
    return;
  }
  const unsigned long long deadline = timerNs() + WAIT_NS;
  unsigned char* buf = (unsigned char*)(((uintptr_t)fg_s + 1023) & ~(uintptr_t)1023);
  const FgLayout L = fgLayout(a.hSS, HK, a.nGroups, nPSF);
  const int tw = L.tw, ldWin = L.ldWin, ldY = L.ldY;
  float* win = (float*)(buf + L.oWin);
  float* fxh = (float*)(buf + L.oF);
  float* fxl = fxh + nPSF * FK;
  float* fyh = fxl + nPSF * FK;
  float* fyl = fyh + a.nGroups * FK;
  float* w0h = (float*)(buf + L.oW0);
  float* w0l = w0h + K;
  float* ytmp = (float*)(buf + L.oY);

  const int2 c = a.ssxy[(size_t)s * a.maxSS + a.cur[s]];
  const int xHalf = a.hSS + HK, wx0 = c.x - xHalf, wy0 = c.y - xHalf;
  const bool tma = a.useTma && wx0 >= 0 && wy0 >= 0 && wx0 + tw <= a.w && wy0 + tw <= a.h;
  const int x0 = wx0 & ~3;              // 16-byte aligned start of the TMA box
  const int dx = tma ? wx0 - x0 : 0;    // window column 0 in the staged rows
  const uint32_t winBar = smemU32(&bars[2]);
  if(tid == 0) {
    barInit(smemU32(&bars[0]), 1);
    barInit(smemU32(&bars[1]), 1);
    barInit(winBar, 1);
    barInit(smemU32(&bars[3]), 1);  // nothing arrives here (test option testStall)
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    if(tma) {
      const uint32_t bytes = (uint32_t)(ldWin * tw * 4);
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(winBar), "r"(bytes)
                   : "memory");
      asm volatile(
          "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
          " [%0], [%1, {%2, %3}], [%4];" ::"r"(smemU32(win)),
          "l"(reinterpret_cast<uint64_t>(&tmap)), "r"(x0), "r"(wy0), "r"(winBar)
          : "memory");
    }
  }
  // the filters as float pairs: X [nPSF][FK] hi, lo; Y [group][FK] hi, lo
  for(int i = tid; i < 2 * (nPSF + a.nGroups) * FK; i += NT) fxh[i] = a.fSplit[i];
  for(int n = tid; n < nPSF; n += NT)
    evenRow[n] = (n > 0 && a.kx[n] % 2 == 0 && a.ky[n] % 2 == 0) ? 1 : 0;
  if(tid < RB) rowMax[tid] = 0u;
  if(!tma) {
    for(int i = tid; i < tw * tw; i += NT) {
      const int gx = min(max(wx0 + i % tw, 0), a.w - 1);
      const int gy = min(max(wy0 + i / tw, 0), a.h - 1);
      win[(i / tw) * ldWin + i % tw] = a.conv[(size_t)gx + (size_t)gy * a.w];
    }
  }
  __syncthreads();  // barrier inits and the tables before any wait or use
  bool ok = true;
  if(tma) {
    int late = 0;
    if(!waitUntil(winBar, 0, deadline)) {
      late = 1;
      waitUntil(winBar, 0, timerNs() + WAIT_NS);  // the copy in flight gets a second chance
    }
    ok = __syncthreads_or(late) == 0;
  }

  const int nRB = (fSS + FG_R8 - 1) / FG_R8;  // row blocks of the Y pass
  const int nXB = (fSS + FG_R8 - 1) / FG_R8;  // pixel blocks of the X pass
  const int yPer = nRB * tw, xPer = fSS * nXB;
  // Y item i of filter g: rows block i / tw, window column i % tw
  auto yItem = [&](int g, int i) {
    const int r0 = (i / tw) * FG_R8, col = i % tw;
    float v[FG_R8];
    yPass8<FK>(win + r0 * ldWin + col + dx, ldWin, fyh + g * FK, fyl + g * FK, v);
    float* yo = ytmp + ((size_t)a.slot[g] * fSS + r0) * ldY + col;
#pragma unroll
    for(int j = 0; j < FG_R8; j++)
      if(r0 + j < fSS) yo[j * ldY] = v[j];
  };
  // stores 8 outputs of row n starting at pixel p0 (nv of them valid) and
  // folds their largest |hi| into the row maximum
  auto putRow = [&](int n, int p0, int nv, const float (&hi)[FG_R8], const float (&lo)[FG_R8]) {
    float m = 0.f;
#pragma unroll
    for(int j = 0; j < FG_R8; j++)
      if(j < nv) {
        Ws[(size_t)n * ldW + p0 + j] = hi[j];
        Wl[(size_t)n * ldW + p0 + j] = lo[j];
        m = fmaxf(m, fabsf(hi[j]));  // NaN is skipped, as in the separate Gram
      }
    maxBits(&rowMax[n], m);
  };
  // X item i of row n: output row i / nXB, pixels from 8 (i % nXB)
  auto xItem = [&](int n, int i) {
    const int row = i / nXB, ii0 = (i % nXB) * FG_R8;
    const int nv = min(FG_R8, fSS - ii0), p0 = row * fSS + ii0;
    float hi[FG_R8], lo[FG_R8];
    xPass8<FK>(ytmp + ((size_t)a.slot[a.groupOf[n]] * fSS + row) * ldY + ii0, fxh + n * FK,
               fxl + n * FK, hi, lo);
    if(n == 0) {
#pragma unroll
      for(int j = 0; j < FG_R8; j++)
        if(j < nv) {
          w0h[p0 + j] = hi[j];
          w0l[p0 + j] = lo[j];
        }
    } else if(evenRow[n]) {
#pragma unroll
      for(int j = 0; j < FG_R8; j++)
        if(j < nv) df::dfSub(hi[j], lo[j], w0h[p0 + j], w0l[p0 + j], hi[j], lo[j]);
    }
    putRow(n, p0, nv, hi, lo);
  };
  // background row b and the image row: item i of xPer
  auto bgItem = [&](int b, int i) {
    // the reference's form: float-normalised coordinates, FP64 powers, each
    // an exact product of at most two floats at background order <= 2
    const int row = i / nXB, ii0 = (i % nXB) * FG_R8;
    const int nv = min(FG_R8, fSS - ii0), p0 = row * fSS + ii0;
    const int ex = a.bgXY[b].x, ey = a.bgXY[b].y;
    const float yf = df::floatNormF(c.y - a.hSS + row, a.h);
    float hi[FG_R8], lo[FG_R8];
#pragma unroll
    for(int j = 0; j < FG_R8; j++) {
      const float xf = df::floatNormF(c.x - a.hSS + ii0 + j, a.w);
      float u = 1.f, v = 1.f;  // the two float factors
      if(ex == 2) u = v = xf;
      else if(ey == 2) u = v = yf;
      else {
        if(ex == 1) u = xf;
        if(ey == 1) v = yf;
      }
      hi[j] = u * v;
      lo[j] = fmaf(u, v, -hi[j]);  // exact: u v = hi + lo
    }
    putRow(nPSF + b, p0, nv, hi, lo);
  };
  auto imgItem = [&](int i) {
    const int row = i / nXB, ii0 = (i % nXB) * FG_R8;
    const int nv = min(FG_R8, fSS - ii0), p0 = row * fSS + ii0;
    const int gy = min(max(c.y - a.hSS + row, 0), a.h - 1);
    float m = 0.f;
    for(int j = 0; j < nv; j++) {
      const int gx = min(max(c.x - a.hSS + ii0 + j, 0), a.w - 1);
      const float v = a.other[(size_t)gx + (size_t)gy * a.w];
      imgRow[p0 + j] = v;
      m = fmaxf(m, fabsf(v));
    }
    maxBits(&rowMax[a.wRows], m);
  };

  const int g0 = a.gOrder[0];
  // pass 0, list A: the Y pass of basis function 0's filter
  for(int it = tid; it < yPer; it += NT) yItem(g0, it);
  __syncthreads();
  // list B: W[0] (kept for the even/even rows), the Y pass of the pass's
  // other filters, the background and image rows, the W and image padding
  {
    const int nG = a.gBeg[1] - 1;
    const int n0 = xPer, n1 = n0 + nG * yPer, n2 = n1 + a.nBG * xPer, n3 = n2 + xPer;
    for(int it = tid; it < n3; it += NT) {
      if(it < n0) xItem(0, it);
      else if(it < n1) yItem(a.gOrder[1 + (it - n0) / yPer], (it - n0) % yPer);
      else if(it < n2) bgItem((it - n1) / xPer, (it - n1) % xPer);
      else imgItem(it - n2);
    }
    const int padW = ldW - K, nChunkK = (K + KC - 1) / KC * KC;
    for(int i = tid; i < a.wRows * padW; i += NT) {
      const size_t o = (size_t)(i / padW) * ldW + K + i % padW;
      Ws[o] = 0.f;
      Wl[o] = 0.f;
    }
    for(int k = K + tid; k < nChunkK; k += NT) imgRow[k] = 0.f;
  }
  __syncthreads();
  // list C: the pass's other X rows
  for(int it = tid; it < (a.rBeg[1] - a.rBeg[0]) * xPer; it += NT)
    xItem(a.rows[a.rBeg[0] + it / xPer], it % xPer);
  // later passes: their Y filters into the freed slots, then their X rows
  for(int p = 1; p < a.nPass; p++) {
    __syncthreads();
    for(int it = tid; it < (a.gBeg[p + 1] - a.gBeg[p]) * yPer; it += NT)
      yItem(a.gOrder[a.gBeg[p] + it / yPer], it % yPer);
    __syncthreads();
    for(int it = tid; it < (a.rBeg[p + 1] - a.rBeg[p]) * xPer; it += NT)
      xItem(a.rows[a.rBeg[p] + it / xPer], it % xPer);
  }
  // the CTA's W stores before its own reads of them (step 4)
  __syncthreads();
  if(tid < RB) expo[tid] = tid < R ? rowExponent(__uint_as_float(rowMax[tid])) : 0;
  if(warp == 0) tmemAlloc512(&tmemBase);
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmemBase;
  if(!gramChunksDirect<NT>(Ws, Wl, a.wRows, ldW, R, K, imgRow, expo, buf, bars, tmem, deadline,
                           a.testStall ? &bars[3] : nullptr))
    ok = false;
  epilogueAtomic(tmem, (long long*)buf, expo, R, Gs);
  if(tid == 0 && !ok) atomicOr(a.timeout, 1);
}

// cuTensorMapEncodeTiled through the runtime's driver entry point, so the
// library has no link-time dependence on the driver library.
using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                   const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                   const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                   CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiledFn encodeTiled() {
  static const EncodeTiledFn fn = [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
           cudaSuccess ||
       q != cudaDriverEntryPointSuccess)
      p = nullptr;
    return (EncodeTiledFn)p;
  }();
  return fn;
}

}  // namespace

bool fillGramFits(const xb_ctx* c) {
  const Geo& g = c->g;
  if(!c->fillGram || c->imgIsF64 || c->p.fitWeighted || c->gramFp64) return false;
  if(g.hK != FG_HK || g.fSS > 31 || g.wRows + 1 > tc::RB || g.nPSF > MAX_NPSF) return false;
  if(c->p.backgroundOrder > 2) return false;
  const int nGroups = (int)c->basis.yGroupStart.size() - 1;
  if(nGroups < 1 || nGroups > FG_MAXG) return false;
  int optin = 0;
  if(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->device) != cudaSuccess)
    return false;
  // the static arrays of the kernel take ~5 KB beside the dynamic area
  return fgLayout(g.hSS, g.hK, nGroups, g.nPSF).total + 8 * 1024 <= (size_t)optin;
}

void fillGramLaunch(xb_ctx* c, int si, const int* dList, int nList, int imgConv, double* G,
                    const int* liveN) {
  const Geo& g = c->g;
  const Basis& bs = c->basis;
  StampSetDev& S = c->set[si];
  const int nGroups = (int)bs.yGroupStart.size() - 1;
  const FgLayout L = fgLayout(g.hSS, g.hK, nGroups, g.nPSF);
  FillGramArgs a{};
  a.conv = (const float*)c->img[imgConv];
  a.other = (const float*)c->img[1 - imgConv];
  a.w = c->w;
  a.h = c->h;
  a.list = dList;
  a.liveN = liveN;
  a.count = S.count;
  a.cur = S.cur;
  a.ssxy = S.ssxy;
  a.maxSS = g.maxSS;
  a.fSplit = c->dFSplit;
  a.kx = c->dKx;
  a.ky = c->dKy;
  a.nPSF = g.nPSF;
  a.nGroups = nGroups;
  a.bgXY = buf<int2>(c, "bgXY", g.nBG);
  a.nBG = g.nBG;
  a.hSS = g.hSS;
  a.wRows = g.wRows;
  a.ldW = mixedLd(g);
  a.W = S.Wf;
  a.Wlo = S.Wlo;
  a.G = G;
  a.timeout = deviceStatus(c) + 1;  // the context's device-timeout word
  a.testStall = c->testWaitTimeout;
  // pass plan: basis function 0's filter first, then the others in order,
  // FG_GP filters per pass; each pass's X rows are its filters' members
  std::vector<int> order, groupOf(g.nPSF, 0);
  for(int gi = 0; gi < nGroups; gi++)
    for(int m = bs.yGroupStart[gi]; m < bs.yGroupStart[gi + 1]; m++) groupOf[bs.yGroupMembers[m]] = gi;
  order.push_back(groupOf[0]);
  for(int gi = 0; gi < nGroups; gi++)
    if(gi != groupOf[0]) order.push_back(gi);
  a.nPass = (nGroups + FG_GP - 1) / FG_GP;
  int nr = 0;
  for(int p = 0; p < a.nPass; p++) {
    a.gBeg[p] = p * FG_GP;
    a.rBeg[p] = nr;
    const int gEnd = std::min(nGroups, (p + 1) * FG_GP);
    for(int k = p * FG_GP; k < gEnd; k++) {
      const int gi = order[k];
      a.gOrder[k] = (unsigned char)gi;
      a.slot[gi] = (unsigned char)(k - p * FG_GP);
      for(int m = bs.yGroupStart[gi]; m < bs.yGroupStart[gi + 1]; m++)
        if(bs.yGroupMembers[m] != 0) a.rows[nr++] = (unsigned char)bs.yGroupMembers[m];
    }
  }
  a.gBeg[a.nPass] = nGroups;
  a.rBeg[a.nPass] = nr;
  for(int n = 0; n < g.nPSF; n++) a.groupOf[n] = (unsigned char)groupOf[n];
  // the window's tile copy: rows of the frame in 16-byte multiples, box
  // ldWin x tw floats (its x start is rounded down to 4 floats in the kernel)
  CUtensorMap tm;
  memset(&tm, 0, sizeof(tm));
  a.useTma = 0;
  const EncodeTiledFn enc = encodeTiled();
  if(enc && c->w % 4 == 0 && ((uintptr_t)a.conv & 15) == 0) {
    const cuuint64_t dims[2] = {(cuuint64_t)c->w, (cuuint64_t)c->h};
    const cuuint64_t strides[1] = {(cuuint64_t)c->w * 4};
    const cuuint32_t box[2] = {(cuuint32_t)L.ldWin, (cuuint32_t)L.tw};
    const cuuint32_t es[2] = {1, 1};
    if(enc(&tm, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, (void*)a.conv, dims, strides, box, es,
           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
           CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS)
      a.useTma = c->fillGramTma;
  }
  // threads per CTA: 384 (variant 0) or 256; both keep two CTAs per SM and
  // give the same W and G bit for bit (every output's arithmetic is per item)
  XB_CUDA(allowMaxDynamicSmem((const void*)k_fill_gram<384>, c->device));
  XB_CUDA(allowMaxDynamicSmem((const void*)k_fill_gram<256>, c->device));
  auto launch = [&](int v) {
    if(v == 1) k_fill_gram<256><<<nList, 256, L.total, c->stream>>>(tm, a);
    else k_fill_gram<384><<<nList, 384, L.total, c->stream>>>(tm, a);
    XB_LAUNCHED(c);
  };
  launch(tunedVariant(c, "fill_gram", (long long)g.fSS * 100000 + g.nPSF * 100 + g.nBG, 2, launch));
}

}  // namespace xb
