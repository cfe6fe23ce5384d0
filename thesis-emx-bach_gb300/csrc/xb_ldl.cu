// xb_ldl.cu — the global normal system of the mixed path: LDL^T factorisation
// on a thread-block cluster and a refined solve.
//
// The global matrix built by createMatrix (src/cdkscUtil.cpp:307-402) is a
// sum of Gram blocks weighted by outer products of the spatial terms, so it
// is symmetric positive semi-definite; the reference solves it with the
// Numerical-Recipes LU with implicit row scaling (src/bachUtil.cpp:319-411).
// The mixed path factors it as L D L^T instead (half the arithmetic, no
// pivot search); a non-positive or non-finite pivot raises a flag and the
// pivoted LU of xb_mixed.cu redoes the system, so singular systems end exactly
// as in the reference.
//
// Factorisation.  Columns are dealt cyclically over the CL CTAs of a cluster
// and live in shared memory.  Step j (1-based) is owned by CTA (j-1) % CL: it
// sends the finished column j (unscaled) and r_j = 1/d_j to every other CTA
// with one bulk shared-to-shared copy per receiver that completes on an
// mbarrier in the receiver; each CTA then applies a_ik -= a_ij * (a_kj * r_j)
// to its own columns k > j, rows i >= k.  The owner of column j+1 applies step j to that column first,
// factors it and sends it before touching its other columns, so the critical
// path per step is one shared-memory hop plus one column update.  Receive
// buffers form a ring of LDL_RING slots per CTA; a slot is refilled only
// after every receiver has released it (an "empty" mbarrier in the CTA that
// sends the step that reuses the slot).  Every wait is bounded by a global
// timer deadline; on expiry the kernel records a timeout and runs to the end
// without waiting, so the launch always terminates.
//
// Solve.  One cluster: the CTAs invert the 32x32 diagonal blocks of L, CTA 0
// runs the blocked triangular solves (a block = one small product with its
// inverse, then the rows below/above it), all CTAs compute the FP64 residual
// r = b - A x of the original matrix, and CTA 0 solves for the correction,
// which is added once.

#include <cooperative_groups.h>

#include <atomic>

#include "xb_internal.h"

namespace cg = cooperative_groups;

namespace xb {

namespace {

constexpr int LDL_THREADS = 256;
constexpr int LDL_RING = 8;  // receive slots per CTA
constexpr unsigned long long LDL_WAIT_NS = 2000000000ull;  // deadline per launch

// ------------------------------------------------------------ PTX helpers --
__device__ __forceinline__ uint32_t smemAddr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ uint32_t mapaRank(uint32_t a, int rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(rank));
  return r;
}
__device__ __forceinline__ void mbarInit(uint32_t bar, int count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbarArriveExpect(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void mbarArriveCluster(uint32_t clusterBar) {
  asm volatile("mbarrier.arrive.release.cluster.shared::cluster.b64 _, [%0];" ::"r"(clusterBar)
               : "memory");
}
__device__ __forceinline__ bool mbarTryWait(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bulk copy of `bytes` from this CTA's shared memory to another CTA's,
// completing `bytes` of transactions on that CTA's mbarrier.
__device__ __forceinline__ void bulkCopyCluster(uint32_t dstCluster, uint32_t srcCta,
                                                uint32_t bytes, uint32_t barCluster) {
  asm volatile(
      "cp.async.bulk.shared::cluster.shared::cta.mbarrier::complete_tx::bytes [%0], [%1], %2, "
      "[%3];" ::"r"(dstCluster),
      "r"(srcCta), "r"(bytes), "r"(barCluster)
      : "memory");
}
// Orders this thread's earlier shared-memory writes before later reads of the
// async proxy (the bulk copies).
__device__ __forceinline__ void fenceProxyAsync() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ unsigned long long globalTimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// 1/d to about one ulp: a single-precision reciprocal as the start value,
// then one third-order Newton-Raphson step, x1 = x0 (1 + e + e^2) with
// e = 1 - d x0 (the truncated series of 1/(1 - e)); |e| <= 2^-22 leaves a
// truncation error below 2^-66.  Outside the float range, plain division.
__device__ __forceinline__ double recipFast(double d) {
  const double ad = fabs(d);
  if(!(ad > 1e-30 && ad < 1e30)) return 1.0 / d;
  const double x0 = (double)__frcp_rn((float)d);
  const double e = fma(-d, x0, 1.0);
  return fma(x0, fma(e, e, e), x0);
}

// Bytes step j sends to one receiver: entries [i0-2, LC) of the column, i0
// the even row at or below j+1 (entry i0-2 carries r_j; LC is even, so the
// size is a multiple of 16 bytes and both ends are 16-byte aligned).
__device__ __forceinline__ uint32_t stepBytes(int j, int LC) {
  return 8u * (uint32_t)(LC - ((j + 1) & ~1) + 2);
}

// Bounded wait on a local mbarrier phase; false (and the timeout flags set)
// once the launch deadline has passed.
__device__ __forceinline__ bool waitPhase(uint32_t bar, uint32_t parity,
                                          unsigned long long deadline, volatile int* sErr,
                                          int* status) {
  if(*sErr) return false;
  while(!mbarTryWait(bar, parity)) {
    if(globalTimer() > deadline) {
      *sErr = 1;
      atomicOr(status + 1, 1);
      return false;
    }
  }
  return true;
}

}  // namespace

// status[0] bit 0: a pivot was not positive and finite (LU fallback);
// status[1] bit 0: a wait ran out of time.  F receives d_k on the diagonal and
// l_ik (i > k) in both triangles (F[k][i] and F[i][k]); rinv[k] = 1/d_k.
template <int CL>
__global__ void __launch_bounds__(LDL_THREADS)
    k_global_ldl(const double* __restrict__ M, double* __restrict__ F, double* __restrict__ rinv,
                 int n, int* __restrict__ status) {
  extern __shared__ __align__(16) double ldl_s[];
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank(), tid = threadIdx.x;
  const int lane = tid & 31, warp = tid >> 5;
  constexpr int NW = LDL_THREADS / 32;
  const int ld = n + 1;
  const int LC = (n + 3) & ~1;  // even, >= n + 2
  const int ncol = (n + CL - 1) / CL;
  double* col = ldl_s;                               // ncol x LC
  double* slot = col + (size_t)ncol * LC;            // LDL_RING x LC
  double* rvec = slot + (size_t)LDL_RING * LC;       // LC
  unsigned long long* bars = (unsigned long long*)(rvec + LC);
  // bars[0..LDL_RING) full (receive) barriers, bars[LDL_RING] the empty barrier
  __shared__ int sErr;
  const unsigned long long deadline = globalTimer() + LDL_WAIT_NS;

  for(int lc = 0; lc < ncol; lc++) {
    const int k = lc * CL + rank + 1;
    double* ck = col + (size_t)lc * LC;
    for(int i = tid; i < LC; i += LDL_THREADS)
      ck[i] = (k <= n && i <= n) ? M[(size_t)k * ld + i] : 0.0;  // row k = column k
  }
  for(int i = tid; i < LC; i += LDL_THREADS) rvec[i] = 0.0;
  if(tid == 0) {
    sErr = 0;
    for(int r = 0; r < LDL_RING; r++) mbarInit(smemAddr(&bars[r]), 1);
    mbarInit(smemAddr(&bars[LDL_RING]), CL - 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    // arm each slot for the first step this CTA receives through it
    for(int r = 0; r < LDL_RING; r++)
      for(int j = r + 1; j <= n - 1; j += LDL_RING)
        if((j - 1) % CL != rank) {
          mbarArriveExpect(smemAddr(&bars[r]), stepBytes(j, LC));
          break;
        }
  }
  __syncthreads();
  cluster.sync();

  uint32_t phaseBits = 0;  // receive-slot parities
  uint32_t emptyPhase = 0;
  volatile int* vErr = &sErr;

  // Pivot of the finished column jp (owned here): r = 1/d is stored in rvec
  // and at entry i0-2 of the column (a row above the diagonal, never used
  // again), where it travels with the column.  One thread.
  auto pivotStore = [&](int jp) {
    double* cp = col + (size_t)((jp - 1) / CL) * LC;
    const double d = cp[jp];
    double r = recipFast(d);
    if(!(d > 0.0) || !isfinite(r)) {
      atomicOr(status, 1);
      r = 0.0;
    }
    rvec[jp] = r;
    cp[((jp + 1) & ~1) - 2] = r;
  };
  // Copy column jp, entries [i0-2, LC), to the same place in every other
  // CTA's receive slot, completing on that CTA's full barrier.  Called by all
  // threads after the column's writes were fenced for the async proxy and
  // the CTA synchronised; thread 0 waits for the slot and issues the copies.
  auto sendColumn = [&](int jp) {
    if(tid == 0) {
      if(jp > LDL_RING) waitPhase(smemAddr(&bars[LDL_RING]), emptyPhase, deadline, vErr, status);
      const int rs = (jp - 1) % LDL_RING;
      const uint32_t off = (uint32_t)(((jp + 1) & ~1) - 2) * 8u;
      const uint32_t src = smemAddr(col + (size_t)((jp - 1) / CL) * LC) + off;
      const uint32_t dstSlot = smemAddr(slot + (size_t)rs * LC) + off;
      const uint32_t fullA = smemAddr(&bars[rs]);
      const uint32_t bytes = stepBytes(jp, LC);
      for(int q = 0; q < CL; q++)
        if(q != rank) bulkCopyCluster(mapaRank(dstSlot, q), src, bytes, mapaRank(fullA, q));
    }
    if(jp > LDL_RING) emptyPhase ^= 1u;
  };

  if(rank == 0) {
    if(tid == 0) pivotStore(1);
    fenceProxyAsync();
    __syncthreads();
    if(n > 1) sendColumn(1);
  }
  for(int j = 1; j < n; j++) {
    const int rs = (j - 1) % LDL_RING;
    const bool own = (j - 1) % CL == rank;
    const double* a;
    if(own) {
      a = col + (size_t)((j - 1) / CL) * LC;
    } else {
      a = slot + (size_t)rs * LC;
      waitPhase(smemAddr(&bars[rs]), (phaseBits >> rs) & 1u, deadline, vErr, status);
      phaseBits ^= 1u << rs;
    }
    const double r = own ? rvec[j] : a[((j + 1) & ~1) - 2];
    if(!own && tid == 0) rvec[j] = r;
    const int lcStart = (j - rank + CL - 1) / CL;  // first local column k > j
    const bool ahead = j % CL == rank;             // this CTA owns column j + 1
    if(ahead) {
      double* c1 = col + (size_t)lcStart * LC;
      const double cf = a[j + 1] * r;
      for(int i = j + 1 + tid; i <= n; i += LDL_THREADS) c1[i] = fma(-a[i], cf, c1[i]);
      if(tid == 0) pivotStore(j + 1);  // row j+1 was this thread's first
      fenceProxyAsync();
      __syncthreads();
      if(j + 1 < n) sendColumn(j + 1);
    }
    for(int lc = lcStart + (ahead ? 1 : 0) + warp; lc < ncol; lc += NW) {
      const int k = lc * CL + rank + 1;
      if(k > n) break;
      double* ck = col + (size_t)lc * LC;
      const double cf = a[k] * r;
      for(int i = k + lane; i <= n; i += 32) ck[i] = fma(-a[i], cf, ck[i]);
    }
    __syncthreads();
    if(!own && tid == 0) {
      for(int jn = j + LDL_RING; jn <= n - 1; jn += LDL_RING)
        if((jn - 1) % CL != rank) {
          mbarArriveExpect(smemAddr(&bars[rs]), stepBytes(jn, LC));
          break;
        }
      if(j + LDL_RING <= n - 1)
        mbarArriveCluster(mapaRank(smemAddr(&bars[LDL_RING]), (j + LDL_RING - 1) % CL));
    }
  }
  __syncthreads();
  for(int lc = 0; lc < ncol; lc++) {
    const int k = lc * CL + rank + 1;
    if(k > n) break;
    const double* ck = col + (size_t)lc * LC;
    const double rk = rvec[k];
    for(int i = k + tid; i <= n; i += LDL_THREADS) {
      const double v = i == k ? ck[k] : ck[i] * rk;
      F[(size_t)k * ld + i] = v;  // row k: l_ik, i > k
      F[(size_t)i * ld + k] = v;  // row i: l_ik, k < i
    }
    if(tid == 0) rinv[k] = rk;
  }
  cluster.sync();  // no CTA leaves while another may still address its shared memory
}

// Panel variant (same factors, bit for bit): panels of P columns, panel p
// owned by CTA p % CL, which applies every earlier panel to it, factors it
// locally (pivot, then the updates inside the panel, in column order) and
// copies the P columns to ring slot p % ring of every other CTA with one
// bulk copy per receiver.  Every column receives the same updates, in the same
// order, with the same FMAs as in the column kernel above; only the number
// of cluster-wide exchanges drops (n/P instead of n).  Receivers arm a slot
// before its copy can come and release it to the sender of panel p + ring
// (ring <= CL keeps the empty-barrier phases in order).  The protocol is
// modelled on the CPU in tests/test_ldl_panel_protocol.py.
template <int CL, int P>
__global__ void __launch_bounds__(LDL_THREADS)
    k_global_ldl_panel(const double* __restrict__ M, double* __restrict__ F,
                       double* __restrict__ rinv, int n, int ring, int* __restrict__ status) {
  extern __shared__ __align__(16) double ldl_s[];
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank(), tid = threadIdx.x;
  const int lane = tid & 31, warp = tid >> 5;
  constexpr int NW = LDL_THREADS / 32;
  const int ld = n + 1;
  const int LC = (n + 3) & ~1;
  const int nP = (n + P - 1) / P, lpn = (nP + CL - 1) / CL, lastSent = nP - 2;
  double* col = ldl_s;                                // lpn * P x LC (panel lp = p / CL)
  double* slot = col + (size_t)lpn * P * LC;          // ring x P x LC
  double* rvec = slot + (size_t)ring * P * LC;        // LC
  unsigned long long* bars = (unsigned long long*)(rvec + LC);  // ring full + 1 empty
  __shared__ int sErr;
  const unsigned long long deadline = globalTimer() + LDL_WAIT_NS;
  const uint32_t panelBytes = (uint32_t)P * (uint32_t)LC * 8u;
  auto ownerOf = [](int p) { return p % CL; };
  auto localCol = [&](int k) {  // column k (1-based) of a panel owned here
    const int p = (k - 1) / P;
    return col + (size_t)((p / CL) * P + (k - 1) % P) * LC;
  };

  for(int lp = 0; lp < lpn; lp++) {
    const int p = lp * CL + rank;
    for(int q = 0; q < P; q++) {
      const int k = 1 + p * P + q;
      double* ck = col + (size_t)(lp * P + q) * LC;
      for(int i = tid; i < LC; i += LDL_THREADS)
        ck[i] = (p < nP && k <= n && i <= n) ? M[(size_t)k * ld + i] : 0.0;
    }
  }
  for(int i = tid; i < LC; i += LDL_THREADS) rvec[i] = 0.0;
  if(tid == 0) {
    sErr = 0;
    for(int r = 0; r < ring; r++) mbarInit(smemAddr(&bars[r]), 1);
    mbarInit(smemAddr(&bars[ring]), CL - 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    for(int r = 0; r < ring; r++)
      for(int p = r; p <= lastSent; p += ring)
        if(ownerOf(p) != rank) {
          mbarArriveExpect(smemAddr(&bars[r]), panelBytes);
          break;
        }
  }
  __syncthreads();
  cluster.sync();

  uint32_t phaseBits = 0, emptyPhase = 0;
  volatile int* vErr = &sErr;

  // pivots and in-panel updates of panel p (owned, earlier panels applied)
  auto factorPanel = [&](int p) {
    const int first = 1 + p * P, last = min(n, first + P - 1);
    for(int j = first; j <= last; j++) {
      double* cj = localCol(j);
      if(tid == 0) {
        const double d = cj[j];
        double r = recipFast(d);
        if(!(d > 0.0) || !isfinite(r)) {
          atomicOr(status, 1);
          r = 0.0;
        }
        rvec[j] = r;
        cj[((j + 1) & ~1) - 2] = r;  // travels with the column, above its diagonal
      }
      __syncthreads();
      const double r = rvec[j];
      for(int k = j + 1 + warp; k <= last; k += NW) {
        double* ck = localCol(k);
        const double cf = cj[k] * r;
        for(int i = k + lane; i <= n; i += 32) ck[i] = fma(-cj[i], cf, ck[i]);
      }
      __syncthreads();
    }
  };
  // panel p (base: its P columns) applied to the local columns of the panels
  // [pFrom, pTo]: per entry, the panel's columns in order
  auto applyPanel = [&](const double* base, int p, int pFrom, int pTo) {
    const int first = 1 + p * P, w = min(P, n - first + 1);
    double rq[P];
#pragma unroll
    for(int q = 0; q < P; q++) rq[q] = q < w ? base[(size_t)q * LC + ((first + q + 1) & ~1) - 2] : 0.0;
    const int lp0 = (pFrom - rank + CL - 1) / CL;  // first local panel >= pFrom
    for(int e = warp; ; e += NW) {
      const int lp = lp0 + e / P, q = e % P, pk = lp * CL + rank, k = 1 + pk * P + q;
      if(pk > pTo || pk >= nP || k > n) break;
      double* ck = col + (size_t)(lp * P + q) * LC;
      double cf[P];
#pragma unroll
      for(int u = 0; u < P; u++) cf[u] = u < w ? base[(size_t)u * LC + k] * rq[u] : 0.0;
      for(int i = k + lane; i <= n; i += 32) {
        double v = ck[i];
#pragma unroll
        for(int u = 0; u < P; u++)
          if(u < w) v = fma(-base[(size_t)u * LC + i], cf[u], v);
        ck[i] = v;
      }
    }
  };
  auto sendPanel = [&](int p) {
    if(tid == 0) {
      if(p >= ring) waitPhase(smemAddr(&bars[ring]), emptyPhase, deadline, vErr, status);
      const int sl = p % ring;
      const uint32_t src = smemAddr(localCol(1 + p * P));
      const uint32_t dst = smemAddr(slot + (size_t)sl * P * LC);
      const uint32_t fullA = smemAddr(&bars[sl]);
      for(int q = 0; q < CL; q++)
        if(q != rank) bulkCopyCluster(mapaRank(dst, q), src, panelBytes, mapaRank(fullA, q));
    }
    if(p >= ring) emptyPhase ^= 1u;
  };

  if(ownerOf(0) == rank) {
    factorPanel(0);
    fenceProxyAsync();
    __syncthreads();
    if(0 <= lastSent) sendPanel(0);
  }
  for(int p = 0; p < nP - 1; p++) {
    const int sl = p % ring;
    const bool own = ownerOf(p) == rank;
    const double* base;
    if(own) {
      base = localCol(1 + p * P);
    } else {
      base = slot + (size_t)sl * P * LC;
      waitPhase(smemAddr(&bars[sl]), (phaseBits >> sl) & 1u, deadline, vErr, status);
      phaseBits ^= 1u << sl;
    }
    const bool ahead = ownerOf(p + 1) == rank;
    if(ahead) {  // look-ahead: the next panel first, factored and sent
      applyPanel(base, p, p + 1, p + 1);
      __syncthreads();
      factorPanel(p + 1);
      fenceProxyAsync();
      __syncthreads();
      if(p + 1 <= lastSent) sendPanel(p + 1);
    }
    applyPanel(base, p, ahead ? p + 2 : p + 1, nP - 1);
    __syncthreads();
    if(!own && tid == 0) {
      for(int pn = p + ring; pn <= lastSent; pn += ring)
        if(ownerOf(pn) != rank) {
          mbarArriveExpect(smemAddr(&bars[sl]), panelBytes);
          break;
        }
      if(p + ring <= lastSent) mbarArriveCluster(mapaRank(smemAddr(&bars[ring]), ownerOf(p + ring)));
    }
  }
  __syncthreads();
  for(int lp = 0; lp < lpn; lp++)
    for(int q = 0; q < P; q++) {
      const int k = 1 + (lp * CL + rank) * P + q;
      if(k > n) break;
      const double* ck = col + (size_t)(lp * P + q) * LC;
      const double rk = rvec[k];
      for(int i = k + tid; i <= n; i += LDL_THREADS) {
        const double v = i == k ? ck[k] : ck[i] * rk;
        F[(size_t)k * ld + i] = v;
        F[(size_t)i * ld + k] = v;
      }
      if(tid == 0) rinv[k] = rk;
    }
  cluster.sync();  // no CTA leaves while another may still address its shared memory
}

// ------------------------------------------------------------------ solve --
namespace {

constexpr int SV_THREADS = 512;
constexpr int SV_NB = 32;  // diagonal block size
constexpr int SV_AW = 4;   // warps of a 32x32 block product (8 terms each)

// Inverse of the unit lower-triangular diagonal block q of L (rows/cols
// [1 + 32q, 1 + 32q + 32), padded with the identity past n) into Linv
// (32 x 32, row-major), by recursive doubling: for a 2m block
// [[A, 0], [C, B]] the inverse's lower-left part is -B^-1 (C A^-1).
// CTA-wide; X is 32 x 33, T 256 doubles of shared memory.
__device__ void invertDiagBlock(const double* __restrict__ F, int n, int q, double* X, double* T,
                                double* __restrict__ Linv) {
  const int tid = threadIdx.x, ld = n + 1, s = 1 + q * SV_NB;
  constexpr int XL = SV_NB + 1;
  for(int e = tid; e < SV_NB * SV_NB; e += SV_THREADS) {
    const int t = e / SV_NB, u = e % SV_NB;
    double v = t == u ? 1.0 : 0.0;
    if(t > u && s + t <= n) v = F[(size_t)(s + t) * ld + s + u];  // L[t][u] (kept in X's lower part)
    X[t * XL + u] = v;
  }
  __syncthreads();
  // X's strictly lower part holds L until each level overwrites its blocks
  for(int m = 1; m < SV_NB; m *= 2) {
    const int nPair = SV_NB / (2 * m), cnt = nPair * m * m;
    // T = C A^-1 for every pair block
    for(int e = tid; e < cnt; e += SV_THREADS) {
      const int p = e / (m * m), a = (e / m) % m, b = e % m, o = p * 2 * m;
      double acc = 0.0;
      for(int c = b; c < m; c++)  // A^-1 is unit lower: entries c >= b
        acc = fma(X[(o + m + a) * XL + o + c], c == b ? 1.0 : X[(o + c) * XL + o + b], acc);
      T[e] = acc;
    }
    __syncthreads();
    // lower-left <- -B^-1 T
    for(int e = tid; e < cnt; e += SV_THREADS) {
      const int p = e / (m * m), a = (e / m) % m, b = e % m, o = p * 2 * m;
      double acc = T[e];  // the unit diagonal of B^-1
      for(int c = 0; c < a; c++) acc = fma(X[(o + m + a) * XL + o + m + c], T[p * m * m + c * m + b], acc);
      X[(o + m + a) * XL + o + b] = -acc;
    }
    __syncthreads();
  }
  for(int e = tid; e < SV_NB * SV_NB; e += SV_THREADS)
    Linv[(size_t)q * SV_NB * SV_NB + e] = X[(e / SV_NB) * XL + e % SV_NB];
  __syncthreads();
}

// x <- L^-T D^-1 L^-1 x on x[1..n] (shared), CTA-wide, with the inverses of
// the diagonal blocks in Li (shared, nB x 32 x 32).  Per block: the 32x32
// product with the inverse (warps 0-3, eight terms each), then the next
// block's rows (warps 0-3) and, at the same time, the rows beyond it
// (warps 4-15, one row per thread; each loads its row's 32 entries of L at
// once, since the chain is bound by L2 latency).  part: SV_AW x 32 doubles.
// sum_t F[s + t][i] x[s + t] over the nb (<= 32) rows of a block: four
// accumulators over t in steps of four, the remainder into the first; the 32
// loads are issued before the products.
__device__ __forceinline__ double rowDot(const double* __restrict__ F, int ld, int s, int nb,
                                         int i, const double* x) {
  double f[SV_NB];
#pragma unroll
  for(int t = 0; t < SV_NB; t++) f[t] = t < nb ? F[(size_t)(s + t) * ld + i] : 0.0;
  double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
#pragma unroll
  for(int t = 0; t < SV_NB; t += 4)
    if(t + 4 <= nb) {
      a0 = fma(f[t], x[s + t], a0);
      a1 = fma(f[t + 1], x[s + t + 1], a1);
      a2 = fma(f[t + 2], x[s + t + 2], a2);
      a3 = fma(f[t + 3], x[s + t + 3], a3);
    }
#pragma unroll
  for(int t = 0; t < SV_NB; t++)
    if(t >= (nb & ~3) && t < nb) a0 = fma(f[t], x[s + t], a0);
  return (a0 + a1) + (a2 + a3);
}

__device__ void ldlSolveCta(const double* __restrict__ F, const double* __restrict__ rinv, int n,
                            const double* Li, double* x, double* part) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, ld = n + 1;
  const int nB = (n + SV_NB - 1) / SV_NB;
  // ---- forward: L y = x
  for(int K = 0; K < nB; K++) {
    const int s = 1 + K * SV_NB, nb = min(SV_NB, n + 1 - s);
    const double* Lk = Li + (size_t)K * SV_NB * SV_NB;
    if(warp < SV_AW) {  // y_K = Linv_K x_K
      double acc = 0.0;
#pragma unroll
      for(int u = 0; u < SV_NB / SV_AW; u++) {
        const int t = warp * (SV_NB / SV_AW) + u;
        if(t < nb) acc = fma(Lk[lane * SV_NB + t], x[s + t], acc);
      }
      part[warp * 32 + lane] = acc;
    }
    __syncthreads();
    if(warp == 0 && lane < nb)
      x[s + lane] = (part[lane] + part[32 + lane]) + (part[64 + lane] + part[96 + lane]);
    __syncthreads();
    const int s2 = s + SV_NB, nb2 = min(SV_NB, n + 1 - s2);  // next block
    if(warp < SV_AW) {
      if(nb2 > 0) {
        double acc = 0.0;
#pragma unroll
        for(int u = 0; u < SV_NB / SV_AW; u++) {
          const int t = warp * (SV_NB / SV_AW) + u;
          if(t < nb && lane < nb2) acc = fma(F[(size_t)(s + t) * ld + s2 + lane], x[s + t], acc);
        }
        part[warp * 32 + lane] = acc;
      }
    } else {
      for(int i = s2 + SV_NB + (tid - SV_AW * 32); i <= n; i += SV_THREADS - SV_AW * 32)
        x[i] -= rowDot(F, ld, s, nb, i, x);
    }
    __syncthreads();
    if(warp == 0 && nb2 > 0 && lane < nb2)
      x[s2 + lane] -= (part[lane] + part[32 + lane]) + (part[64 + lane] + part[96 + lane]);
    __syncthreads();
  }
  for(int i = 1 + tid; i <= n; i += SV_THREADS) x[i] *= rinv[i];
  __syncthreads();
  // ---- backward: L^T x = z, blocks from the bottom; (Linv_K)^T on the block
  for(int K = nB - 1; K >= 0; K--) {
    const int s = 1 + K * SV_NB, nb = min(SV_NB, n + 1 - s);
    const double* Lk = Li + (size_t)K * SV_NB * SV_NB;
    if(warp < SV_AW) {
      double acc = 0.0;
#pragma unroll
      for(int u = 0; u < SV_NB / SV_AW; u++) {
        const int t = warp * (SV_NB / SV_AW) + u;
        if(t < nb) acc = fma(Lk[t * SV_NB + lane], x[s + t], acc);
      }
      part[warp * 32 + lane] = acc;
    }
    __syncthreads();
    if(warp == 0 && lane < nb)
      x[s + lane] = (part[lane] + part[32 + lane]) + (part[64 + lane] + part[96 + lane]);
    __syncthreads();
    const int s2 = s - SV_NB;  // previous block (full size)
    if(warp < SV_AW) {
      if(K > 0) {
        double acc = 0.0;
#pragma unroll
        for(int u = 0; u < SV_NB / SV_AW; u++) {
          const int t = warp * (SV_NB / SV_AW) + u;  // row s+t of L, column s2+lane
          if(t < nb) acc = fma(F[(size_t)(s + t) * ld + s2 + lane], x[s + t], acc);
        }
        part[warp * 32 + lane] = acc;
      }
    } else {
      for(int k = 1 + (tid - SV_AW * 32); k < s2; k += SV_THREADS - SV_AW * 32)
        x[k] -= rowDot(F, ld, s, nb, k, x);
    }
    __syncthreads();
    if(warp == 0 && K > 0)
      x[s2 + lane] -= (part[lane] + part[32 + lane]) + (part[64 + lane] + part[96 + lane]);
    __syncthreads();
  }
}

}  // namespace

// Inverses of the diagonal blocks of L, one CTA per block (Linv: global,
// ceil(n/32) x 32 x 32).  With status bit 0 set the pivoted LU solves the
// system instead and the kernel returns at once.
__global__ void __launch_bounds__(SV_THREADS)
    k_ldl_block_inv(const double* __restrict__ F, int n, const int* __restrict__ status,
                    double* __restrict__ Linv) {
  __shared__ double X[SV_NB * (SV_NB + 1)];
  __shared__ double T[256];
  if(status[0] & 1) return;
  invertDiagBlock(F, n, blockIdx.x, X, T, Linv);
}

// One triangular-solve pass of the refined solve, on one CTA (the pivot
// chain is sequential; no other SM waits on it).  first = 1: x1 = (L D L^T)^-1
// rhs into x1g.  first = 0: x2 = (L D L^T)^-1 res and rhs <- x1g + x2.
// With status bit 0 set the pivoted LU solves the system instead.
__global__ void __launch_bounds__(SV_THREADS)
    k_ldl_solve(const double* __restrict__ F, const double* __restrict__ rinv, int n,
                double* __restrict__ rhs, const double* __restrict__ res,
                double* __restrict__ x1g, const int* __restrict__ status,
                const double* __restrict__ Linv, int first) {
  extern __shared__ __align__(16) double sv_s[];
  const int tid = threadIdx.x;
  const int LX = (n + 2) & ~1, nB = (n + SV_NB - 1) / SV_NB;
  double* x = sv_s;                  // LX
  double* part = x + LX;             // SV_AW x 32
  double* Li = part + SV_AW * 32;    // nB x 32 x 32
  if(status[0] & 1) return;  // the LU fallback solves this system
  for(int e = tid; e < nB * SV_NB * SV_NB; e += SV_THREADS) Li[e] = Linv[e];
  const double* src = first ? rhs : res;
  for(int i = tid; i < LX; i += SV_THREADS) x[i] = i >= 1 && i <= n ? src[i] : 0.0;
  __syncthreads();
  ldlSolveCta(F, rinv, n, Li, x, part);
  if(first) {
    for(int i = tid; i < LX; i += SV_THREADS) x1g[i] = x[i];
  } else {
    for(int i = 1 + tid; i <= n; i += SV_THREADS) rhs[i] = x1g[i] + x[i];
  }
}

// Residual of the first pass, res_i = rhs_i - A_i . x1, one row per warp
// (lane-strided FMA chain, loads issued ahead, xor-shuffle sum) over
// ceil(n / 16) CTAs: FP64 runs at ~1.7 FMA per clock per SM on this part, so
// the n^2 products are spread over SMs.
__global__ void __launch_bounds__(SV_THREADS)
    k_ldl_residual(const double* __restrict__ A, int n, const double* __restrict__ rhs,
                   const double* __restrict__ x1g, const int* __restrict__ status,
                   double* __restrict__ res) {
  if(status[0] & 1) return;
  constexpr int NW = SV_THREADS / 32, RU = 8;
  const int lane = threadIdx.x & 31, ld = n + 1;
  const int i = 1 + blockIdx.x * NW + (threadIdx.x >> 5);
  if(i > n) return;
  double a = 0.0;
  for(int j0 = 1 + lane; j0 <= n; j0 += 32 * RU) {
    double av[RU], xv[RU];
#pragma unroll
    for(int u = 0; u < RU; u++) {
      const int j = j0 + 32 * u;
      av[u] = j <= n ? A[(size_t)i * ld + j] : 0.0;
      xv[u] = j <= n ? x1g[j] : 0.0;
    }
#pragma unroll
    for(int u = 0; u < RU; u++)
      if(j0 + 32 * u <= n) a = fma(av[u], xv[u], a);
  }
#pragma unroll
  for(int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
  if(lane == 0) res[i] = rhs[i] - a;
}

template __global__ void k_global_ldl<8>(const double*, double*, double*, int, int*);
template __global__ void k_global_ldl_panel<16, 2>(const double*, double*, double*, int, int, int*);
template __global__ void k_global_ldl_panel<16, 4>(const double*, double*, double*, int, int, int*);
template __global__ void k_global_ldl_panel<16, 8>(const double*, double*, double*, int, int, int*);
template __global__ void k_global_ldl_panel<8, 2>(const double*, double*, double*, int, int, int*);
template __global__ void k_global_ldl_panel<8, 4>(const double*, double*, double*, int, int, int*);
template __global__ void k_global_ldl_panel<8, 8>(const double*, double*, double*, int, int, int*);
template __global__ void k_global_ldl<16>(const double*, double*, double*, int, int*);

namespace {

size_t ldlSmemBytes(int n, int CL) {
  const int LC = (n + 3) & ~1, ncol = (n + CL - 1) / CL;
  return ((size_t)ncol * LC + (size_t)LDL_RING * LC + LC) * sizeof(double) +
         (LDL_RING + 1) * sizeof(unsigned long long);
}

// Shared memory of the panel kernel: the owned panels, the receive ring, the
// pivots and the barriers.
size_t ldlPanelSmemBytes(int n, int CL, int P, int ring) {
  const int LC = (n + 3) & ~1, nP = (n + P - 1) / P, lpn = (nP + CL - 1) / CL;
  return ((size_t)lpn * P * LC + (size_t)ring * P * LC + LC) * sizeof(double) +
         (size_t)(ring + 1) * sizeof(unsigned long long);
}

template <class Kern, class... Args>
cudaError_t launchCluster(xb_ctx* c, Kern kernel, int CL, int threads, size_t smem,
                          Args... args) {
  cudaError_t e =
      allowMaxDynamicSmem((const void*)kernel, c->device);
  if(e != cudaSuccess) return e;
  if(CL > 8) {
    e = cudaFuncSetAttribute(kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if(e != cudaSuccess) return e;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(CL);
  cfg.blockDim = dim3(threads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = c->stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = CL;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, args...);
}

}  // namespace

int* deviceStatus(xb_ctx* c) {
  const bool fresh = c->pool.find("ldl_status") == c->pool.end();
  int* status = buf<int>(c, "ldl_status", 2);
  if(fresh) {
    const int zero[2] = {0, 0};
    if(c->capturing) uploadNow(c, status, zero, sizeof(zero));
    else XB_CUDA(cudaMemsetAsync(status, 0, 2 * sizeof(int), c->stream));
  }
  return status;
}

void globalSolveMixed(xb_ctx* c, const double* M, int n, double* rhs, int* piv, int* singular) {
  const int ld = n + 1;
  int* status = deviceStatus(c);
  XB_CUDA(cudaMemsetAsync(status, 0, sizeof(int), c->stream));
  double* F = buf<double>(c, "ldl_F", (size_t)ld * ld);
  double* rinv = buf<double>(c, "ldl_rinv", ld);
  // 16-CTA clusters where the device allows them, else 8
  static std::atomic<int> clusterSize{0};
  {
    // Variants with the same factors bit for bit: the column kernel (0) and
    // panels of 2, 4 or 8 columns (1-3), where shared memory holds a receive
    // ring of at least two panels.  Wider panels need fewer cluster-wide
    // exchanges but put more FP64 work on the owner of the next panel (the
    // look-ahead), so the autotuner times them.
    int maxSmem = 0;
    XB_CUDA(cudaDeviceGetAttribute(&maxSmem, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->device));
    auto ringFor = [&](int CL, int P) {
      for(int rg = std::min(4, CL); rg >= 2; rg--)
        if(ldlPanelSmemBytes(n, CL, P, rg) <= (size_t)maxSmem) return rg;
      return 0;
    };
    auto launchVariant = [&](int v, int CL) -> cudaError_t {
      const int P = v == 1 ? 2 : v == 2 ? 4 : 8;
      const int rg = v > 0 ? ringFor(CL, P) : 0;
      if(v == 0 || rg == 0)
        return CL == 16 ? launchCluster(c, k_global_ldl<16>, 16, LDL_THREADS, ldlSmemBytes(n, 16),
                                        M, F, rinv, n, status)
                        : launchCluster(c, k_global_ldl<8>, 8, LDL_THREADS, ldlSmemBytes(n, 8), M,
                                        F, rinv, n, status);
      const size_t sm = ldlPanelSmemBytes(n, CL, P, rg);
      if(CL == 16)
        return P == 2 ? launchCluster(c, k_global_ldl_panel<16, 2>, 16, LDL_THREADS, sm, M, F, rinv,
                                      n, rg, status)
             : P == 4 ? launchCluster(c, k_global_ldl_panel<16, 4>, 16, LDL_THREADS, sm, M, F, rinv,
                                      n, rg, status)
                      : launchCluster(c, k_global_ldl_panel<16, 8>, 16, LDL_THREADS, sm, M, F, rinv,
                                      n, rg, status);
      return P == 2 ? launchCluster(c, k_global_ldl_panel<8, 2>, 8, LDL_THREADS, sm, M, F, rinv, n,
                                    rg, status)
           : P == 4 ? launchCluster(c, k_global_ldl_panel<8, 4>, 8, LDL_THREADS, sm, M, F, rinv, n,
                                    rg, status)
                    : launchCluster(c, k_global_ldl_panel<8, 8>, 8, LDL_THREADS, sm, M, F, rinv, n,
                                    rg, status);
    };
    // 16-CTA clusters where the device allows them and the context asks for
    // them, else 8
    auto launch = [&](int v) {
      cudaError_t e = cudaErrorUnknown;
      if(clusterSize.load() != 8 && c->ldlCluster == 16) {
        e = launchVariant(v, 16);
        if(e == cudaSuccess) clusterSize = 16;
        else cudaGetLastError();
      }
      if(e != cudaSuccess) {
        XB_CUDA(launchVariant(v, 8));
        if(c->ldlCluster == 16) clusterSize = 8;
      }
      XB_LAUNCHED(c);
    };
    const int v = c->ldlPanel ? tunedVariant(c, "global_ldl", (long long)n * 32 + c->ldlCluster, 4,
                                             launch)
                              : 0;
    KT_SCOPE(c, "global_ldl");
    launch(v);
  }
  luFallbackSolve(c, M, F, n, rhs, piv, singular, status);
  {
    KT_SCOPE(c, "global_solve");
    const int nB = (n + SV_NB - 1) / SV_NB;
    double* Linv = buf<double>(c, "ldl_linv", (size_t)nB * SV_NB * SV_NB);
    const size_t smem =
        ((size_t)((n + 2) & ~1) + SV_AW * 32 + (size_t)nB * SV_NB * SV_NB) * sizeof(double);
    double* x1g = buf<double>(c, "ldl_x1", (size_t)n + 2);
    double* res = buf<double>(c, "ldl_res", (size_t)n + 2);
    k_ldl_block_inv<<<nB, SV_THREADS, 0, c->stream>>>((const double*)F, n, (const int*)status, Linv);
    XB_LAUNCHED(c);
    XB_CUDA(allowMaxDynamicSmem((const void*)k_ldl_solve, c->device));
    k_ldl_solve<<<1, SV_THREADS, smem, c->stream>>>((const double*)F, (const double*)rinv, n, rhs,
                                                    res, x1g, (const int*)status, Linv, 1);
    XB_LAUNCHED(c);
    k_ldl_residual<<<(n + SV_THREADS / 32 - 1) / (SV_THREADS / 32), SV_THREADS, 0, c->stream>>>(
        (const double*)M, n, rhs, x1g, (const int*)status, res);
    XB_LAUNCHED(c);
    k_ldl_solve<<<1, SV_THREADS, smem, c->stream>>>((const double*)F, (const double*)rinv, n, rhs,
                                                    res, x1g, (const int*)status, Linv, 0);
    XB_LAUNCHED(c);
  }
}

void checkSolveTimeout(xb_ctx* c) {
  auto it = c->pool.find("ldl_status");
  if(it == c->pool.end()) return;
  int st[2] = {0, 0};
  XB_CUDA(cudaMemcpyAsync(st, it->second.p, sizeof(st), cudaMemcpyDeviceToHost, c->stream));
  XB_CUDA(cudaStreamSynchronize(c->stream));
  if(st[1]) {
    XB_CUDA(cudaMemsetAsync((int*)it->second.p + 1, 0, sizeof(int), c->stream));
    throw XbError{XB_ERR_DEVICE_TIMEOUT, "a bounded device-side wait ran out of time"};
  }
}

}  // namespace xb
