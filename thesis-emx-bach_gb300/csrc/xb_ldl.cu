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
// with st.async stores that complete on an mbarrier in the receiver; each CTA
// then applies a_ik -= a_ij * (a_kj * r_j) to its own columns k > j, rows
// i >= k.  The owner of column j+1 applies step j to that column first,
// factors it and sends it before touching its other columns, so the critical
// path per step is one shared-memory hop plus one column update.  Receive
// buffers form a ring of LDL_RING slots per CTA; a slot is refilled only
// after every receiver has released it (an "empty" mbarrier in the CTA that
// sends the step that reuses the slot).  Every wait is bounded by a global
// timer deadline; on expiry the kernel records a timeout and runs to the end
// without waiting, so the launch always terminates.
//
// Solve.  One cluster: CTA 0 runs the triangular solves (blocks of 32 rows, a
// warp per diagonal block, the other warps update the remaining rows), all
// CTAs compute the FP64 residual r = b - A x of the original matrix, and
// CTA 0 solves for the correction, which is added once.

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
__device__ __forceinline__ void stAsync2(uint32_t clusterAddr, double a, double b,
                                         uint32_t clusterBar) {
  asm volatile(
      "st.async.shared::cluster.mbarrier::complete_tx::bytes.v2.f64 [%0], {%1, %2}, [%3];" ::"r"(
          clusterAddr),
      "d"(a), "d"(b), "r"(clusterBar)
      : "memory");
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

// Bytes step j sends to one receiver: the pair (r_j, 0) at slot entry 0 and
// the column entries from the even row at or below j+1 up to n (pairs, so the
// last pair may carry row n+1, which is zero).
__device__ __forceinline__ uint32_t stepBytes(int j, int n) {
  const int i0 = (j + 1) & ~1;
  return 16u * (uint32_t)((n - i0) / 2 + 2);
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
// l_ik (i > k) in row k (F[k][i], the upper triangle); rinv[k] = 1/d_k.
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
  double* cbuf = rvec + LC;                          // ncol, padded to even
  unsigned long long* bars = (unsigned long long*)(cbuf + ((ncol + 1) & ~1));
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
          mbarArriveExpect(smemAddr(&bars[r]), stepBytes(j, n));
          break;
        }
  }
  __syncthreads();
  cluster.sync();

  uint32_t phaseBits = 0;  // receive-slot parities
  uint32_t emptyPhase = 0;
  volatile int* vErr = &sErr;

  // Send the finished column jp (owned here) to every other CTA.
  auto produce = [&](int jp) {
    const double* cp = col + (size_t)((jp - 1) / CL) * LC;
    const int rs = (jp - 1) % LDL_RING;
    if(jp > LDL_RING) {
      waitPhase(smemAddr(&bars[LDL_RING]), emptyPhase, deadline, vErr, status);
      emptyPhase ^= 1u;
    }
    const uint32_t slotA = smemAddr(slot + (size_t)rs * LC);
    const uint32_t fullA = smemAddr(&bars[rs]);
    if(warp == 0) {
      const double d = cp[jp];
      double r = recipFast(d);
      if(!(d > 0.0) || !isfinite(r)) {
        if(lane == 0) atomicOr(status, 1);
        r = 0.0;
      }
      if(lane < CL - 1) {
        const int dst = lane < rank ? lane : lane + 1;
        stAsync2(mapaRank(slotA, dst), r, 0.0, mapaRank(fullA, dst));
      }
      if(lane == 0) rvec[jp] = r;
    }
    const int i0 = (jp + 1) & ~1, P = (n - i0) / 2 + 1;
    for(int e = tid; e < (CL - 1) * P; e += LDL_THREADS) {
      const int q = e / P, i = i0 + 2 * (e - q * P);
      const int dst = q < rank ? q : q + 1;
      const double2 v = *reinterpret_cast<const double2*>(cp + i);
      stAsync2(mapaRank(slotA + (uint32_t)i * 8u, dst), v.x, v.y, mapaRank(fullA, dst));
    }
  };

  // The last pivot is only used by its owner: it is not sent.
  auto lastPivot = [&]() {
    if(tid == 0) {
      const double d = col[(size_t)((n - 1) / CL) * LC + n];
      double r = recipFast(d);
      if(!(d > 0.0) || !isfinite(r)) {
        atomicOr(status, 1);
        r = 0.0;
      }
      rvec[n] = r;
    }
  };

  if(rank == 0) {
    if(n > 1) produce(1);
    else lastPivot();
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
    const double r = own ? rvec[j] : a[0];
    const int lcStart = (j - rank + CL - 1) / CL;  // first local column k > j
    for(int lc = lcStart + tid; lc < ncol; lc += LDL_THREADS) {
      const int k = lc * CL + rank + 1;
      if(k <= n) cbuf[lc] = a[k] * r;
    }
    if(!own && tid == 0) rvec[j] = r;
    __syncthreads();
    const bool ahead = j % CL == rank;  // this CTA owns column j + 1
    if(ahead) {
      double* c1 = col + (size_t)lcStart * LC;
      const double cf = cbuf[lcStart];
      for(int i = j + 1 + tid; i <= n; i += LDL_THREADS) c1[i] = fma(-a[i], cf, c1[i]);
      __syncthreads();
      if(j + 1 < n) produce(j + 1);
      else lastPivot();
    }
    for(int lc = lcStart + (ahead ? 1 : 0) + warp; lc < ncol; lc += NW) {
      const int k = lc * CL + rank + 1;
      if(k > n) break;
      double* ck = col + (size_t)lc * LC;
      const double cf = cbuf[lc];
      for(int i = k + lane; i <= n; i += 32) ck[i] = fma(-a[i], cf, ck[i]);
    }
    __syncthreads();
    if(!own && tid == 0) {
      for(int jn = j + LDL_RING; jn <= n - 1; jn += LDL_RING)
        if((jn - 1) % CL != rank) {
          mbarArriveExpect(smemAddr(&bars[rs]), stepBytes(jn, n));
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
    for(int i = k + tid; i <= n; i += LDL_THREADS)
      F[(size_t)k * ld + i] = i == k ? ck[k] : ck[i] * rk;
    if(tid == 0) rinv[k] = rk;
  }
  cluster.sync();  // no CTA leaves while another may still address its shared memory
}

// ------------------------------------------------------------------ solve --
namespace {

constexpr int SV_THREADS = 1024;
constexpr int SV_NB = 32;

// L y = b then x = L^-T D^-1 y in place on x[1..n] (shared), CTA-wide.
// U[k][i] = l_ik for i > k (row k of F).  blk: SV_NB x (SV_NB + 1) doubles.
__device__ void ldlSolveCta(const double* __restrict__ F, const double* __restrict__ rinv, int n,
                            double* x, double* blk) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, ld = n + 1;
  constexpr int BL = SV_NB + 1;
  // forward, right-looking by blocks of rows [s, e)
  for(int s = 1; s <= n; s += SV_NB) {
    const int e = min(s + SV_NB, n + 1), nb = e - s;
    for(int q = tid; q < SV_NB * SV_NB; q += SV_THREADS) {
      const int jj = q / SV_NB, t = q % SV_NB;  // blk[jj][t] = l_{s+t, s+jj}
      blk[jj * BL + t] = (jj < nb && t < nb && t > jj) ? F[(size_t)(s + jj) * ld + s + t] : 0.0;
    }
    __syncthreads();
    if(warp == 0) {
      double v = lane < nb ? x[s + lane] : 0.0;
#pragma unroll
      for(int jj = 0; jj < SV_NB; jj++) {
        const double yj = __shfl_sync(0xffffffffu, v, jj);
        v = fma(-blk[jj * BL + lane], yj, v);
      }
      if(lane < nb) x[s + lane] = v;
    }
    __syncthreads();
    for(int i = e + tid; i <= n; i += SV_THREADS) {
      double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
      int jj = 0;
      for(; jj + 4 <= nb; jj += 4) {
        a0 = fma(F[(size_t)(s + jj) * ld + i], x[s + jj], a0);
        a1 = fma(F[(size_t)(s + jj + 1) * ld + i], x[s + jj + 1], a1);
        a2 = fma(F[(size_t)(s + jj + 2) * ld + i], x[s + jj + 2], a2);
        a3 = fma(F[(size_t)(s + jj + 3) * ld + i], x[s + jj + 3], a3);
      }
      for(; jj < nb; jj++) a0 = fma(F[(size_t)(s + jj) * ld + i], x[s + jj], a0);
      x[i] -= (a0 + a1) + (a2 + a3);
    }
    __syncthreads();
  }
  for(int i = 1 + tid; i <= n; i += SV_THREADS) x[i] *= rinv[i];
  __syncthreads();
  // backward: x_k = z_k - sum_{i>k} l_ik x_i, blocks from the bottom
  const int nBlk = (n + SV_NB - 1) / SV_NB;
  for(int b = nBlk - 1; b >= 0; b--) {
    const int s = 1 + b * SV_NB, e = min(s + SV_NB, n + 1), nb = e - s;
    for(int q = tid; q < SV_NB * SV_NB; q += SV_THREADS) {
      const int t = q / SV_NB, ii = q % SV_NB;  // blk[t][ii] = l_{s+ii, s+t}
      blk[t * BL + ii] = (t < nb && ii < nb && ii > t) ? F[(size_t)(s + t) * ld + s + ii] : 0.0;
    }
    // tails: row s + warp against the final x beyond the block
    if(warp < nb) {
      const int k = s + warp;
      double a = 0.0;
      for(int i = e + lane; i <= n; i += 32) a = fma(F[(size_t)k * ld + i], x[i], a);
#pragma unroll
      for(int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
      if(lane == 0) x[k] -= a;
    }
    __syncthreads();
    if(warp == 0) {
      double v = lane < nb ? x[s + lane] : 0.0;
#pragma unroll
      for(int ii = SV_NB - 1; ii >= 0; ii--) {
        const double xi = __shfl_sync(0xffffffffu, v, ii);
        v = fma(-blk[lane * BL + ii], xi, v);
      }
      if(lane < nb) x[s + lane] = v;
    }
    __syncthreads();
  }
}

}  // namespace

// Refined solve on a cluster: rhs (n+1 entries, index 0 unused) is replaced by
// the solution.  With status bit 0 set the LU factors and pivots of the
// fallback are used instead (F holds the LU of the pivoted kernel).
template <int CL>
__global__ void __launch_bounds__(SV_THREADS)
    k_ldl_solve(const double* __restrict__ A, const double* __restrict__ F,
                const double* __restrict__ rinv, int n, double* __restrict__ rhs,
                const int* __restrict__ status) {
  extern __shared__ __align__(16) double sv_s[];
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank(), tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int ld = n + 1, LX = (n + 2) & ~1;
  double* x = sv_s;          // LX: solution, then correction (CTA 0)
  double* b = x + LX;        // LX: right-hand side, then residual
  double* x1 = b + LX;       // LX: first solution
  double* blk = x1 + LX;     // SV_NB x (SV_NB + 1)
  if(status[0] & 1) return;  // the LU fallback solves this system
  if(rank == 0) {
    for(int i = tid; i < LX; i += SV_THREADS) {
      const double v = i >= 1 && i <= n ? rhs[i] : 0.0;
      b[i] = v;
      x[i] = v;
    }
    __syncthreads();
    ldlSolveCta(F, rinv, n, x, blk);
    for(int i = tid; i < LX; i += SV_THREADS) x1[i] = x[i];
  }
  cluster.sync();
  // residual rows, spread over the cluster: b_i <- b_i - A_i . x1 (in CTA 0)
  {
    const double* x0 = cluster.map_shared_rank(x1, 0);
    double* b0 = cluster.map_shared_rank(b, 0);
    double* xl = x;  // local copy of x1 (CTA 0 copies onto itself harmlessly later)
    if(rank != 0)
      for(int i = tid; i < LX; i += SV_THREADS) xl[i] = x0[i];
    __syncthreads();
    const double* xs = rank == 0 ? x1 : xl;
    constexpr int NWv = SV_THREADS / 32;
    for(int i = 1 + rank * NWv + warp; i <= n; i += CL * NWv) {
      double a = 0.0;
      for(int j = 1 + lane; j <= n; j += 32) a = fma(A[(size_t)i * ld + j], xs[j], a);
#pragma unroll
      for(int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
      if(lane == 0) b0[i] -= a;
    }
  }
  cluster.sync();
  if(rank == 0) {
    for(int i = tid; i < LX; i += SV_THREADS) x[i] = i >= 1 && i <= n ? b[i] : 0.0;
    __syncthreads();
    ldlSolveCta(F, rinv, n, x, blk);
    for(int i = 1 + tid; i <= n; i += SV_THREADS) rhs[i] = x1[i] + x[i];
  }
}

template __global__ void k_global_ldl<8>(const double*, double*, double*, int, int*);
template __global__ void k_global_ldl<16>(const double*, double*, double*, int, int*);
template __global__ void k_ldl_solve<8>(const double*, const double*, const double*, int, double*,
                                        const int*);
template __global__ void k_ldl_solve<16>(const double*, const double*, const double*, int, double*,
                                         const int*);

namespace {

size_t ldlSmemBytes(int n, int CL) {
  const int LC = (n + 3) & ~1, ncol = (n + CL - 1) / CL;
  return ((size_t)ncol * LC + (size_t)LDL_RING * LC + LC + ((ncol + 1) & ~1)) * sizeof(double) +
         (LDL_RING + 1) * sizeof(unsigned long long);
}

template <class Kern, class... Args>
cudaError_t launchCluster(xb_ctx* c, Kern kernel, int CL, int threads, size_t smem,
                          Args... args) {
  cudaError_t e =
      cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
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

void globalSolveMixed(xb_ctx* c, const double* M, int n, double* rhs, int* piv, int* singular) {
  const int ld = n + 1;
  const bool fresh = c->pool.find("ldl_status") == c->pool.end();
  int* status = buf<int>(c, "ldl_status", 2);
  if(fresh) XB_CUDA(cudaMemsetAsync(status, 0, 2 * sizeof(int), c->stream));
  else XB_CUDA(cudaMemsetAsync(status, 0, sizeof(int), c->stream));
  double* F = buf<double>(c, "ldl_F", (size_t)ld * ld);
  double* rinv = buf<double>(c, "ldl_rinv", ld);
  // 16-CTA clusters where the device allows them, else 8
  static std::atomic<int> clusterSize{0};
  {
    KT_SCOPE(c, "global_ldl");
    cudaError_t e = cudaErrorUnknown;
    if(clusterSize.load() != 8) {
      e = launchCluster(c, k_global_ldl<16>, 16, LDL_THREADS, ldlSmemBytes(n, 16), M, F, rinv, n,
                        status);
      if(e == cudaSuccess) clusterSize = 16;
      else cudaGetLastError();
    }
    if(e != cudaSuccess) {
      XB_CUDA(launchCluster(c, k_global_ldl<8>, 8, LDL_THREADS, ldlSmemBytes(n, 8), M, F, rinv, n,
                            status));
      clusterSize = 8;
    }
    XB_LAUNCHED(c);
  }
  luFallbackSolve(c, M, F, n, rhs, piv, singular, status);
  {
    KT_SCOPE(c, "global_solve");
    const size_t smem = ((size_t)3 * ((n + 2) & ~1) + SV_NB * (SV_NB + 1)) * sizeof(double);
    if(clusterSize.load() == 16)
      XB_CUDA(launchCluster(c, k_ldl_solve<16>, 16, SV_THREADS, smem, (const double*)M,
                            (const double*)F, (const double*)rinv, n, rhs, (const int*)status));
    else
      XB_CUDA(launchCluster(c, k_ldl_solve<8>, 8, SV_THREADS, smem, (const double*)M,
                            (const double*)F, (const double*)rinv, n, rhs, (const int*)status));
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
    throw XbError{XB_ERR_DEVICE_TIMEOUT, "cluster solve: a bounded wait ran out of time"};
  }
}

}  // namespace xb
