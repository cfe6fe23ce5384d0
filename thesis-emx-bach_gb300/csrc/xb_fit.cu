// xb_fit.cu — cd and ksc: per-stamp test fits, convolution-direction merit,
// global normal matrix, global LU solve, per-stamp chi^2 and the
// reject/refill loop (src/cdkscUtil.cpp, src/bachUtil.cpp:288-541,
// cl_kern/cd.cl, cl_kern/ksc.cl, cl_kern/bach.cl:1-127).
//
// Plain mode reproduces the reference's FP64 operation order, so kernel sums,
// merits, chi^2 and therefore the test-stamp and rejection sets are
// bit-identical to the CPU oracle.  Atomic-order compactions of the
// reference (genCdTestStamps, removeBadSigs, checkBadSubStamps) keep
// ascending stamp order.

#include <cooperative_groups.h>

#include <algorithm>
#include <climits>

#include "xb_device.cuh"
#include "xb_internal.h"

namespace cg = cooperative_groups;

namespace xb {

namespace {

// ----------------------------------------------------------- LU helpers ---
// NR lubksb (bach.cl:89-127 / bachUtil.cpp:386-411) by one warp: lanes form
// the products, lane 0 runs each row's subtraction chain in the reference's
// order.  a is row-major with leading dimension ld, 1-based.
__device__ void warpLubksb(const double* a, int ld, int n, const int* idx, double* b,
                           double* prod) {
  const int lane = threadIdx.x & 31;
  int ii = 0;
  for(int i = 1; i <= n; i++) {
    const int ip = idx[i];
    double sum = b[ip];
    __syncwarp();
    if(lane == 0) b[ip] = b[i];
    __syncwarp();
    if(ii != 0) {
      for(int j = ii + lane; j < i; j += 32) prod[j] = a[(size_t)i * ld + j] * b[j];
      __syncwarp();
      if(lane == 0)
        for(int j = ii; j < i; j++) sum -= prod[j];
      sum = __shfl_sync(0xffffffffu, sum, 0);
    } else if(sum != 0.0) {
      ii = i;
    }
    if(lane == 0) b[i] = sum;
    __syncwarp();
  }
  for(int i = n; i >= 1; i--) {
    double sum = b[i];
    for(int j = i + 1 + lane; j <= n; j += 32) prod[j] = a[(size_t)i * ld + j] * b[j];
    __syncwarp();
    if(lane == 0) {
      for(int j = i + 1; j <= n; j++) sum -= prod[j];
      b[i] = sum / a[(size_t)i * ld + i];
    }
    __syncwarp();
  }
}

// Pivot reduction: larger value wins, ties go to the larger row (the
// sequential `dum >= big` rule), NaN never wins.
__device__ __forceinline__ void pivotCombine(double& v, int& i, double ov, int oi) {
  if(oi >= 0 && (i < 0 || ov > v || (ov == v && oi > i))) {
    v = ov;
    i = oi;
  }
}

// ------------------------------------------------------ per-stamp test fit --
// createTestVec/createTestMat (cd.cl:15-44), GPU ludcmp (bach.cl:1-87, no
// zero-row check) and lubksb, saveKernelSums (cd.cl:46-52).  The Crout
// elimination of the reference is run right-looking: every entry receives
// the same products in the same order, so the factors are identical.
constexpr int LU_THREADS = 128;
__global__ void __launch_bounds__(LU_THREADS)
    k_stamp_test_fit(const double* __restrict__ Q, const double* __restrict__ B, int qc,
                     const int* __restrict__ liveN, double* __restrict__ kernelSums) {
  extern __shared__ double lu_s[];
  if(liveN && (int)blockIdx.x >= *liveN) return;
  const int s = blockIdx.x, tid = threadIdx.x, n = qc - 1;
  double* a = lu_s;                 // qc * qc
  double* b = a + qc * qc;          // qc
  double* vv = b + qc;              // qc
  double* prod = vv + qc;           // qc
  int* idx = (int*)(prod + qc);     // qc
  __shared__ double rv[LU_THREADS / 32];
  __shared__ int ri[LU_THREADS / 32];
  __shared__ int sMaxI;
  const double* Qs = Q + (size_t)s * qc * qc;
  for(int k = tid; k < qc * qc; k += LU_THREADS) {
    int i = k / qc, j = k % qc;
    a[k] = (i > 0 && j > 0) ? Qs[(size_t)max(i, j) * qc + min(i, j)] : 0.0;
  }
  for(int i = tid; i < qc; i += LU_THREADS) {
    b[i] = i > 0 ? B[(size_t)s * qc + i] : 0.0;
    idx[i] = 0;
  }
  __syncthreads();
  for(int i = tid; i < qc; i += LU_THREADS) {
    double big = 0.0;
    if(i > 0)
      for(int j = 1; j <= n; j++) {
        double t = fabs(a[i * qc + j]);
        if(t > big) big = t;
      }
    vv[i] = i > 0 ? 1.0 / big : 0.0;
  }
  if(tid == 0) sMaxI = 0;
  __syncthreads();
  for(int j = 1; j <= n; j++) {
    double bv = 0.0;
    int bi = -1;
    for(int i = j + tid; i <= n; i += LU_THREADS) {
      double dum = vv[i] * fabs(a[i * qc + j]);
      if(dum >= 0.0) pivotCombine(bv, bi, dum, i);
    }
#pragma unroll
    for(int o = 16; o > 0; o >>= 1) {
      double ov = __shfl_down_sync(0xffffffffu, bv, o);
      int oi = __shfl_down_sync(0xffffffffu, bi, o);
      pivotCombine(bv, bi, ov, oi);
    }
    if((tid & 31) == 0) {
      rv[tid >> 5] = bv;
      ri[tid >> 5] = bi;
    }
    __syncthreads();
    if(tid == 0) {
      double v = rv[0];
      int i0 = ri[0];
      for(int w = 1; w < LU_THREADS / 32; w++) pivotCombine(v, i0, rv[w], ri[w]);
      if(i0 >= 0) sMaxI = i0;
      idx[j] = sMaxI;
    }
    __syncthreads();
    const int p = sMaxI;
    if(p != j) {
      for(int k = 1 + tid; k <= n; k += LU_THREADS) {
        double t = a[p * qc + k];
        a[p * qc + k] = a[j * qc + k];
        a[j * qc + k] = t;
      }
      __syncthreads();
      if(tid == 0) vv[p] = vv[j];
    }
    __syncthreads();
    if(tid == 0 && a[j * qc + j] == 0.0) a[j * qc + j] = 1.0e-20;
    __syncthreads();
    if(j != n) {
      const double dum = 1.0 / a[j * qc + j];
      for(int i = j + 1 + tid; i <= n; i += LU_THREADS) a[i * qc + j] *= dum;
    }
    __syncthreads();
    const int m = n - j;
    for(int e = tid; e < m * m; e += LU_THREADS) {
      int i = j + 1 + e / m, k = j + 1 + e % m;
      a[i * qc + k] -= a[i * qc + j] * a[j * qc + k];
    }
    __syncthreads();
  }
  if(tid < 32) warpLubksb(a, qc, n, idx, b, prod);
  __syncthreads();
  if(tid == 0) kernelSums[s] = b[1];
}

// ------------------------------------------- per-stamp test fit, mixed ----
// The mixed path only needs each stamp's kernel sum (the first unknown of
// its test system; cd.cl:46-52) for the sigma clip of cd, and its Q, B already
// differ from the plain ones at the 1e-11 level, so it solves the symmetric
// positive definite test system (createTestMat / createTestVec, cd.cl:15-44)
// by LDL^T without pivoting, one warp per stamp, instead of the reference's
// LU with partial pivoting.  The kernel-sum unknown is ordered last and the
// right-hand side rides along as an extra column of the elimination, so after
// it the kernel sum is that column's last entry over the last pivot (with L D
// L^T x = b and z = L^-1 b, the last row of L^T x = D^-1 z is x_n = z_n / d_n):
// no back substitution.  A zero pivot becomes 1e-20, as in the reference's LU.
// Warps (stamps) per CTA: 4 (variant 0), 2 or 8; identical results.
template <int TF_WARPS>
__global__ void __launch_bounds__(TF_WARPS * 32)
    k_stamp_test_fit_ldl(const double* __restrict__ Q, const double* __restrict__ B, int qc,
                         int nStamps, const int* __restrict__ liveN,
                         double* __restrict__ kernelSums) {
  extern __shared__ double tf_s[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int s = blockIdx.x * TF_WARPS + warp;
  const int nLive = liveN ? min(nStamps, *liveN) : nStamps;
  if(s >= nLive) return;  // whole warps only; the kernel has no block barrier
  const int n = qc - 1, ld = n + 1;  // unknowns; row stride (column n = the RHS)
  double* a = tf_s + (size_t)warp * n * ld;
  const double* Qs = Q + (size_t)s * qc * qc;
  // unknown order: 2, 3, ..., n, then 1 (the kernel sum)
  auto unk = [&](int p) { return p < n - 1 ? p + 2 : 1; };
  for(int e = lane; e < n * ld; e += 32) {
    const int p = e / ld, q = e % ld, u = unk(p);
    double v;
    if(q == n) {
      v = B[(size_t)s * qc + u];
    } else {
      const int t = unk(q);
      v = Qs[(size_t)max(u, t) * qc + min(u, t)];
    }
    a[e] = v;
  }
  __syncwarp();
  for(int k = 0; k < n; k++) {
    double d = a[k * ld + k];
    if(d == 0.0) d = 1.0e-20;
    const double rd = 1.0 / d;
    const double bk = a[k * ld + n];
    for(int i = k + 1 + lane; i < n; i += 32) {
      double* ai = a + i * ld;
      const double li = ai[k] * rd;
      for(int j = k + 1; j <= i; j++) ai[j] = fma(-li, a[j * ld + k], ai[j]);
      ai[n] = fma(-li, bk, ai[n]);
    }
    __syncwarp();
  }
  if(lane == 0) {
    double d = a[(n - 1) * ld + n - 1];
    if(d == 0.0) d = 1.0e-20;
    kernelSums[s] = a[(n - 1) * ld + n] / d;
  }
}

// ------------------------------------------------------------ cd select ---
// sigmaClip of the kernel sums (10 iterations, cdkscUtil.cpp:74-76) and
// genCdTestStamps (cd.cl:54-94) in ascending order.
__global__ void __launch_bounds__(256)
    k_cd_select(const double* __restrict__ ks, int n, const int* __restrict__ liveN, double alpha,
                double sigKernFit, uint8_t* flags, double* cs, double* cs2,
                int* __restrict__ testIdx, int* __restrict__ nTest, double* __restrict__ stats) {
  if(liveN) n = *liveN;
  __shared__ double sMean, sStd;
  __shared__ int sh[4];
  __shared__ int warpTot[8];
  __shared__ int sTotal;
  blockSigmaClip(ks, n, 10, alpha, flags, cs, cs2, &sMean, &sStd, sh);
  const double m = sMean, sd = sStd;
  int done = 0;
  for(int base = 0; base < n; base += 256) {
    int s = base + threadIdx.x;
    int keep = (s < n && fabs((ks[s] - m) / sd) < sigKernFit) ? 1 : 0;
    int pos = blockScanExcl(keep, warpTot, &sTotal) + done;
    if(keep) testIdx[pos] = s;
    done += sTotal;
    __syncthreads();
  }
  if(threadIdx.x == 0) {
    *nTest = done;
    stats[0] = m;
    stats[1] = sd;
  }
}

// ---------------------------------------------------- spatial weights -----
// createMatrixWeights (cd.cl:152-180) = the weight loop of CPU createMatrix
// (cdkscUtil.cpp:331-342).
__global__ void k_weights(const int* __restrict__ list, int nList, const int* __restrict__ liveN,
                          const int* __restrict__ count, const int* __restrict__ cur,
                          const int2* __restrict__ ssxy, int maxSS, const int2* __restrict__ kp,
                          int nC2, int w, int h, double* __restrict__ wts) {
  if(liveN) nList = min(nList, *liveN);
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if(e >= nList * nC2) return;
  int t = e / nC2, k = e % nC2, s = list[t];
  double a = 0.0;
  if(cur[s] < count[s]) {
    int2 c = ssxy[(size_t)s * maxSS + cur[s]];
    a = ipowD(floatNormD(c.x, w), kp[k].x) * ipowD(floatNormD(c.y, h), kp[k].y);
  }
  wts[e] = a;
}

// ------------------------------------------------------- per-stamp dots ---
// The W dot products the global matrix needs (cd.cl:199-261,
// cdkscUtil.cpp:363-392) and the background projections of both RHS forms:
//   dots[t][0 .. nC1*nBG)            W[i1] . W[bg]       (i1 = 1..nC1)
//   dots[t][nC1*nBG + ib]            W[0]  . W[bg ib]
//   dots[t][.. + nBG + ib*nBG + jb]  W[bg ib] . W[bg jb]  (jb <= ib)
//   dots[t][.. + nBG*nBG + ib]       W[bg ib] . O, row-major, FP64 (cd.cl:331-339)
//   dots[t][.. + nBG + ib]           W[bg ib] . float(O), column-major
//                                    (cdkscUtil.cpp:459-469)
// Every dot runs in ascending pixel order (or the stated order) per thread.
constexpr int DOT_THREADS = 256, DOT_KT = 32, DOT_PAIRS = 4;
template <class T>
__global__ void __launch_bounds__(DOT_THREADS)
    k_stamp_dots(const int* __restrict__ list, const int* __restrict__ count,
                 const int* __restrict__ cur, const int2* __restrict__ ssxy, int maxSS,
                 const double* __restrict__ W, int wRows, int hSS, int nPSF, int nBG,
                 const T* __restrict__ O, int w, int h, double* __restrict__ dots, int stride,
                 const double* __restrict__ omega) {
  extern __shared__ double dot_s[];
  const int t = blockIdx.x, s = list[t], tid = threadIdx.x;
  const int fSS = 2 * hSS + 1, wCols = fSS * fSS, nC1 = nPSF - 1;
  const double* Ws = W + (size_t)s * wRows * wCols;
  double* out = dots + (size_t)t * stride;
  const bool live = cur[s] < count[s];
  double* tile = dot_s;                       // wRows x (DOT_KT+1)
  double* sub = dot_s + wRows * (DOT_KT + 1); // wCols (image) values
  double* om = sub + wCols;                   // wCols pixel weights (weighted fit)
  if(omega)
    for(int i = tid; i < wCols; i += DOT_THREADS) om[i] = omega[(size_t)s * wCols + i];
  // products: the (rowA, rowB) pairs tid, tid + DOT_THREADS, ... (up to
  // DOT_PAIRS per thread; the host checks the bound), each summed over the
  // pixels in ascending order
  const int nKB = nC1 * nBG, nPairs = nKB + nBG + nBG * nBG;
  int ra[DOT_PAIRS], rb[DOT_PAIRS], oi[DOT_PAIRS];
  double acc[DOT_PAIRS];
#pragma unroll
  for(int q = 0; q < DOT_PAIRS; q++) {
    const int pi = tid + q * DOT_THREADS;
    ra[q] = rb[q] = oi[q] = -1;
    acc[q] = 0.0;
    if(pi >= nPairs) continue;
    if(pi < nKB) {
      ra[q] = 1 + pi / nBG;
      rb[q] = nPSF + pi % nBG;
      oi[q] = pi;
    } else if(pi < nKB + nBG) {
      ra[q] = 0;
      rb[q] = nPSF + (pi - nKB);
      oi[q] = pi;
    } else {
      int e = pi - nKB - nBG, ib = e / nBG, jb = e % nBG;
      if(jb <= ib) {
        ra[q] = nPSF + ib;
        rb[q] = nPSF + jb;
        oi[q] = nKB + nBG + ib * nBG + jb;
      }
    }
  }
  for(int k0 = 0; k0 < wCols; k0 += DOT_KT) {
    const int kt = min(DOT_KT, wCols - k0);
    for(int i = tid; i < wRows * DOT_KT; i += DOT_THREADS) {
      int r = i / DOT_KT, kk = i % DOT_KT;
      tile[r * (DOT_KT + 1) + kk] = kk < kt ? Ws[(size_t)r * wCols + k0 + kk] : 0.0;
    }
    __syncthreads();
#pragma unroll
    for(int q = 0; q < DOT_PAIRS; q++) {
      if(ra[q] < 0) continue;
      const double* pa = tile + ra[q] * (DOT_KT + 1);
      const double* pb = tile + rb[q] * (DOT_KT + 1);
      double a = acc[q];
      if(omega) {
        for(int kk = 0; kk < kt; kk++) a += pa[kk] * (pb[kk] * om[k0 + kk]);
      } else {
        for(int kk = 0; kk < kt; kk++) a += pa[kk] * pb[kk];
      }
      acc[q] = a;
    }
    __syncthreads();
  }
#pragma unroll
  for(int q = 0; q < DOT_PAIRS; q++)
    if(ra[q] >= 0) out[oi[q]] = acc[q];
  // background projections on the other image
  const int base = nKB + nBG + nBG * nBG;
  if(live) {
    const int2 c = ssxy[(size_t)s * maxSS + cur[s]];
    for(int i = tid; i < wCols; i += DOT_THREADS) {
      int x = i % fSS - hSS, y = i / fSS - hSS;
      int gx = min(max(x + c.x, 0), w - 1), gy = min(max(y + c.y, 0), h - 1);
      sub[i] = (double)O[(size_t)gx + (size_t)gy * w];
    }
  }
  __syncthreads();
  if(tid < 2 * nBG) {
    const int ib = tid % nBG;
    const double* wb = Ws + (size_t)(nPSF + ib) * wCols;
    double q = 0.0;
    if(live) {
      if(tid < nBG) {
        for(int k = 0; k < wCols; k++) q += omega ? wb[k] * (sub[k] * om[k]) : wb[k] * sub[k];
      } else {
        for(int x = 0; x < fSS; x++)
          for(int y = 0; y < fSS; y++) {
            int k = x + fSS * y;
            q += omega ? wb[k] * ((double)(float)sub[k] * om[k]) : wb[k] * (double)(float)sub[k];
          }
      }
    }
    out[base + tid] = q;
  }
}

// ------------------------------------------------------ global matrix ------
// Lower triangle of createMatrix (cd.cl:182-295 == cdkscUtil.cpp:307-402),
// each entry summed over the listed stamps in order, then mirrored.
__global__ void __launch_bounds__(256)
    k_build_matrix(const int* __restrict__ list, int nList, const int* __restrict__ count,
                   const int* __restrict__ cur, const double* __restrict__ Q, int qc,
                   const double* __restrict__ wts, const double* __restrict__ dots, int stride,
                   int byStamp, int nC1, int nC2, int nBG, int matSize, double* __restrict__ M) {
  const int ld = matSize + 1, nComp = nC1 * nC2;
  const long long nTri = (long long)matSize * (matSize + 1) / 2;
  for(long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < nTri;
      e += (long long)gridDim.x * blockDim.x) {
    // e -> (r, c) with 1 <= c <= r <= matSize
    int r = (int)((sqrt(8.0 * (double)e + 1.0) - 1.0) * 0.5);
    while((long long)(r + 1) * (r + 2) / 2 <= e) r++;
    while((long long)r * (r + 1) / 2 > e) r--;
    const int row = r + 1, col = (int)(e - (long long)r * (r + 1) / 2) + 1;
    double m0 = 0.0;
    for(int t = 0; t < nList; t++) {
      const int s = list[t];
      const double* Qs = Q + (size_t)s * qc * qc;
      const double* wt = wts + (size_t)t * nC2;
      const double* dt = dots + (size_t)(byStamp ? s : t) * stride;
      if(row == 1 && col == 1) {
        m0 += Qs[1 * qc + 1];
      } else if(row > nComp + 1 && col > nComp + 1) {
        m0 += dt[nC1 * nBG + nBG + (row - (nComp + 2)) * nBG + (col - (nComp + 2))];
      } else if(col == 1 && row > nComp + 1) {
        m0 += dt[nC1 * nBG + (row - (nComp + 2))];
      } else if(row > nComp + 1 && col >= 2) {
        int ib = row - (nComp + 2), i1 = (col - 2) / nC2 + 1, i2 = (col - 2) % nC2;
        m0 += dt[(i1 - 1) * nBG + ib] * wt[i2];
      } else if(col == 1 && row >= 2) {
        int i = row - 2, i1 = i / nC2, i2 = i - i1 * nC2;
        m0 += wt[i2] * Qs[(i1 + 2) * qc + 1];
      } else {
        int i = row - 2, j = col - 2;
        int i1 = i / nC2, i2 = i - i1 * nC2, j1 = j / nC2, j2 = j - j1 * nC2;
        m0 += wt[i2] * wt[j2] * Qs[(i1 + 2) * qc + (j1 + 2)];
      }
    }
    M[(size_t)row * ld + col] = m0;
    M[(size_t)col * ld + row] = m0;
  }
  // row 0 / column 0 stay zero
  for(int i = blockIdx.x * blockDim.x + threadIdx.x; i < ld; i += gridDim.x * blockDim.x) {
    M[i] = 0.0;
    M[(size_t)i * ld] = 0.0;
  }
}

// createScProd: kernel terms and the constant term are common to both forms;
// the background terms come from k_stamp_dots (form selects the column).
__global__ void k_build_rhs(const int* __restrict__ list, int nList, const int* __restrict__ count,
                            const int* __restrict__ cur, const double* __restrict__ B, int qc,
                            const double* __restrict__ wts, const double* __restrict__ dots,
                            int stride, int byStamp, int bgBase, int nC1, int nC2, int nBG,
                            int nSol, double* __restrict__ res) {
  const int id = blockIdx.x * blockDim.x + threadIdx.x;
  if(id >= nSol) return;
  const int nComp = nC1 * nC2;
  double r0 = 0.0;
  for(int t = 0; t < nList; t++) {
    const int s = list[t];
    if(cur[s] >= count[s]) continue;
    const double* Bs = B + (size_t)s * qc;
    if(id == 1) {
      r0 += Bs[1];
    } else if(id >= 2 && id < nComp + 2) {
      int i = (id - 2) / nC2 + 1, j = (id - 2) % nC2;
      r0 += Bs[i + 1] * wts[(size_t)t * nC2 + j];
    } else if(id >= nComp + 2 && id < nComp + 2 + nBG) {
      r0 += dots[(size_t)(byStamp ? s : t) * stride + bgBase + (id - (nComp + 2))];
    }
  }
  res[id] = r0;
}

// ------------------------------------------------------ global LU ---------
// CPU ludcmp (bachUtil.cpp:319-384) on the (matSize)^2 system, distributed
// over a thread-block cluster: CTA r owns the columns j with (j-1) % CL == r
// in shared memory.  Per step the owner of column j finds the pivot, scales
// the L column and publishes both; every CTA then swaps the pivot rows and
// updates its own trailing columns.  Right-looking elimination gives the
// same products in the same order as the reference's Crout loops.
template <int CL>
__global__ void __launch_bounds__(256)
    k_global_lu(double* __restrict__ M, int n, int* __restrict__ idxOut,
                int* __restrict__ singular) {
  extern __shared__ double glu_s[];
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank(), tid = threadIdx.x, nt = blockDim.x;
  const int ld = n + 1;
  const int ncol = (n + CL - 1) / CL;  // local columns (some may be past n)
  double* col = glu_s;                          // ncol * ld (column-major)
  double* vv = col + (size_t)ncol * ld;         // ld
  double* bc = vv + ld;                         // 2 * (ld + 1) broadcast buffers
  double* L = bc + 2 * (ld + 1);                // ld
  __shared__ double rv[8];
  __shared__ int ri[8];
  __shared__ int sP, sMaxI, sSing;
  // row scaling (CPU form: a zero row aborts before the elimination)
  if(tid == 0) sSing = 0;
  __syncthreads();
  for(int i = 1 + tid; i <= n; i += nt) {
    double big = 0.0;
    for(int j = 1; j <= n; j++) {
      double t = fabs(M[(size_t)i * ld + j]);
      if(t > big) big = t;
    }
    if(big == 0.0) sSing = 1;
    vv[i] = 1.0 / big;
  }
  __syncthreads();
  if(sSing) {
    if(rank == 0 && tid == 0) *singular = 1;
    for(int i = tid; i <= n; i += nt)
      if(rank == 0) idxOut[i] = 0;
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
      double bv = 0.0;
      int bi = -1;
      for(int i = j + tid; i <= n; i += nt) {
        double dum = vv[i] * fabs(cj[i]);
        if(dum >= 0.0) pivotCombine(bv, bi, dum, i);
      }
#pragma unroll
      for(int o = 16; o > 0; o >>= 1) {
        double ov = __shfl_down_sync(0xffffffffu, bv, o);
        int oi = __shfl_down_sync(0xffffffffu, bi, o);
        pivotCombine(bv, bi, ov, oi);
      }
      if((tid & 31) == 0) {
        rv[tid >> 5] = bv;
        ri[tid >> 5] = bi;
      }
      __syncthreads();
      if(tid == 0) {
        double v = rv[0];
        int i0 = ri[0];
        for(int w = 1; w < nt / 32; w++) pivotCombine(v, i0, rv[w], ri[w]);
        int p = i0 >= 0 ? i0 : sMaxI;
        if(p != j) {
          double t = cj[p];
          cj[p] = cj[j];
          cj[j] = t;
        }
        if(cj[j] == 0.0) cj[j] = 1.0e-20;
        myBc[0] = (double)p;
      }
      __syncthreads();
      if(j != n) {
        const double dum = 1.0 / cj[j];
        for(int i = j + 1 + tid; i <= n; i += nt) cj[i] *= dum;
      }
      __syncthreads();
      for(int i = j + 1 + tid; i <= n; i += nt) myBc[i] = cj[i];
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
        if(rank == owner && lc == lcj) continue;  // already swapped by the owner
        double* c = col + (size_t)lc * ld;
        double t = c[p];
        c[p] = c[j];
        c[j] = t;
      }
      if(tid == 0) vv[p] = vv[j];
    }
    __syncthreads();
    // trailing update of the local columns k > j
    const int lcStart = (j - rank + CL - 1) / CL;  // first lc with lc*CL + rank + 1 > j
    const int nLoc = ncol - lcStart, m = n - j;
    for(int e = tid; e < nLoc * m; e += nt) {
      const int lc = lcStart + e / m, i = j + 1 + e % m;
      if(lc * CL + rank + 1 > n) continue;
      double* c = col + (size_t)lc * ld;
      c[i] -= L[i] * c[j];
    }
    __syncthreads();
  }
  cluster.sync();
  for(int lc = 0; lc < ncol; lc++) {
    const int j = lc * CL + rank + 1;
    if(j > n) break;
    for(int i = tid; i <= n; i += nt) M[(size_t)i * ld + j] = col[(size_t)lc * ld + i];
  }
  if(rank == 0 && tid == 0) idxOut[0] = 0;
}

// lubksb of the global system (bachUtil.cpp:380-411) on two warps: lane 0 of
// warp 0 runs each row's sequential chain `sum -= a[i][j] * b[j]` (the
// reference's order and roundings), while warp 1 forms the next row's
// products a[i'][j] * b[j] for the b[j] already final; lane 0 forms the one
// product that needs the row it just finished, from a value it loaded before
// its chain.  One 64-thread barrier per row.
constexpr int LUB_THREADS = 64;
__global__ void __launch_bounds__(LUB_THREADS)
    k_global_lubksb(const double* __restrict__ M, int n, const int* __restrict__ idx,
                    double* __restrict__ b) {
  extern __shared__ double sol_s[];
  double* bs = sol_s;          // n + 1
  double* pA = bs + n + 1;     // n + 1: products of the current row
  double* pB = pA + n + 1;     // n + 1: products of the next row
  int* is = (int*)(pB + n + 1);
  __shared__ int iiS[2];  // ii for row i in slot i & 1 (written one row ahead)
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, ld = n + 1;
  for(int i = tid; i <= n; i += LUB_THREADS) {
    bs[i] = b[i];
    is[i] = idx[i];
  }
  if(tid == 0) iiS[0] = iiS[1] = 0;
  __syncthreads();
  double* cur = pA;
  double* nxt = pB;
  // forward: L y = P b
  for(int i = 1; i <= n; i++) {
    const int ii0 = iiS[i & 1];
    if(tid == 0) {
      const double aNext = i < n ? M[(size_t)(i + 1) * ld + i] : 0.0;
      const int ip = is[i];
      double sum = bs[ip];
      bs[ip] = bs[i];
      int ii = ii0;
      if(ii0 != 0) {
#pragma unroll 8
        for(int j = ii0; j < i; j++) sum -= cur[j];
      } else if(sum != 0.0) {
        ii = i;
      }
      iiS[(i + 1) & 1] = ii;
      bs[i] = sum;
      if(i < n && ii != 0) nxt[i] = aNext * sum;
    } else if(warp == 1 && ii0 != 0 && i < n) {
      for(int j = ii0 + lane; j < i; j += 32) nxt[j] = M[(size_t)(i + 1) * ld + j] * bs[j];
    }
    __syncthreads();
    double* t = cur;
    cur = nxt;
    nxt = t;
  }
  // backward: U x = y (row n has no products)
  for(int i = n; i >= 1; i--) {
    if(tid == 0) {
      const double aii = M[(size_t)i * ld + i];
      const double aPrev = i > 1 ? M[(size_t)(i - 1) * ld + i] : 0.0;
      double sum = bs[i];
      if(i < n) {
#pragma unroll 8
        for(int j = i + 1; j <= n; j++) sum -= cur[j];
      }
      const double xi = sum / aii;
      bs[i] = xi;
      if(i > 1) nxt[i] = aPrev * xi;
    } else if(warp == 1 && i > 1) {
      for(int j = i + 1 + lane; j <= n; j += 32) nxt[j] = M[(size_t)(i - 1) * ld + j] * bs[j];
    }
    __syncthreads();
    double* t = cur;
    cur = nxt;
    nxt = t;
  }
  for(int i = tid; i <= n; i += LUB_THREADS) b[i] = bs[i];
}

// ----------------------------------------------------- kernel sums --------
// makeKernelCoeffs + makeKernel + sumKernel (cd.cl:354-442): kernel image at
// (x, y) and its sum; tree=1 sums in 32-wide groups like sumKernel, tree=0
// sequentially like the CPU makeKernel (bachUtil.cpp:532-538).
__global__ void k_kernel_sum(const double* __restrict__ sol, const double* __restrict__ vec,
                             int nPSF, int kOrder, int fK, double xf, double yf, int tree,
                             double* __restrict__ out) {
  __shared__ double coeff[MAX_NPSF];
  __shared__ double kern[MAX_FK * MAX_FK];
  __shared__ double part[64];
  const int tid = threadIdx.x, nk = fK * fK;
  for(int i = tid; i < nPSF; i += blockDim.x) {
    double c = 0.0;
    if(i == 0) {
      c = sol[1];
    } else {
      int k = 2 + (i - 1) * ((kOrder + 1) * (kOrder + 2) / 2);
      double aX = 1.0;
      for(int x = 0; x <= kOrder; x++) {
        double aY = 1.0;
        for(int y = 0; y <= kOrder - x; y++) {
          c += sol[k++] * aX * aY;
          aY *= yf;
        }
        aX *= xf;
      }
    }
    coeff[i] = c;
  }
  __syncthreads();
  for(int p = tid; p < nk; p += blockDim.x) {
    double k0 = 0.0;
    for(int q = 0; q < nPSF; q++) k0 += coeff[q] * vec[(size_t)q * nk + p];
    kern[p] = k0;
  }
  __syncthreads();
  if(tid == 0) {
    double s = 0.0;
    if(!tree) {
      for(int p = 0; p < nk; p++) s += kern[p];
    } else {
      int count = nk;
      double* cur = kern;
      while(count > 1) {
        int groups = (count + 31) / 32;
        for(int g = 0; g < groups; g++) {
          double a = 0.0;
          int lc = min(32, count - g * 32);
          for(int l = 0; l < lc; l++) a += cur[g * 32 + l];
          part[g] = a;
        }
        for(int g = 0; g < groups; g++) kern[g] = part[g];
        cur = kern;
        count = groups;
      }
      s = kern[0];
    }
    *out = s;
  }
}

// --------------------------------------------------------------- chi^2 ----
// calcSigs (cdkscUtil.cpp:477-583): calcSigBg + getBackground (cd.cl:444-487),
// makeModel (:489-531, FP32 model), calcSig (:533-598) and reduceSig
// (:600-655), one CTA per listed stamp.
constexpr int SIG_THREADS = 256;
template <class T>
__global__ void __launch_bounds__(SIG_THREADS)
    k_sigs(const int* __restrict__ list, const int* __restrict__ count,
           const int* __restrict__ cur, const int2* __restrict__ ssxy, int maxSS,
           const double* __restrict__ W, int wRows, int hSS, int nPSF, int kOrder, int bgOrder,
           int nComp, const double* __restrict__ sol, const T* __restrict__ tImg,
           const T* __restrict__ sImg, uint16_t* __restrict__ mask, int w, int h,
           double invGain, double rn2x2, double* __restrict__ sig) {
  extern __shared__ double sig_s[];
  const int t = blockIdx.x, s = list[t], tid = threadIdx.x;
  const int fSS = 2 * hSS + 1, pix = fSS * fSS, reduceCount = (pix + 31) / 32;
  double* coeff = sig_s;                        // nPSF
  double* term = coeff + nPSF;                  // reduceCount*32
  double* part = term + reduceCount * 32;       // reduceCount
  int* cnt = (int*)(part + reduceCount);        // reduceCount*32
  int* pcnt = cnt + reduceCount * 32;           // reduceCount
  __shared__ double sBg;
  const bool live = cur[s] < count[s];
  int2 c = make_int2(0, 0);
  if(live) c = ssxy[(size_t)s * maxSS + cur[s]];
  const double* Ws = W + (size_t)s * wRows * pix;
  if(live) {
    const double xf = (c.x - w * 0.5) / (w * 0.5), yf = (c.y - h * 0.5) / (h * 0.5);
    const int nC2 = (kOrder + 1) * (kOrder + 2) / 2;
    for(int i = 1 + tid; i < nPSF; i += SIG_THREADS) {
      int k = 2 + (i - 1) * nC2;
      double cc = 0.0, ax = 1.0;
      for(int x = 0; x <= kOrder; x++) {
        double ay = 1.0;
        for(int y = 0; y <= kOrder - x; y++) {
          cc += sol[k++] * ax * ay;
          ay *= yf;
        }
        ax *= xf;
      }
      coeff[i] = cc;
    }
    if(tid == 0) {
      // getBackground with the double normalisation of cd.cl:446-447
      const double bxf = (c.x - 0.5 * w) / (0.5 * w), byf = (c.y - 0.5 * h) / (0.5 * h);
      double bg = 0.0, ax = 1.0;
      int k = nComp + 2;
      for(int i = 0; i <= bgOrder; i++) {
        double ay = 1.0;
        for(int j = 0; j <= bgOrder - i; j++) {
          bg += sol[k++] * ax * ay;
          ay *= byf;
        }
        ax *= bxf;
      }
      sBg = bg;
    }
  }
  __syncthreads();
  const double bg = sBg, sol1 = sol[1];
  for(int gi = tid; gi < reduceCount * 32; gi += SIG_THREADS) {
    const int gx = gi % fSS, gy = gi / fSS;
    double s0 = 0.0;
    int ok = 0;
    if(live && gy < fSS) {
      const int j = gx + gy * fSS;
      float m0 = (float)(sol1 * Ws[j]);
      for(int i = 1; i < nPSF; i++) m0 = (float)((double)m0 + coeff[i] * Ws[(size_t)i * pix + j]);
      const int ax = gx - fSS / 2 + c.x, ay = gy - fSS / 2 + c.y;
      const size_t ai = (size_t)min(max(ax, 0), w - 1) + (size_t)min(max(ay, 0), h - 1) * w;
      const double tD = (double)m0, sD = (double)sImg[ai];
      const double diff = tD - sD + bg;
      if((mask[ai] & BAD_INPUT) == 0 && fabs(sD) > 1e-10) {
        if(isnan(tD) || isnan(sD)) {
          maskOr(mask, ai, NAN_PIXEL);
        } else {
          ok = 1;
          s0 = diff * diff / ((fabs((double)tImg[ai]) + fabs(sD)) * invGain + rn2x2);
        }
      }
    }
    term[gi] = s0;
    cnt[gi] = ok;
  }
  __syncthreads();
  for(int g = tid; g < reduceCount; g += SIG_THREADS) {
    double a = 0.0;
    int k = 0;
    for(int l = 0; l < 32; l++) {
      a += term[g * 32 + l];
      k += cnt[g * 32 + l];
    }
    part[g] = a;
    pcnt[g] = k;
  }
  __syncthreads();
  if(tid == 0) {
    int count_ = reduceCount;
    double result = 0.0;
    bool first = true;
    while(count_ > 1 || first) {
      const int next = (count_ + 31) / 32;
      for(int g = 0; g < next; g++) {
        double a = 0.0;
        int k = 0;
        const int lc = min(32, count_ - g * 32);
        for(int l = 0; l < lc; l++) {
          a += part[g * 32 + l];
          k += pcnt[g * 32 + l];
        }
        if(next == 1) {
          if(k == 0) a = -1.0;
          else {
            a /= k;
            if(a >= 1e10) a = -1.0;
          }
          result = a;
        }
        part[g] = a;
        pcnt[g] = k;
      }
      count_ = next;
      first = false;
    }
    sig[t] = result;
  }
}

// ------------------------------------------------------- cd merit ----------
// removeBadSigs (cd.cl:657-695, ascending order) + sigmaClip (10 iterations)
// + merit = mean / kernelMean, or 666 when nothing survives
// (cdkscUtil.cpp:234-265).
__global__ void __launch_bounds__(256)
    k_cd_merit(const double* __restrict__ sig, int n, const int* __restrict__ liveN,
               const double* __restrict__ kernelMean, double alpha, double* clean, uint8_t* flags,
               double* cs, double* cs2, double* __restrict__ merit) {
  if(liveN) n = *liveN;
  __shared__ int warpTot[8];
  __shared__ int sTotal;
  __shared__ double sMean, sStd;
  __shared__ int sh[4];
  int done = 0;
  for(int base = 0; base < n; base += 256) {
    int i = base + threadIdx.x;
    int keep = (i < n && sig[i] >= 0.0) ? 1 : 0;
    int pos = blockScanExcl(keep, warpTot, &sTotal) + done;
    if(keep) clean[pos] = sig[i];
    done += sTotal;
    __syncthreads();
  }
  if(done == 0) {
    if(threadIdx.x == 0) *merit = 666;
    return;
  }
  blockSigmaClip(clean, done, 10, alpha, flags, cs, cs2, &sMean, &sStd, sh);
  if(threadIdx.x == 0) *merit = sMean / *kernelMean;
}

// ---------------------------------------------------------- ksc check -----
// checkFitSolution (cdkscUtil.cpp:686-770): checkBadSubStamps (ksc.cl:1-49,
// ascending chi^2 list), sigmaClip (10 iterations),
// checkBadSubStampsFromSigmaClip (ksc.cl:51-72) on the stale chi^2 with the
// advanced indices.  The two refills of the reference are merged into one
// list: a stamp advanced in the first pass has chi^2 = -1, which the second
// pass can never reject, and a refill depends only on the new index.
__global__ void __launch_bounds__(256)
    k_ksc_check(const double* __restrict__ sig, int n, const int* __restrict__ liveN,
                const int* __restrict__ count, int* __restrict__ cur, double alpha,
                double sigKernFit, double* chi2, uint8_t* flags, double* cs, double* cs2,
                int* __restrict__ refill,
                int* __restrict__ out /* [0]=nRefill [1]=nPass1 [2]=nPass2 */,
                int* __restrict__ passOf) {
  if(liveN) n = *liveN;
  __shared__ int warpTot[8];
  __shared__ int sTotal;
  __shared__ double sMean, sStd;
  __shared__ int sh[4];
  int done = 0;
  for(int base = 0; base < n; base += 256) {
    int s = base + threadIdx.x;
    int keep = 0;
    if(s < n) {
      passOf[s] = -1;
      if(cur[s] < count[s]) {
        if(sig[s] == -1.0) {
          cur[s] = cur[s] + 1;
          passOf[s] = 0;
        } else {
          keep = 1;
        }
      }
    }
    int pos = blockScanExcl(keep, warpTot, &sTotal) + done;
    if(keep) chi2[pos] = sig[s];
    done += sTotal;
    __syncthreads();
  }
  blockSigmaClip(chi2, done, 10, alpha, flags, cs, cs2, &sMean, &sStd, sh);
  const double m = sMean, sd = sStd;
  int nRef = 0, n1 = 0, n2 = 0;
  for(int base = 0; base < n; base += 256) {
    int s = base + threadIdx.x;
    int inv = 0;
    if(s < n) {
      if(passOf[s] == 0) {
        inv = 1;
        n1++;
      } else if(cur[s] < count[s] && (sig[s] - m) > sigKernFit * sd) {
        cur[s] = cur[s] + 1;
        passOf[s] = 1;
        inv = 1;
        n2++;
      }
    }
    int pos = blockScanExcl(inv, warpTot, &sTotal) + nRef;
    if(inv) refill[pos] = s;
    nRef += sTotal;
    __syncthreads();
  }
  atomicAdd(&out[1], n1);
  atomicAdd(&out[2], n2);
  if(threadIdx.x == 0) out[0] = nRef;
}

__global__ void k_zero_ints(int* p, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if(i < n) p[i] = 0;
}

}  // namespace

// ========================================================= host side ======

struct FitBuffers {
  int* list;
  double* wts;
  double* dots;
  int stride;
  double* M;
  double* rhs;
  int* piv;
  int* singular;
  double* sig;
  double* scratchD;   // clip data copies
  uint8_t* flags;
  double* cs;
  double* cs2;
};

static FitBuffers fitBuffers(xb_ctx* c, int nMax) {
  const Geo& g = c->g;
  FitBuffers f{};
  const int ld = g.matSize + 1;
  f.list = buf<int>(c, "fit_list", std::max(nMax, 1));
  f.wts = buf<double>(c, "fit_wts", (size_t)std::max(nMax, 1) * g.nComp2);
  f.stride = g.nComp1 * g.nBG + g.nBG + g.nBG * g.nBG + 2 * g.nBG;
  f.dots = buf<double>(c, "fit_dots", (size_t)std::max(nMax, 1) * f.stride);
  f.M = buf<double>(c, "fit_M", (size_t)ld * ld);
  f.rhs = buf<double>(c, "fit_rhs", std::max(g.nSol, ld));
  f.piv = buf<int>(c, "fit_piv", ld);
  f.singular = buf<int>(c, "fit_singular", 1);
  f.sig = buf<double>(c, "fit_sig", std::max(nMax, 1));
  f.scratchD = buf<double>(c, "fit_clipdata", std::max(nMax, 1));
  f.flags = buf<uint8_t>(c, "fit_flags", std::max(nMax, 1));
  f.cs = buf<double>(c, "fit_cs", std::max(nMax, 1));
  f.cs2 = buf<double>(c, "fit_cs2", std::max(nMax, 1));
  return f;
}

static int2* kernelPowers(xb_ctx* c) {
  const Geo& g = c->g;
  std::vector<int2> kp(g.nComp2);
  for(int k = 0; k < g.nComp2; k++) kp[k] = make_int2(c->basis.kpX[k], c->basis.kpY[k]);
  int2* d = buf<int2>(c, "kernelPowers", g.nComp2);
  toDevice(c, d, kp);
  return d;
}

// matrix + RHS + LU + solve for the stamps list[0..nList) of set si, with
// the other image `other`; cpuRhs selects the ksc RHS form.  liveN, when
// set, holds the live length of the list on the device (nList bounds it).
static void solveGlobal(xb_ctx* c, int si, const FitBuffers& f, const int* list, int nList,
                        const int* liveN, int other, bool cpuRhs, double* dSol) {
  const Geo& g = c->g;
  StampSetDev& S = c->set[si];
  const bool mixed = mixedMode(c);
  if(!mixed) {  // the mixed build forms its spatial weights itself
  const int2* kp = kernelPowers(c);
  const int nW = nList * g.nComp2;
  { KT_SCOPE(c, "weights");
  k_weights<<<(nW + 255) / 256, 256, 0, c->stream>>>(list, nList, liveN, S.count, S.cur, S.ssxy,
                                                    g.maxSS, kp, g.nComp2, c->w, c->h, f.wts);
  XB_LAUNCHED(c);
  }
  }
  const double* dots = mixed ? S.dots : f.dots;  // mixed: filled per stamp by the Gram kernel
  if(nList > 0 && !mixed) {
    if(g.nComp1 * g.nBG + g.nBG + g.nBG * g.nBG > DOT_PAIRS * DOT_THREADS)
      throw XbError{XB_ERR_UNSUPPORTED, "too many basis and background terms for the dot kernel"};
    const size_t smem = ((size_t)g.wRows * (DOT_KT + 1) + 2 * (size_t)g.wCols) * sizeof(double);
    const double* omega = c->p.fitWeighted ? S.omega : nullptr;
    { KT_SCOPE(c, "stamp_dots");
    if(c->imgIsF64)
      k_stamp_dots<double><<<nList, DOT_THREADS, smem, c->stream>>>(
          list, S.count, S.cur, S.ssxy, g.maxSS, (const double*)S.W, g.wRows, g.hSS, g.nPSF,
          g.nBG, (const double*)c->img[other], c->w, c->h, f.dots, f.stride, omega);
    else
      k_stamp_dots<float><<<nList, DOT_THREADS, smem, c->stream>>>(
          list, S.count, S.cur, S.ssxy, g.maxSS, (const double*)S.W, g.wRows, g.hSS, g.nPSF,
          g.nBG, (const float*)c->img[other], c->w, c->h, f.dots, f.stride, omega);
    XB_LAUNCHED(c);
    }
  }
  const int bgBase = g.nComp1 * g.nBG + g.nBG + g.nBG * g.nBG + (cpuRhs ? g.nBG : 0);
  const long long nTri = (long long)g.matSize * (g.matSize + 1) / 2;
  if(mixed) {
    buildSystemMixed(c, si, list, nList, bgBase, f.M, dSol, liveN);
  } else {
  { KT_SCOPE(c, "build_matrix");
  k_build_matrix<<<(int)std::min<long long>((nTri + 255) / 256, c->smCount * 8), 256, 0, c->stream>>>(
      list, nList, S.count, S.cur, S.Q, g.qCount, f.wts, dots, f.stride, mixed ? 1 : 0, g.nComp1,
      g.nComp2, g.nBG, g.matSize, f.M);
  XB_LAUNCHED(c);
  }
  { KT_SCOPE(c, "build_rhs");
  k_build_rhs<<<(g.nSol + 127) / 128, 128, 0, c->stream>>>(list, nList, S.count, S.cur, S.B,
                                                          g.qCount, f.wts, dots, f.stride,
                                                          mixed ? 1 : 0, bgBase, g.nComp1,
                                                          g.nComp2, g.nBG, g.nSol, dSol);
  XB_LAUNCHED(c);
  }
  }
  if(c->trace) {
    const int ld = g.matSize + 1;
    std::string key = cpuRhs ? "ksc_matrix" : ("cd_matrix" + std::to_string(si));
    if(!cpuRhs || !c->arrays.count("ksc_matrix0"))
      c->put(cpuRhs ? "ksc_matrix0" : key, toHost(c, f.M, (size_t)ld * ld));
  }
  // LU on a thread-block cluster
  const int n = g.matSize, ld = n + 1;
  k_zero_ints<<<1, 32, 0, c->stream>>>(f.singular, 1);
  XB_LAUNCHED(c);
  if(mixed) {
    globalSolveMixed(c, f.M, n, dSol, f.piv, f.singular);
    return;
  }
  // 8 CTAs, or 16 when 8 cannot hold the columns (the same products in the
  // same order either way)
  int maxSmem = 0;
  XB_CUDA(cudaDeviceGetAttribute(&maxSmem, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->device));
  auto luSmem = [&](int cl) {
    return ((size_t)((n + cl - 1) / cl) * ld + ld + 2 * (ld + 1) + ld) * sizeof(double);
  };
  const int CL = luSmem(8) <= (size_t)maxSmem ? 8 : 16;
  const size_t smem = luSmem(CL);
  auto luKernel = CL == 8 ? k_global_lu<8> : k_global_lu<16>;
  XB_CUDA(allowMaxDynamicSmem((const void*)luKernel, c->device));
  if(CL > 8) XB_CUDA(cudaFuncSetAttribute(luKernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
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
  { KT_SCOPE(c, "global_lu");
  XB_CUDA(cudaLaunchKernelEx(&cfg, luKernel, f.M, n, f.piv, f.singular));
  XB_LAUNCHED(c);
  }
  const size_t smemS = (size_t)(3 * (n + 1)) * sizeof(double) + (size_t)(n + 1) * sizeof(int);
  { KT_SCOPE(c, "global_lubksb");
  k_global_lubksb<<<1, LUB_THREADS, smemS, c->stream>>>(f.M, n, f.piv, dSol);
  XB_LAUNCHED(c);
  }
}

static void computeSigs(xb_ctx* c, int si, const int* dList, int nList, const double* dSol,
                        int convImg, double* dSig, const int* liveN = nullptr) {
  if(nList <= 0) return;
  if(mixedMode(c)) {
    sigsMixed(c, si, dList, nList, dSol, convImg, dSig, liveN);
    return;
  }
  const Geo& g = c->g;
  StampSetDev& S = c->set[si];
  const int pix = g.wCols, rc = (pix + 31) / 32;
  const size_t smem = ((size_t)g.nPSF + rc * 32 + rc) * sizeof(double) + (size_t)(rc * 32 + rc) * sizeof(int);
  const int other = 1 - convImg;
  { KT_SCOPE(c, "sigs");
  if(c->imgIsF64)
    k_sigs<double><<<nList, SIG_THREADS, smem, c->stream>>>(
        dList, S.count, S.cur, S.ssxy, g.maxSS, (const double*)S.W, g.wRows, g.hSS, g.nPSF,
        c->p.kernelOrder, c->p.backgroundOrder, g.nComp, dSol, (const double*)c->img[convImg],
        (const double*)c->img[other], c->mask, c->w, c->h, noiseInvGain(c->p),
        noiseRn2x2(c->p), dSig);
  else
    k_sigs<float><<<nList, SIG_THREADS, smem, c->stream>>>(
        dList, S.count, S.cur, S.ssxy, g.maxSS, (const double*)S.W, g.wRows, g.hSS, g.nPSF,
        c->p.kernelOrder, c->p.backgroundOrder, g.nComp, dSol, (const float*)c->img[convImg],
        (const float*)c->img[other], c->mask, c->w, c->h, noiseInvGain(c->p),
        noiseRn2x2(c->p), dSig);
  XB_LAUNCHED(c);
  }
}

void kernelSumLaunch(xb_ctx* c, const double* dSol, double xf, double yf, int tree, double* dOut) {
  { KT_SCOPE(c, "kernel_sum");
  k_kernel_sum<<<1, 256, 0, c->stream>>>(dSol, c->dVec, c->g.nPSF, c->p.kernelOrder, c->g.fK, xf, yf,
                                         tree, dOut);
  XB_LAUNCHED(c);
  }
}

// The mixed path's per-stamp test fits (k_stamp_test_fit_ldl), with the
// tuned number of warps (stamps) per CTA among those whose factors fit in
// shared memory (8 warps of a 61-row system do not); systems too large for
// two warps take the one-CTA-per-stamp LU of the plain path.
static void testFitLdl(xb_ctx* c, const StampSetDev& S, int qc, const int* liveN, double* ks) {
  int optin = 0;
  XB_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->device));
  const size_t perWarp = (size_t)(qc - 1) * qc * sizeof(double);
  if(2 * perWarp > (size_t)optin) {
    const size_t smemLU = ((size_t)qc * qc + 3 * qc) * sizeof(double) + qc * sizeof(int);
    if(smemLU > (size_t)optin) throw XbError{XB_ERR_UNSUPPORTED, "test fit: system too large"};
    XB_CUDA(allowMaxDynamicSmem((const void*)k_stamp_test_fit, c->device));
    k_stamp_test_fit<<<S.n, LU_THREADS, smemLU, c->stream>>>(S.Q, S.B, qc, liveN, ks);
    XB_LAUNCHED(c);
    return;
  }
  // variants: 0 = 4 warps, 1 = 2 warps, 2 = 8 warps
  const int nVar = 8 * perWarp <= (size_t)optin ? 3 : 2;
  auto launch = [&](int v) {
    if(v == 0 && 4 * perWarp > (size_t)optin) v = 1;
    const int W = v == 1 ? 2 : (v == 2 ? 8 : 4);
    const size_t smem = (size_t)W * (qc - 1) * qc * sizeof(double);
    const int grid = (S.n + W - 1) / W;
    if(W == 2) k_stamp_test_fit_ldl<2><<<grid, 64, smem, c->stream>>>(S.Q, S.B, qc, S.n, liveN, ks);
    else if(W == 8) k_stamp_test_fit_ldl<8><<<grid, 256, smem, c->stream>>>(S.Q, S.B, qc, S.n, liveN, ks);
    else k_stamp_test_fit_ldl<4><<<grid, 128, smem, c->stream>>>(S.Q, S.B, qc, S.n, liveN, ks);
    XB_LAUNCHED(c);
  };
  XB_CUDA(allowMaxDynamicSmem((const void*)k_stamp_test_fit_ldl<2>, c->device));
  XB_CUDA(allowMaxDynamicSmem((const void*)k_stamp_test_fit_ldl<4>, c->device));
  XB_CUDA(allowMaxDynamicSmem((const void*)k_stamp_test_fit_ldl<8>, c->device));
  launch(tunedVariant(c, "stamp_test_fit_ldl", (long long)qc, nVar, launch));
}

void stageCd(xb_ctx* c) {
  const Geo& g = c->g;
  const int nMax = std::max(std::max(c->set[0].n, c->set[1].n), 1);
  FitBuffers f = fitBuffers(c, nMax);
  double* ks[2] = {buf<double>(c, "cd_ks0", nMax), buf<double>(c, "cd_ks1", nMax)};
  int* testIdx[2] = {buf<int>(c, "cd_test0", nMax), buf<int>(c, "cd_test1", nMax)};
  int* nTest = buf<int>(c, "cd_ntest", 2);
  double* stats = buf<double>(c, "cd_stats", 4);
  double* dSolCd = buf<double>(c, "cd_sol", 2 * (size_t)std::max(g.nSol, g.matSize + 1));
  double* kMean = buf<double>(c, "cd_kmean", 2);
  double* merit = buf<double>(c, "cd_merit", 2);
  const int qc = g.qCount;
  const size_t smemLU = ((size_t)qc * qc + 3 * qc) * sizeof(double) + qc * sizeof(int);
  for(int si = 0; si < 2; si++) {
    StampSetDev& S = c->set[si];
    if(S.n > 0) {
      { KT_SCOPE(c, "stamp_test_fit");
      if(mixedMode(c)) {
        testFitLdl(c, S, qc, nullptr, ks[si]);
      } else {
        XB_CUDA(allowMaxDynamicSmem((const void*)k_stamp_test_fit, c->device));
        k_stamp_test_fit<<<S.n, LU_THREADS, smemLU, c->stream>>>(S.Q, S.B, qc, nullptr, ks[si]);
        XB_LAUNCHED(c);
      }
      }
    }
    { KT_SCOPE(c, "cd_select");
    k_cd_select<<<1, 256, 0, c->stream>>>(ks[si], S.n, nullptr, c->p.sigClipAlpha, c->p.sigKernFit,
                                          f.flags, f.cs, f.cs2, testIdx[si], nTest + si,
                                          stats + 2 * si);
    XB_LAUNCHED(c);
    }
  }
  std::vector<int> hT = toHost(c, nTest, 2);
  const int solStride = std::max(g.nSol, g.matSize + 1);
  for(int si = 0; si < 2; si++) {
    double* sol = dSolCd + (size_t)si * solStride;
    if(c->trace) c->put("kernel_sums" + std::to_string(si), toHost(c, ks[si], c->set[si].n));
    if(hT[si] == 0) {
      c->merit[si] = 666;
      continue;
    }
    solveGlobal(c, si, f, testIdx[si], hT[si], nullptr, 1 - si, false, sol);
    kernelSumLaunch(c, sol, (0 - 0.5 * c->w) / (0.5 * c->w), (0 - 0.5 * c->h) / (0.5 * c->h), 1,
                    kMean + si);
    computeSigs(c, si, testIdx[si], hT[si], sol, si, f.sig);
    { KT_SCOPE(c, "cd_merit");
    k_cd_merit<<<1, 256, 0, c->stream>>>(f.sig, hT[si], nullptr, kMean + si, c->p.sigClipAlpha,
                                         f.scratchD, f.flags, f.cs, f.cs2, merit + si);
    XB_LAUNCHED(c);
    }
    std::vector<double> m = toHost(c, merit + si, 1);
    c->merit[si] = m[0];
    if(c->trace) {
      const std::string sfx = std::to_string(si);
      c->put("cd_test" + sfx, toHost(c, testIdx[si], hT[si]));
      c->put("cd_solution" + sfx, toHost(c, sol, g.nSol));
      c->put("cd_sig" + sfx, toHost(c, f.sig, hT[si]));
      c->scalars["cd_kernel_mean" + sfx] = toHost(c, kMean + si, 1)[0];
    }
  }
  if(mixedMode(c)) checkSolveTimeout(c);
  c->convTemplate = c->merit[1] > c->merit[0] ? 1 : 0;
  c->chosen = c->convTemplate ? 0 : 1;
  c->scalars["merit0"] = c->merit[0];
  c->scalars["merit1"] = c->merit[1];
  c->scalars["convTemplate"] = c->convTemplate;
}

void stageKsc(xb_ctx* c) {
  const Geo& g = c->g;
  const int si = c->chosen;
  StampSetDev& S = c->set[si];
  const int n = S.n;
  FitBuffers f = fitBuffers(c, std::max(n, 1));
  std::vector<int> all(std::max(n, 1));
  for(int s = 0; s < n; s++) all[s] = s;
  int* allList = buf<int>(c, "ksc_all", std::max(n, 1));
  toDevice(c, allList, all);
  int* refill = buf<int>(c, "ksc_refill", std::max(n, 1));
  int* passOf = buf<int>(c, "ksc_passof", std::max(n, 1));
  int* outs = buf<int>(c, "ksc_out", 4);
  double* chi2 = buf<double>(c, "ksc_chi2", std::max(n, 1));
  c->dSol = buf<double>(c, "solution", std::max(g.nSol, g.matSize + 1));
  std::vector<int> rejects;
  int iteration = 0;
  long long refills = 0;  // substamps replaced over the loop
  bool check;
  do {
    solveGlobal(c, si, f, allList, n, nullptr, 1 - si, true, c->dSol);
    computeSigs(c, si, allList, n, c->dSol, si, f.sig);
    k_zero_ints<<<1, 32, 0, c->stream>>>(outs, 4);
    XB_LAUNCHED(c);
    { KT_SCOPE(c, "ksc_check");
    k_ksc_check<<<1, 256, 0, c->stream>>>(f.sig, n, nullptr, S.count, S.cur, c->p.sigClipAlpha,
                                          c->p.sigKernFit, chi2, f.flags, f.cs, f.cs2, refill,
                                          outs, passOf);
    XB_LAUNCHED(c);
    }
    std::vector<int> o = toHost(c, outs, 3);
    const int nRefill = o[0];
    refills += nRefill;
    check = nRefill > 0;
    if(c->trace && nRefill > 0) {
      std::vector<int> po = toHost(c, passOf, n);
      for(int pass = 0; pass < 2; pass++)
        for(int s = 0; s < n; s++)
          if(po[s] == pass) rejects.insert(rejects.end(), {iteration, pass, s});
    }
    if(nRefill > 0) fillStamps(c, si, refill, nRefill, si);
    if(c->trace && !check) c->put("ksc_sig_last", toHost(c, f.sig, n));
    iteration++;
    if(iteration > 4 * std::max(n, 1) * g.maxSS + 8)
      throw XbError{XB_ERR_STATE, "ksc did not converge"};  // cannot happen: indices only grow
  } while(check);
  c->kscIterations = iteration;
  c->hSol = toHost(c, c->dSol, g.nSol);
  c->singular = toHost(c, f.singular, 1)[0];
  if(mixedMode(c)) checkSolveTimeout(c);
  c->scalars["ksc_iterations"] = iteration;
  c->scalars["ksc_refills"] = (double)refills;
  c->scalars["singular"] = c->singular;
  if(c->trace) {
    c->put("ksc_rejects", rejects);
    c->put("cur", toHost(c, S.cur, n));
    c->put("solution", c->hSol);
  }
}

// cd as a frame graph captures it: the kept counts and the test-list
// lengths stay on the device (S.n is the stamp-grid bound, S.dN the count);
// each set's global test fit runs in a conditional node when its list is not
// empty, and its merit is 666 otherwise (cdkscUtil.cpp:234-265).
void stageCdGraph(xb_ctx* c, long long lCd[2]) {
  const Geo& g = c->g;
  const int nMax = std::max(std::max(c->set[0].n, c->set[1].n), 1);
  FitBuffers f = fitBuffers(c, nMax);
  double* ks[2] = {buf<double>(c, "cd_ks0", nMax), buf<double>(c, "cd_ks1", nMax)};
  int* testIdx[2] = {buf<int>(c, "cd_test0", nMax), buf<int>(c, "cd_test1", nMax)};
  int* nTest = buf<int>(c, "cd_ntest", 2);
  double* stats = buf<double>(c, "cd_stats", 4);
  double* dSolCd = buf<double>(c, "cd_sol", 2 * (size_t)std::max(g.nSol, g.matSize + 1));
  double* kMean = buf<double>(c, "cd_kmean", 2);
  double* merit = buf<double>(c, "cd_merit", 2);
  const int qc = g.qCount;
  const size_t smemLU = ((size_t)qc * qc + 3 * qc) * sizeof(double) + qc * sizeof(int);
  for(int si = 0; si < 2; si++) {
    StampSetDev& S = c->set[si];
    if(mixedMode(c)) {
      testFitLdl(c, S, qc, S.dN, ks[si]);
    } else {
      XB_CUDA(allowMaxDynamicSmem((const void*)k_stamp_test_fit, c->device));
      k_stamp_test_fit<<<S.n, LU_THREADS, smemLU, c->stream>>>(S.Q, S.B, qc, S.dN, ks[si]);
      XB_LAUNCHED(c);
    }
    k_cd_select<<<1, 256, 0, c->stream>>>(ks[si], S.n, S.dN, c->p.sigClipAlpha, c->p.sigKernFit,
                                          f.flags, f.cs, f.cs2, testIdx[si], nTest + si,
                                          stats + 2 * si);
    XB_LAUNCHED(c);
  }
  const int solStride = std::max(g.nSol, g.matSize + 1);
  for(int si = 0; si < 2; si++) {
    double* sol = dSolCd + (size_t)si * solStride;
    const int bound = c->set[si].n;
    graphSetDouble(c, merit + si, 666.0);
    lCd[si] = graphIfPositive(c, nTest + si, 1, [&] {
      solveGlobal(c, si, f, testIdx[si], bound, nTest + si, 1 - si, false, sol);
      kernelSumLaunch(c, sol, (0 - 0.5 * c->w) / (0.5 * c->w), (0 - 0.5 * c->h) / (0.5 * c->h), 1,
                      kMean + si);
      computeSigs(c, si, testIdx[si], bound, sol, si, f.sig, nTest + si);
      k_cd_merit<<<1, 256, 0, c->stream>>>(f.sig, bound, nTest + si, kMean + si,
                                           c->p.sigClipAlpha, f.scratchD, f.flags, f.cs, f.cs2,
                                           merit + si);
      XB_LAUNCHED(c);
    });
  }
}

// ksc as a frame graph captures it: the reject-and-refit loop is a WHILE
// node; each pass solves, checks, refills the rejected stamps (count on the
// device) and continues while refills were made.
long long stageKscGraph(xb_ctx* c) {
  const Geo& g = c->g;
  const int si = c->chosen;
  StampSetDev& S = c->set[si];
  const int n = std::max(S.n, 1);  // bound; the kept count is *S.dN
  FitBuffers f = fitBuffers(c, n);
  std::vector<int> all(n);
  for(int s = 0; s < n; s++) all[s] = s;
  int* allList = buf<int>(c, "ksc_all", n);
  toDevice(c, allList, all);
  int* refill = buf<int>(c, "ksc_refill", n);
  int* passOf = buf<int>(c, "ksc_passof", n);
  int* outs = buf<int>(c, "ksc_out", 4);
  double* chi2 = buf<double>(c, "ksc_chi2", n);
  c->dSol = buf<double>(c, "solution", std::max(g.nSol, g.matSize + 1));
  k_zero_ints<<<1, 32, 0, c->stream>>>(graphRec(c) + 2, 3);  // iterations, overflow, refills
  XB_LAUNCHED(c);
  const int limit = 4 * n * g.maxSS + 8;
  return graphWhile(c, [&](cudaGraphConditionalHandle h) {
    solveGlobal(c, si, f, allList, n, S.dN, 1 - si, true, c->dSol);
    computeSigs(c, si, allList, n, c->dSol, si, f.sig, S.dN);
    k_zero_ints<<<1, 32, 0, c->stream>>>(outs, 4);
    XB_LAUNCHED(c);
    k_ksc_check<<<1, 256, 0, c->stream>>>(f.sig, n, S.dN, S.count, S.cur, c->p.sigClipAlpha,
                                          c->p.sigKernFit, chi2, f.flags, f.cs, f.cs2, refill,
                                          outs, passOf);
    XB_LAUNCHED(c);
    fillStamps(c, si, refill, n, si, outs);
    graphKscContinue(c, h, outs, limit);
  });
}

}  // namespace xb
