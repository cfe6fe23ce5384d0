// xb_device.cuh — device helpers shared by the stage kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace xb {

// Block-wide exclusive scan of one int per thread; *total receives the sum.
// Every thread of the block must call it.
__device__ __forceinline__ int blockScanExcl(int v, int* warpTot, int* total) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int x = v;
#pragma unroll
  for(int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, x, o);
    if(lane >= o) x += y;
  }
  if(lane == 31) warpTot[wid] = x;
  __syncthreads();
  if(threadIdx.x == 0) {
    int s = 0;
    for(int i = 0; i < (int)(blockDim.x >> 5); i++) {
      int t = warpTot[i];
      warpTot[i] = s;
      s += t;
    }
    *total = s;
  }
  __syncthreads();
  int r = warpTot[wid] + x - v;
  __syncthreads();
  return r;
}

// (x - (w * 0.5f)) / (w * 0.5f) evaluated in float, as cl_kern/cmv.cl:180 and
// cl_kern/cd.cl:170 write it (an int times a float literal is float).
__device__ __forceinline__ double floatNormD(int x, int w) {
  float hw = (float)w * 0.5f;
  float r = ((float)x - hw) / hw;
  return (double)r;
}

// OpenCL pown(x, n) as the repeated product 1*x*x*...
__device__ __forceinline__ double ipowD(double x, int n) {
  double r = 1.0;
  for(int i = 0; i < n; i++) r *= x;
  return r;
}

// OR `bits` into the 16-bit mask entry i with a 32-bit atomic on its
// aligned word (the mask buffer carries two spare entries at the end).
__device__ __forceinline__ void maskOr(uint16_t* m, size_t i, uint16_t bits) {
  uintptr_t a = (uintptr_t)(m + i);
  unsigned* w32 = (unsigned*)(a & ~(uintptr_t)3);
  unsigned sh = (a & 2) ? 16u : 0u;
  atomicOr(w32, (unsigned)bits << sh);
}

// sigmaClip of src/bachUtil.cpp:34-128 for one CTA: data[0..n) in global
// memory, sums in 32-element chunks (sequential inside a chunk,
// cl_kern/bach.cl:135-170) added sequentially (bachUtil.cpp:103-104); the
// clipped flags live in `flags` (n bytes), chunk sums in cs/cs2.  The result
// is written to *outMean / *outStd (shared) by thread 0; all threads must
// call it.
__device__ inline void blockSigmaClip(const double* data, int n, int maxIter, double alpha,
                                      uint8_t* flags, double* cs, double* cs2,
                                      double* outMean, double* outStd, int* sh) {
  // sh[0] = prev, sh[1] = curr, sh[2] = clip, sh[3] = stop
  const int tid = threadIdx.x, nt = blockDim.x;
  __shared__ double sInv;
  for(int k = tid; k < n; k += nt) flags[k] = 0;
  if(tid == 0) {
    sh[0] = n;
    sh[1] = 0;
    sh[3] = 0;
    *outMean = 0.0;
    *outStd = 1e10;
    if(n == 0) sh[3] = 1;
  }
  __syncthreads();
  const int nChunks = (n + 31) / 32;
  for(int it = 0; it < maxIter; it++) {
    if(sh[3] || sh[1] == sh[0]) break;
    if(sh[0] <= 1) {
      __syncthreads();
      if(tid == 0) {
        *outMean = 0.0;
        *outStd = 1e10;
      }
      break;
    }
    __syncthreads();
    if(tid == 0) sh[1] = sh[0];
    for(int c = tid; c < nChunks; c += nt) {
      double a = 0.0, a2 = 0.0;
      int lc = min(32, n - c * 32);
      for(int l = 0; l < lc; l++) {
        int k = c * 32 + l;
        double d = flags[k] == 0 ? data[k] : 0.0;
        a += d;
        a2 += d * d;
      }
      cs[c] = a;
      cs2[c] = a2;
    }
    __syncthreads();
    if(tid == 0) {
      double sum = 0.0, sum2 = 0.0;
      for(int c = 0; c < nChunks; c++) {
        sum += cs[c];
        sum2 += cs2[c];
      }
      double nn = (double)sh[1];
      double m = sum / nn;
      double sd = sqrt((sum2 - nn * m * m) / (double)(sh[1] - 1));
      *outMean = m;
      *outStd = sd;
      sInv = 1.0 / sd;
      sh[2] = 0;
    }
    __syncthreads();
    const double m = *outMean, inv = sInv;
    int myClip = 0;
    for(int k = tid; k < n; k += nt)
      if(flags[k] == 0 && fabs(data[k] - m) * inv > alpha) {
        flags[k] = 1;
        myClip++;
      }
    if(myClip) atomicAdd(&sh[2], myClip);
    __syncthreads();
    if(tid == 0) sh[0] = sh[1] - sh[2];
    __syncthreads();
  }
  __syncthreads();
}

}  // namespace xb
