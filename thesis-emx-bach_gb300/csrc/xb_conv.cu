// xb_conv.cu — conv + sub (src/bach.cpp:325-440): the spatially varying
// convolution of the chosen image, the output mask and the difference image
// in one pass over the frame.
//
// Reference structure: a host-built table of one 21x21 kernel per 21x21
// block (bachUtil.cpp:502-541, 34 MB of FP64 at 2048^2), createConvMask,
// conv (cl_kern/conv.cl:31-97), a read-back, maskAfterConv (:99-113) and sub
// (cl_kern/sub.cl:15-32).  Here each CTA owns one kernel block: it builds
// that block's kernel in shared memory (the same coefficient and basis sums
// as the reference's table), stages the image tile with its halo, and
// writes conv, the final mask and the difference for its pixels.  The
// frame border (hK pixels) is written by a separate streaming kernel.
//
// Plain mode: FP64 accumulation in the reference's tap order with fused
// multiply-adds for the pixel sums; the mask decisions (uks/aks) use plain
// additions in the reference order, so they match the oracle exactly.

#include <algorithm>

#include "xb_device.cuh"
#include "xb_internal.h"

namespace xb {

namespace {

constexpr int CONV_THREADS = 224;

__device__ __forceinline__ uint16_t convMaskOf(double t, double tH, double tL) {
  uint16_t m = 0;
  if(t == 0.0) m |= BAD_INPUT | BAD_PIX_VAL;
  if(t >= tH) m |= BAD_INPUT | SAT_PIXEL;
  if(t <= tL) m |= BAD_INPUT | LOW_PIXEL;
  return m;
}
__device__ __forceinline__ uint16_t afterMaskOf(double t, double tH, double tL) {
  uint16_t m = 0;
  if(t == 0.0) m |= BAD_OUTPUT | BAD_INPUT | BAD_PIX_VAL;
  if(t >= tH) m |= BAD_OUTPUT | BAD_INPUT | SAT_PIXEL;
  if(t <= tL) m |= BAD_OUTPUT | BAD_INPUT | LOW_PIXEL;
  return m;
}

struct ConvArgs {
  int w, h, hK, fK, xSteps, nPSF, kOrder, bgOrder, nComp, scaleConv;
  double tH, tL;
};

template <class T>
__global__ void __launch_bounds__(CONV_THREADS)
    k_conv_sub_f64(const T* __restrict__ I, const T* __restrict__ O,
                   const double* __restrict__ sol, const double* __restrict__ vec,
                   const double* __restrict__ kernSumPtr, ConvArgs a,
                   const uint8_t* __restrict__ inMask, uint16_t* __restrict__ mask,
                   double* __restrict__ convD, float* __restrict__ convF,
                   double* __restrict__ diffD, float* __restrict__ diffF) {
  extern __shared__ double cv_s[];
  const int fK = a.fK, hK = a.hK, nk = fK * fK, tw = fK + 2 * hK;
  double* kern = cv_s;                       // nk
  double* tile = kern + nk;                  // tw * tw
  double* coeff = tile + tw * tw;            // nPSF
  uint8_t* bad = (uint8_t*)(coeff + a.nPSF); // tw * tw
  __shared__ double sAks;
  const int xS = blockIdx.x, yS = blockIdx.y, tid = threadIdx.x;
  // kernel of this block at its centre (conv(), src/bach.cpp:339-350)
  {
    const int kx = xS * fK + 2 * hK, ky = yS * fK + 2 * hK;
    const double hx = 0.5 * a.w, hy = 0.5 * a.h;
    const double xf = (kx - hx) / hx, yf = (ky - hy) / hy;
    const int nC2 = (a.kOrder + 1) * (a.kOrder + 2) / 2;
    for(int i = tid; i < a.nPSF; i += CONV_THREADS) {
      double c = 0.0;
      if(i == 0) {
        c = sol[1];
      } else {
        int k = 2 + (i - 1) * nC2;
        double aX = 1.0;
        for(int x = 0; x <= a.kOrder; x++) {
          double aY = 1.0;
          for(int y = 0; y <= a.kOrder - x; y++) {
            c += sol[k++] * aX * aY;
            aY *= yf;
          }
          aX *= xf;
        }
      }
      coeff[i] = c;
    }
  }
  const int x0 = xS * fK, y0 = yS * fK;  // tile origin (block pixels start at +hK)
  for(int i = tid; i < tw * tw; i += CONV_THREADS) {
    int lx = i % tw, ly = i / tw;
    int gx = min(x0 + lx, a.w - 1), gy = min(y0 + ly, a.h - 1);
    double v = (double)I[(size_t)gx + (size_t)gy * a.w];
    tile[i] = v;
    bad[i] = ((convMaskOf(v, a.tH, a.tL) & BAD_INPUT) ||
              (inMask && inMask[(size_t)gx + (size_t)gy * a.w])) ? 1 : 0;
  }
  __syncthreads();
  for(int p = tid; p < nk; p += CONV_THREADS) {
    double k0 = 0.0;
    for(int q = 0; q < a.nPSF; q++) k0 += coeff[q] * vec[(size_t)q * nk + p];
    kern[p] = k0;
  }
  __syncthreads();
  if(tid == 0) {
    // aks: |kernel| summed in the tap order of conv.cl:54-70 (j, i ascending)
    double s = 0.0;
    for(int jk = 2 * hK; jk >= 0; jk--)
      for(int ik = 2 * hK; ik >= 0; ik--) s += fabs(kern[ik + jk * fK]);
    sAks = s;
  }
  __syncthreads();
  const double aks = sAks;
  const double kernSum = *kernSumPtr;
  const double invKernMult = a.scaleConv ? 1.0 / kernSum : 1.0;
  const double convFactor = a.scaleConv ? kernSum : 1.0;
  const double finalFactor = a.scaleConv ? -(1.0 / kernSum) : 1.0;
  for(int p = tid; p < nk; p += CONV_THREADS) {
    const int lx = p % fK, ly = p / fK;
    const int x = x0 + hK + lx, y = y0 + hK + ly;
    if(x >= a.w - hK || y >= a.h - hK) continue;
    double acc = 0.0;
    int anyBad = 0;
    for(int jj = 0; jj < fK; jj++) {
      const double* trow = tile + (ly + jj) * tw + lx;
      const uint8_t* brow = bad + (ly + jj) * tw + lx;
      const double* krow = kern + (2 * hK - jj) * fK;
#pragma unroll 7
      for(int ii = 0; ii < fK; ii++) {
        acc = fma(krow[2 * hK - ii], trow[ii], acc);
        anyBad |= brow[ii];
      }
    }
    // background polynomial (getBackground, cd.cl:444-467)
    {
      const double bxf = (x - 0.5 * a.w) / (0.5 * a.w), byf = (y - 0.5 * a.h) / (0.5 * a.h);
      double bg = 0.0, ax = 1.0;
      int k = a.nComp + 2;
      for(int i = 0; i <= a.bgOrder; i++) {
        double ay = 1.0;
        for(int j = 0; j <= a.bgOrder - i; j++) {
          bg += sol[k++] * ax * ay;
          ay *= byf;
        }
        ax *= bxf;
      }
      acc += bg;
    }
    acc *= invKernMult;
    const size_t id = (size_t)x + (size_t)y * a.w;
    const double tc = tile[(ly + hK) * tw + lx + hK];
    uint16_t cm = convMaskOf(tc, a.tH, a.tL);
    if(inMask && inMask[id]) cm |= INPUT_MASK | BAD_INPUT;
    uint16_t nm = cm;
    if(cm & BAD_INPUT) nm |= BAD_OUTPUT;
    if(anyBad) {
      double uks = 0.0;
      for(int jj = 0; jj < fK; jj++)
        for(int ii = 0; ii < fK; ii++)
          if(!bad[(ly + jj) * tw + lx + ii]) uks += fabs(kern[(2 * hK - ii) + (2 * hK - jj) * fK]);
      if((uks / aks) < (double)0.99f) nm |= BAD_OUTPUT | BAD_CONV;
      else nm |= OK_CONV;
    }
    const double o = (double)O[id];
    nm |= afterMaskOf(o, a.tH, a.tL);
    mask[id] = nm;
    convD[id] = acc;
    convF[id] = (float)acc;
    const double d = (nm & BAD_OUTPUT) ? 1e-30 : (acc * convFactor - o) * finalFactor;
    diffD[id] = d;
    diffF[id] = (float)d;
  }
}

// Border pixels: conv = diff = 1e-30 (conv.cl:95, sub.cl:24); the mask
// keeps its value plus maskAfterConv's bits.
// Per-pixel kernel (option convPerPixel; no counterpart in the reference,
// whose conv.cl evaluates the kernel once per fK x fK block at the block
// centre).  The kernel at output pixel (x, y) is sum_t P_t(x, y) Kt[t] with
// P_t = xf^i yf^j of the pixel itself, so the convolved value is
// sum_t P_t (Kt[t] * I)(x, y): nComp2 convolutions per pixel, each summed in
// the block kernel's tap order, then combined in t order.  Pixels whose
// window holds a bad input evaluate the kernel tap by tap for the
// 0.99 |kernel| rule (conv.cl:70-100).
template <class T>
__global__ void __launch_bounds__(CONV_THREADS)
    k_conv_sub_pp_f64(const T* __restrict__ I, const T* __restrict__ O,
                      const double* __restrict__ sol, const double* __restrict__ Kt,
                      const double* __restrict__ kernSumPtr, ConvArgs a,
                      const uint8_t* __restrict__ inMask, uint16_t* __restrict__ mask,
                      double* __restrict__ convD, float* __restrict__ convF,
                      double* __restrict__ diffD, float* __restrict__ diffF) {
  extern __shared__ double cv_s[];
  const int fK = a.fK, hK = a.hK, nk = fK * fK, tw = fK + 2 * hK;
  const int nC2 = (a.kOrder + 1) * (a.kOrder + 2) / 2;
  double* kt = cv_s;                         // nC2 * nk
  double* tile = kt + nC2 * nk;              // tw * tw
  uint8_t* bad = (uint8_t*)(tile + tw * tw); // tw * tw
  const int xS = blockIdx.x, yS = blockIdx.y, tid = threadIdx.x;
  for(int i = tid; i < nC2 * nk; i += CONV_THREADS) kt[i] = Kt[i];
  const int x0 = xS * fK, y0 = yS * fK;
  for(int i = tid; i < tw * tw; i += CONV_THREADS) {
    int lx = i % tw, ly = i / tw;
    int gx = min(x0 + lx, a.w - 1), gy = min(y0 + ly, a.h - 1);
    double v = (double)I[(size_t)gx + (size_t)gy * a.w];
    tile[i] = v;
    bad[i] = ((convMaskOf(v, a.tH, a.tL) & BAD_INPUT) ||
              (inMask && inMask[(size_t)gx + (size_t)gy * a.w])) ? 1 : 0;
  }
  __syncthreads();
  const double kernSum = *kernSumPtr;
  const double invKernMult = a.scaleConv ? 1.0 / kernSum : 1.0;
  const double convFactor = a.scaleConv ? kernSum : 1.0;
  const double finalFactor = a.scaleConv ? -(1.0 / kernSum) : 1.0;
  const double hx = 0.5 * a.w, hy = 0.5 * a.h;
  for(int p = tid; p < nk; p += CONV_THREADS) {
    const int lx = p % fK, ly = p / fK;
    const int x = x0 + hK + lx, y = y0 + hK + ly;
    if(x >= a.w - hK || y >= a.h - hK) continue;
    // spatial monomials of this pixel, x power outer (makeKernelCoeffs order)
    double P[(MAX_KORDER + 1) * (MAX_KORDER + 2) / 2];
    {
      const double xf = (x - hx) / hx, yf = (y - hy) / hy;
      double ax = 1.0;
      int t = 0;
      for(int i = 0; i <= a.kOrder; i++) {
        double ay = 1.0;
        for(int j = 0; j <= a.kOrder - i; j++) {
          P[t++] = ax * ay;
          ay *= yf;
        }
        ax *= xf;
      }
    }
    double acc = 0.0;
    int anyBad = 0;
    for(int t = 0; t < nC2; t++) {
      const double* kk = kt + t * nk;
      double ct = 0.0;
      for(int jj = 0; jj < fK; jj++) {
        const double* trow = tile + (ly + jj) * tw + lx;
        const double* krow = kk + (2 * hK - jj) * fK;
#pragma unroll 7
        for(int ii = 0; ii < fK; ii++) ct = fma(krow[2 * hK - ii], trow[ii], ct);
      }
      acc = fma(P[t], ct, acc);
    }
    for(int jj = 0; jj < fK && !anyBad; jj++) {
      const uint8_t* brow = bad + (ly + jj) * tw + lx;
      for(int ii = 0; ii < fK; ii++) anyBad |= brow[ii];
    }
    // background polynomial (getBackground, cd.cl:444-467)
    {
      const double bxf = (x - 0.5 * a.w) / (0.5 * a.w), byf = (y - 0.5 * a.h) / (0.5 * a.h);
      double bg = 0.0, ax = 1.0;
      int k = a.nComp + 2;
      for(int i = 0; i <= a.bgOrder; i++) {
        double ay = 1.0;
        for(int j = 0; j <= a.bgOrder - i; j++) {
          bg += sol[k++] * ax * ay;
          ay *= byf;
        }
        ax *= bxf;
      }
      acc += bg;
    }
    acc *= invKernMult;
    const size_t id = (size_t)x + (size_t)y * a.w;
    const double tc = tile[(ly + hK) * tw + lx + hK];
    uint16_t cm = convMaskOf(tc, a.tH, a.tL);
    if(inMask && inMask[id]) cm |= INPUT_MASK | BAD_INPUT;
    uint16_t nm = cm;
    if(cm & BAD_INPUT) nm |= BAD_OUTPUT;
    if(anyBad) {
      // this pixel's kernel, tap by tap in window order
      double aks = 0.0, uks = 0.0;
      for(int jj = 0; jj < fK; jj++)
        for(int ii = 0; ii < fK; ii++) {
          const int tap = (2 * hK - ii) + (2 * hK - jj) * fK;
          double kv = 0.0;
          for(int t = 0; t < nC2; t++) kv = fma(P[t], kt[t * nk + tap], kv);
          aks += fabs(kv);
          if(!bad[(ly + jj) * tw + lx + ii]) uks += fabs(kv);
        }
      if((uks / aks) < (double)0.99f) nm |= BAD_OUTPUT | BAD_CONV;
      else nm |= OK_CONV;
    }
    const double o = (double)O[id];
    nm |= afterMaskOf(o, a.tH, a.tL);
    mask[id] = nm;
    convD[id] = acc;
    convF[id] = (float)acc;
    const double d = (nm & BAD_OUTPUT) ? 1e-30 : (acc * convFactor - o) * finalFactor;
    diffD[id] = d;
    diffF[id] = (float)d;
  }
}

template <class T>
__global__ void k_border(const T* __restrict__ O, int w, int h, int hK, double tH, double tL,
                         const uint8_t* __restrict__ inMask, uint16_t* __restrict__ mask,
                         double* __restrict__ convD,
                         float* __restrict__ convF, double* __restrict__ diffD,
                         float* __restrict__ diffF) {
  const long long n = (long long)w * h;
  for(long long id = (long long)blockIdx.x * blockDim.x + threadIdx.x; id < n;
      id += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(id % w), y = (int)(id / w);
    if(x >= hK && x < w - hK && y >= hK && y < h - hK) continue;
    mask[id] |= afterMaskOf((double)O[id], tH, tL);
    if(inMask && inMask[id]) mask[id] |= INPUT_MASK | BAD_INPUT | BAD_OUTPUT;
    convD[id] = 1e-30;
    convF[id] = (float)1e-30;
    diffD[id] = 1e-30;
    diffF[id] = (float)1e-30;
  }
}

}  // namespace

void stageConvSub(xb_ctx* c, bool doSub) {
  if(doSub) return;  // the difference is written by the fused conv pass
  const Geo& g = c->g;
  const size_t n = (size_t)c->w * c->h;
  c->convF = buf<float>(c, "convF", n);
  c->diffF = buf<float>(c, "diffF", n);
  double* ks = buf<double>(c, "kernSum", 1);
  // kernel sum at the frame centre, sequential sum (bachUtil.cpp:532-538)
  {
    const double hx = 0.5 * c->w, hy = 0.5 * c->h;
    const double xf = (c->w / 2 - hx) / hx, yf = (c->h / 2 - hy) / hy;
    kernelSumLaunch(c, c->dSol, xf, yf, 0, ks);
  }
  // the FP32 conv tile is built for 21-px kernels; mixed frames with another
  // kernel width take the FP64 block conv below
  if(mixedMode(c) && g.fK == 21) {
    c->convD = nullptr;
    c->diffD = nullptr;
    convSubMixed(c, ks);
    if(c->capturing) return;  // a frame graph records the kernel sum on the device
    c->kernSum = toHost(c, ks, 1)[0];
    c->scalars["kernSum"] = c->kernSum;
    if(c->trace) {
      std::vector<float> cf = toHost(c, c->convF, n), df = toHost(c, c->diffF, n);
      c->put("conv", std::vector<double>(cf.begin(), cf.end()));
      c->put("diff", std::vector<double>(df.begin(), df.end()));
      c->put("mask", toHost(c, c->mask, n));
    }
    return;
  }
  c->convD = buf<double>(c, "convD", n);
  c->diffD = buf<double>(c, "diffD", n);
  ConvArgs a{};
  a.w = c->w;
  a.h = c->h;
  a.hK = g.hK;
  a.fK = g.fK;
  a.xSteps = (c->w + g.fK - 1) / g.fK;
  a.nPSF = g.nPSF;
  a.kOrder = c->p.kernelOrder;
  a.bgOrder = c->p.backgroundOrder;
  a.nComp = g.nComp;
  a.scaleConv = (c->p.normalizeTemplate && c->convTemplate) || (!c->p.normalizeTemplate && !c->convTemplate);
  a.tH = c->p.threshHigh;
  a.tL = c->p.threshLow;
  const int ySteps = (c->h + g.fK - 1) / g.fK;
  const int tw = g.fK + 2 * g.hK;
  const size_t smem = ((size_t)g.fK * g.fK + (size_t)tw * tw + g.nPSF) * sizeof(double) + (size_t)tw * tw;
  const int I = c->chosen, O = 1 - c->chosen;
  dim3 grid(a.xSteps, ySteps);
  if(c->p.convPerPixel) {
    const double* Kt = kernelTermsLaunch(c);
    const size_t smemPP = ((size_t)g.nComp2 * g.fK * g.fK + (size_t)tw * tw) * sizeof(double) +
                          (size_t)tw * tw;
    int optin = 0;
    XB_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->device));
    if(c->p.kernelOrder > MAX_KORDER || smemPP > (size_t)optin)
      throw XbError{XB_ERR_UNSUPPORTED, "per-pixel kernel: kernel order or width too large"};
    XB_CUDA(allowMaxDynamicSmem((const void*)k_conv_sub_pp_f64<double>, c->device));
    XB_CUDA(allowMaxDynamicSmem((const void*)k_conv_sub_pp_f64<float>, c->device));
    KT_SCOPE(c, "conv_sub");
    if(c->imgIsF64)
      k_conv_sub_pp_f64<double><<<grid, CONV_THREADS, smemPP, c->stream>>>(
          (const double*)c->img[I], (const double*)c->img[O], c->dSol, Kt, ks, a, c->inputMask,
          c->mask, c->convD, c->convF, c->diffD, c->diffF);
    else
      k_conv_sub_pp_f64<float><<<grid, CONV_THREADS, smemPP, c->stream>>>(
          (const float*)c->img[I], (const float*)c->img[O], c->dSol, Kt, ks, a, c->inputMask,
          c->mask, c->convD, c->convF, c->diffD, c->diffF);
    XB_LAUNCHED(c);
  }
  if(c->p.convPerPixel) {
    const int blocks = (int)std::min<long long>((n + 255) / 256, c->smCount * 8);
    if(c->imgIsF64)
      k_border<double><<<blocks, 256, 0, c->stream>>>(
          (const double*)c->img[O], c->w, c->h, g.hK, a.tH, a.tL, c->inputMask, c->mask, c->convD,
          c->convF, c->diffD, c->diffF);
    else
      k_border<float><<<blocks, 256, 0, c->stream>>>(
          (const float*)c->img[O], c->w, c->h, g.hK, a.tH, a.tL, c->inputMask, c->mask, c->convD,
          c->convF, c->diffD, c->diffF);
  } else if(c->imgIsF64) {
    { KT_SCOPE(c, "conv_sub");
    k_conv_sub_f64<double><<<grid, CONV_THREADS, smem, c->stream>>>(
        (const double*)c->img[I], (const double*)c->img[O], c->dSol, c->dVec, ks, a, c->inputMask,
        c->mask, c->convD, c->convF, c->diffD, c->diffF);
    XB_LAUNCHED(c);
    }
    k_border<double><<<std::min<long long>((n + 255) / 256, c->smCount * 8), 256, 0, c->stream>>>(
        (const double*)c->img[O], c->w, c->h, g.hK, a.tH, a.tL, c->inputMask, c->mask, c->convD, c->convF,
        c->diffD, c->diffF);
  } else {
    { KT_SCOPE(c, "conv_sub");
    k_conv_sub_f64<float><<<grid, CONV_THREADS, smem, c->stream>>>(
        (const float*)c->img[I], (const float*)c->img[O], c->dSol, c->dVec, ks, a, c->inputMask,
        c->mask, c->convD, c->convF, c->diffD, c->diffF);
    XB_LAUNCHED(c);
    }
    k_border<float><<<std::min<long long>((n + 255) / 256, c->smCount * 8), 256, 0, c->stream>>>(
        (const float*)c->img[O], c->w, c->h, g.hK, a.tH, a.tL, c->inputMask, c->mask, c->convD, c->convF,
        c->diffD, c->diffF);
  }
  XB_LAUNCHED(c);
  if(c->capturing) return;  // a frame graph records the kernel sum on the device
  c->kernSum = toHost(c, ks, 1)[0];
  c->scalars["kernSum"] = c->kernSum;
  if(c->trace) {
    c->put("conv", toHost(c, c->convD, n));
    c->put("diff", toHost(c, c->diffD, n));
    c->put("mask", toHost(c, c->mask, n));
  }
}

}  // namespace xb
