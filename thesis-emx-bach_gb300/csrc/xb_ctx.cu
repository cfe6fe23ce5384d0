// xb_ctx.cu — context lifetime, basis tables and the init stage.
//
// init (src/bach.cpp:14-42): the images are uploaded once and the mask is
// built by two streaming kernels, maskInput (cl_kern/ini.cl:15-35) and
// spreadMask (cl_kern/ini.cl:37-67).

#include <algorithm>
#include <cmath>
#include <cstring>

#include <mutex>
#include <set>
#include <utility>

#include "xb_internal.h"

namespace xb {

Geo makeGeo(const xb_params& p) {
  Geo g{};
  g.hSS = p.hSStampWidth;
  g.fSS = 2 * g.hSS + 1;
  g.hK = p.hKernelWidth;
  g.fK = 2 * g.hK + 1;
  g.nPSF = xb_params_npsf(&p);
  g.nComp1 = g.nPSF - 1;
  g.nComp2 = triNum(p.kernelOrder + 1);
  g.nComp = g.nComp1 * g.nComp2;
  g.nBG = triNum(p.backgroundOrder + 1);
  g.matSize = g.nComp + g.nBG + 1;
  g.nSol = g.nPSF * g.nComp2 + g.nBG + 1;
  g.wRows = g.nPSF + g.nBG;
  g.wCols = g.fSS * g.fSS;
  g.qCount = g.nPSF + 2;
  g.bCount = g.nPSF + 2;
  g.maxSS = 2 * p.maxKSStamps;
  return g;
}

// pown(x, n) of the OpenCL kernels, evaluated as 1*x*x*... (the form the
// host loops of src/cdkscUtil.cpp:334-342 use).
static double ipowHost(double x, int n) {
  double r = 1.0;
  for(int i = 0; i < n; i++) r *= x;
  return r;
}

Basis buildBasis(const xb_params& p, const Geo& g) {
  Basis b;
  const int fK = g.fK, hK = g.hK;
  // enumeration order of src/bach.cpp:181-188: Gaussian, x degree, y degree
  for(int gs = 0; gs < p.nGauss; gs++)
    for(int x = 0; x <= p.dg[gs]; x++)
      for(int y = 0; y <= p.dg[gs] - x; y++) {
        b.gauss.push_back(gs);
        b.kx.push_back(x);
        b.ky.push_back(y);
      }
  const int nPSF = (int)b.kx.size();
  b.fX.assign((size_t)nPSF * fK, 0.0);
  b.fY.assign((size_t)nPSF * fK, 0.0);
  for(int n = 0; n < nPSF; n++) {
    const double bw = (double)p.bg[b.gauss[n]];  // float width, as the reference
    double sx = 0.0, sy = 0.0;
    for(int i = 0; i < fK; i++) {
      const double x = (double)(i - hK);
      const double qe = std::exp(-x * x * bw);
      const double fx = qe * ipowHost(x, b.kx[n]);
      const double fy = qe * ipowHost(x, b.ky[n]);
      b.fX[(size_t)n * fK + i] = fx;
      b.fY[(size_t)n * fK + i] = fy;
      sx += fx;
      sy += fy;
    }
    if(b.kx[n] % 2 == 0 && b.ky[n] % 2 == 0) {  // normalise even/even filters
      const double ix = 1.0 / sx, iy = 1.0 / sy;
      for(int i = 0; i < fK; i++) {
        b.fX[(size_t)n * fK + i] *= ix;
        b.fY[(size_t)n * fK + i] *= iy;
      }
    }
  }
  b.vec.assign((size_t)nPSF * fK * fK, 0.0);
  for(int n = 0; n < nPSF; n++)
    for(int v = 0; v < fK; v++)
      for(int u = 0; u < fK; u++) {
        double vv = b.fX[(size_t)n * fK + u] * b.fY[(size_t)n * fK + v];
        if(b.kx[n] % 2 == 0 && b.ky[n] % 2 == 0 && n > 0) vv -= b.fX[u] * b.fY[v];
        b.vec[(size_t)n * fK * fK + (size_t)v * fK + u] = vv;
      }
  for(int x = 0; x <= p.backgroundOrder; x++)
    for(int y = 0; y <= p.backgroundOrder - x; y++) {
      b.bgX.push_back(x);
      b.bgY.push_back(y);
    }
  for(int i = 0; i <= p.kernelOrder; i++)
    for(int j = 0; j <= p.kernelOrder - i; j++) {
      b.kpX.push_back(i);
      b.kpY.push_back(j);
    }
  // Group basis functions whose Y filters are bit-identical: the Y pass of
  // the substamp convolution (cl_kern/cmv.cl:70-106) depends only on the Y
  // filter, so one pass serves the whole group with identical results.
  std::vector<int> groupOf(nPSF, -1);
  std::vector<std::vector<int>> groups;
  for(int n = 0; n < nPSF; n++) {
    for(size_t gi = 0; gi < groups.size(); gi++) {
      int m = groups[gi][0];
      if(memcmp(&b.fY[(size_t)m * fK], &b.fY[(size_t)n * fK], sizeof(double) * fK) == 0) {
        groupOf[n] = (int)gi;
        groups[gi].push_back(n);
        break;
      }
    }
    if(groupOf[n] < 0) {
      groupOf[n] = (int)groups.size();
      groups.push_back({n});
    }
  }
  b.yGroupStart.push_back(0);
  for(auto& gr : groups) {
    for(int n : gr) b.yGroupMembers.push_back(n);
    b.yGroupStart.push_back((int)b.yGroupMembers.size());
  }
  return b;
}

cudaError_t allowMaxDynamicSmem(const void* func, int device) {
  // once per (function, device): the attribute outlives the call
  static std::mutex mu;
  static std::set<std::pair<const void*, int>> done;
  {
    std::lock_guard<std::mutex> l(mu);
    if(done.count({func, device})) return cudaSuccess;
  }
  int optin = 0;
  cudaError_t e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
  if(e != cudaSuccess) return e;
  cudaFuncAttributes fa;
  e = cudaFuncGetAttributes(&fa, func);
  if(e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           optin - (int)fa.sharedSizeBytes);
  if(e == cudaSuccess) {
    std::lock_guard<std::mutex> l(mu);
    done.insert({func, device});
  }
  return e;
}

void* poolGet(xb_ctx* c, const char* name, size_t bytes) {
  DevBuf& b = c->pool[name];
  if(b.bytes >= bytes) return b.p;
  if(b.p) {
    if(c->keepBuffers) {
      // a captured frame graph may still address it: freed with the context
      c->retired.push_back(b.p);
    } else {
      XB_CUDA(cudaStreamSynchronize(c->stream));
      cudaFree(b.p);
    }
    b.p = nullptr;
    b.bytes = 0;
  }
  void* p = nullptr;
  if(cudaMalloc(&p, bytes) != cudaSuccess) {
    cudaGetLastError();
    throw XbError{XB_ERR_NOMEM, std::string("cudaMalloc failed for ") + name};
  }
  b.p = p;
  b.bytes = bytes;
  return p;
}

cudaEvent_t ktEvent(xb_ctx* c) {
  if(!c->kt.pool.empty()) {
    cudaEvent_t e = c->kt.pool.back();
    c->kt.pool.pop_back();
    return e;
  }
  cudaEvent_t e;
  XB_CUDA(cudaEventCreate(&e));
  return e;
}

void ktCollect(xb_ctx* c) {
  if(c->kt.pending.empty()) return;
  XB_CUDA(cudaStreamSynchronize(c->stream));
  for(auto& o : c->kt.pending) {
    float ms = 0.f;
    XB_CUDA(cudaEventElapsedTime(&ms, o.a, o.b));
    auto& t = c->kt.total[o.name];
    t.first += ms;
    t.second += 1;
    c->kt.pool.push_back(o.a);
    c->kt.pool.push_back(o.b);
  }
  c->kt.pending.clear();
}

// ---------------------------------------------------------------- kernels --

// maskInput (cl_kern/ini.cl:15-35).  Four pixels per thread.
template <class T>
__global__ void __launch_bounds__(256) k_mask_input(const T* __restrict__ tImg,
                                                    const T* __restrict__ sImg,
                                                    uint16_t* __restrict__ mask,
                                                    int w, int h, int border,
                                                    double tH, double tL) {
  const long long n = (long long)w * h;
  for(long long base = ((long long)blockIdx.x * blockDim.x + threadIdx.x) * 4; base < n;
      base += (long long)gridDim.x * blockDim.x * 4) {
#pragma unroll
    for(int k = 0; k < 4; k++) {
      long long id = base + k;
      if(id >= n) break;
      const int x = (int)(id % w), y = (int)(id / w);
      const double t = (double)tImg[id], s = (double)sImg[id];
      uint16_t m = 0;
      if(t == 0.0 || s == 0.0) m |= BAD_INPUT | BAD_PIX_VAL;
      if(t >= tH || s >= tH) m |= BAD_INPUT | SAT_PIXEL;
      if(t <= tL || s <= tL) m |= BAD_INPUT | LOW_PIXEL;
      if(x < border || x >= w - border || y < border || y >= h - border)
        m |= BAD_PIXEL_S | BAD_PIXEL_T;
      mask[id] = m;
    }
  }
}

// spreadMask (cl_kern/ini.cl:37-67): OK_CONV on every pixel without
// BAD_INPUT that has a BAD_INPUT pixel within +-r (clipped to the frame).
// The BAD_INPUT flags of the tile plus its halo are staged in shared
// memory; the dilation is separable (row OR, then column OR).
constexpr int SP_TX = 64, SP_TY = 16;
__global__ void __launch_bounds__(SP_TX * 4) k_spread_mask(uint16_t* __restrict__ mask,
                                                          int w, int h, int r) {
  extern __shared__ uint8_t sp_s[];
  const int tw = SP_TX + 2 * r, th = SP_TY + 2 * r;
  uint8_t* bad = sp_s;               // th * tw
  uint8_t* rowOr = sp_s + tw * th;   // th * SP_TX
  const int x0 = blockIdx.x * SP_TX - r, y0 = blockIdx.y * SP_TY - r;
  for(int i = threadIdx.x; i < tw * th; i += blockDim.x) {
    int lx = i % tw, ly = i / tw;
    int gx = x0 + lx, gy = y0 + ly;
    uint8_t b = 0;
    if(gx >= 0 && gx < w && gy >= 0 && gy < h)
      b = (mask[(size_t)gy * w + gx] & BAD_INPUT) ? 1 : 0;
    bad[i] = b;
  }
  __syncthreads();
  for(int i = threadIdx.x; i < th * SP_TX; i += blockDim.x) {
    int lx = i % SP_TX, ly = i / SP_TX;
    uint8_t o = 0;
    for(int d = 0; d <= 2 * r; d++) o |= bad[ly * tw + lx + d];
    rowOr[i] = o;
  }
  __syncthreads();
  for(int i = threadIdx.x; i < SP_TX * SP_TY; i += blockDim.x) {
    int lx = i % SP_TX, ly = i / SP_TX;
    int gx = blockIdx.x * SP_TX + lx, gy = blockIdx.y * SP_TY + ly;
    if(gx >= w || gy >= h) continue;
    if(bad[(ly + r) * tw + lx + r]) continue;
    uint8_t o = 0;
    for(int d = 0; d <= 2 * r; d++) o |= rowOr[(ly + d) * SP_TX + lx];
    if(o) mask[(size_t)gy * w + gx] |= OK_CONV;
  }
}

__global__ void k_apply_input_mask(const uint8_t* __restrict__ in, uint16_t* __restrict__ mask,
                                   long long n) {
  for(long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
      i += (long long)gridDim.x * blockDim.x)
    if(in[i]) mask[i] |= INPUT_MASK | BAD_INPUT;
}

void stageInitMask(xb_ctx* c) {
  const int border = c->p.hSStampWidth + c->p.hKernelWidth;
  if(c->inputMask && (c->inputMaskW != c->w || c->inputMaskH != c->h))
    throw XbError{XB_ERR_SIZE_MISMATCH, "input mask and frame differ in size"};
  const long long n = (long long)c->w * c->h;
  int blocks = (int)std::min<long long>((n + 1023) / 1024, (long long)c->smCount * 16);
  { KT_SCOPE(c, "mask_input");
  if(c->imgIsF64)
    k_mask_input<double><<<blocks, 256, 0, c->stream>>>(
        (const double*)c->img[0], (const double*)c->img[1], c->mask, c->w, c->h,
        border, c->p.threshHigh, c->p.threshLow);
  else
    k_mask_input<float><<<blocks, 256, 0, c->stream>>>(
        (const float*)c->img[0], (const float*)c->img[1], c->mask, c->w, c->h,
        border, c->p.threshHigh, c->p.threshLow);
  XB_LAUNCHED(c);
  }
  if(c->inputMask) {
    k_apply_input_mask<<<blocks, 256, 0, c->stream>>>(c->inputMask, c->mask, n);
    XB_LAUNCHED(c);
  }
  const int spreadWidth = (int)(c->p.hKernelWidth * c->p.inSpreadMaskFactor);
  const int r = spreadWidth / 2;
  if(r > 0) {
    dim3 grid((c->w + SP_TX - 1) / SP_TX, (c->h + SP_TY - 1) / SP_TY);
    size_t smem = (size_t)(SP_TX + 2 * r) * (SP_TY + 2 * r) + (size_t)(SP_TY + 2 * r) * SP_TX;
    { KT_SCOPE(c, "spread_mask");
    k_spread_mask<<<grid, SP_TX * 4, smem, c->stream>>>(c->mask, c->w, c->h, r);
    XB_LAUNCHED(c);
    }
  }
}

}  // namespace xb
