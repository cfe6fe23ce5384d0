// xb_capi.cpp — the extern "C" boundary of include/xbach.h.
//
// Every entry point converts the library's internal exceptions (CUDA errors,
// parameter errors, the reference's exit paths) into status codes and keeps
// a readable message for xb_last_error().

#include <cmath>
#include <cstring>
#include <string>

#include "xb_internal.h"

using namespace xb;

namespace {

template <class F>
int guarded(xb_ctx* c, F&& f) {
  if(!c) return XB_ERR_ARG;
  try {
    cudaError_t e = cudaSetDevice(c->device);
    if(e != cudaSuccess) throw CudaError{e, "cudaSetDevice"};
    f();
    return XB_OK;
  } catch(const CudaError& e) {
    c->lastError = std::string(e.where) + ": " + cudaGetErrorString(e.code);
    return XB_ERR_CUDA;
  } catch(const XbError& e) {
    c->lastError = e.msg;
    return e.code;
  } catch(const std::exception& e) {
    c->lastError = e.what();
    return XB_ERR_NOMEM;
  }
}

int validate(const xb_params& p, std::string& why) {
  if(p.nGauss < 1 || p.nGauss > XB_MAX_GAUSS) return why = "nGauss out of range", XB_ERR_ARG;
  for(int i = 0; i < p.nGauss; i++)
    if(p.dg[i] < 0 || !(p.bg[i] > 0.0f)) return why = "bad Gaussian degree/width", XB_ERR_ARG;
  if(p.hSStampWidth < 1 || p.hKernelWidth < 1 || p.maxKSStamps < 1 || p.stampsx < 1 ||
     p.stampsy < 1 || p.kernelOrder < 0 || p.backgroundOrder < 0)
    return why = "non-positive size parameter", XB_ERR_ARG;
  Geo g = makeGeo(p);
  if(g.nPSF > MAX_NPSF || g.fK > MAX_FK || g.fSS > MAX_FSS || g.maxSS > MAX_MAXSS ||
     g.nSol > MAX_SOL)
    return why = "parameters exceed this build's limits", XB_ERR_UNSUPPORTED;
  if(p.mode != XB_MODE_PLAIN && p.mode != XB_MODE_MIXED) return why = "unknown mode", XB_ERR_ARG;
  if(!(p.readNoise >= 0.0) || !std::isfinite(p.readNoise) || !std::isfinite(p.gain))
    return why = "bad gain or read noise", XB_ERR_ARG;
  if(p.convPerPixel != 0 && p.convPerPixel != 1) return why = "convPerPixel is 0 or 1", XB_ERR_ARG;
  if(p.fitWeighted != 0 && p.fitWeighted != 1) return why = "fitWeighted is 0 or 1", XB_ERR_ARG;
  return XB_OK;
}

}  // namespace

namespace xb {
// Parameters that size the fit or build its basis: a context keeps them for
// its lifetime (its basis tables and launch shapes depend on them).
bool sameFit(const xb_params& a, const xb_params& b) {
  const Geo ga = makeGeo(a), gb = makeGeo(b);
  if(std::memcmp(&ga, &gb, sizeof(Geo)) != 0) return false;
  if(a.mode != b.mode || a.nGauss != b.nGauss) return false;
  for(int i = 0; i < a.nGauss; i++)
    if(a.dg[i] != b.dg[i] || a.bg[i] != b.bg[i]) return false;
  return true;
}
}  // namespace xb

namespace {

template <class T>
void uploadImages(xb_ctx* c, const T* t, const T* s, int w, int h, bool f64) {
  const size_t n = (size_t)w * h;
  c->w = w;
  c->h = h;
  c->imgIsF64 = f64 ? 1 : 0;
  for(int i = 0; i < 2; i++) {
    T* d = buf<T>(c, i == 0 ? "imgT" : "imgS", n);
    XB_CUDA(cudaMemcpyAsync(d, i == 0 ? t : s, n * sizeof(T), cudaMemcpyHostToDevice, c->stream));
    c->img[i] = d;
  }
}

void afterUpload(xb_ctx* c) {
  const size_t n = (size_t)c->w * c->h;
  // two spare words: the substamp search ORs bits with 32-bit atomics on the
  // aligned word that holds a 16-bit mask entry
  c->mask = buf<uint16_t>(c, "mask", n + 2);
  c->arrays.clear();
  c->scalars.clear();
  c->scalars["w"] = c->w;
  c->scalars["h"] = c->h;
  c->stage = 1;
  stageInitMask(c);
  if(c->trace) c->put("mask_init", toHost(c, c->mask, n));
}

void needStage(xb_ctx* c, int st) {
  if(c->stage < st) throw XbError{XB_ERR_STATE, "stage called out of order"};
}

}  // namespace

extern "C" {

void xb_params_default(xb_params* p) {
  std::memset(p, 0, sizeof(*p));
  p->stampsx = 10;
  p->stampsy = 10;
  p->threshLow = 0.0;
  p->threshHigh = 25000.0;
  p->threshKernFit = 20.0;
  p->sigKernFit = 2.0;
  p->sigClipAlpha = 3.0;
  p->iqRange = 1.35;
  p->maxKSStamps = 3;
  p->hSStampWidth = 15;
  p->hKernelWidth = 10;
  p->inSpreadMaskFactor = 1.0;
  p->normalizeTemplate = 1;
  p->backgroundOrder = 1;
  p->kernelOrder = 2;
  p->nGauss = 3;
  p->dg[0] = 6;
  p->dg[1] = 4;
  p->dg[2] = 2;
  p->bg[0] = (float)(1.0 / (2.0 * 0.7 * 0.7));
  p->bg[1] = (float)(1.0 / (2.0 * 1.5 * 1.5));
  p->bg[2] = (float)(1.0 / (2.0 * 3.0 * 3.0));
  p->mode = XB_MODE_PLAIN;
  p->verbose = 0;
}

int xb_params_npsf(const xb_params* p) {
  int n = 0;
  for(int i = 0; i < p->nGauss && i < XB_MAX_GAUSS; i++) n += (p->dg[i] + 1) * (p->dg[i] + 2) / 2;
  return n;
}

int xb_ctx_create(const xb_params* p, int device, xb_ctx** out) {
  if(!p || !out) return XB_ERR_ARG;
  *out = nullptr;
  std::string why;
  int rc = validate(*p, why);
  if(rc != XB_OK) return rc;
  auto* c = new xb_ctx();
  c->p = *p;
  c->device = device;
  c->g = makeGeo(*p);
  rc = guarded(c, [&] {
    XB_CUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    XB_CUDA(cudaDeviceGetAttribute(&c->smCount, cudaDevAttrMultiProcessorCount, device));
    c->basis = buildBasis(c->p, c->g);
    const Basis& b = c->basis;
    c->dFX = buf<double>(c, "fX", b.fX.size());
    c->dFY = buf<double>(c, "fY", b.fY.size());
    c->dVec = buf<double>(c, "vec", b.vec.size());
    c->dYGroupStart = buf<int>(c, "yGroupStart", b.yGroupStart.size());
    c->dYGroupMembers = buf<int>(c, "yGroupMembers", b.yGroupMembers.size());
    c->dKx = buf<int>(c, "kx", b.kx.size());
    c->dKy = buf<int>(c, "ky", b.ky.size());
    toDevice(c, c->dFX, b.fX);
    toDevice(c, c->dFY, b.fY);
    toDevice(c, c->dVec, b.vec);
    toDevice(c, c->dYGroupStart, b.yGroupStart);
    toDevice(c, c->dYGroupMembers, b.yGroupMembers);
    toDevice(c, c->dKx, b.kx);
    toDevice(c, c->dKy, b.ky);
    {
      const int fK = c->g.fK, nPSF = c->g.nPSF, nG = (int)b.yGroupStart.size() - 1;
      std::vector<float> fs((size_t)2 * (nPSF + nG) * fK);
      auto split = [&](double v, float& hi, float& lo) {
        hi = (float)v;
        lo = (float)(v - (double)hi);
      };
      for(int i = 0; i < nPSF * fK; i++) split(b.fX[i], fs[i], fs[(size_t)nPSF * fK + i]);
      float* fy = fs.data() + (size_t)2 * nPSF * fK;
      for(int gi = 0; gi < nG; gi++)
        for(int k = 0; k < fK; k++)
          split(b.fY[(size_t)b.yGroupMembers[b.yGroupStart[gi]] * fK + k], fy[gi * fK + k],
                fy[(size_t)nG * fK + gi * fK + k]);
      c->dFSplit = buf<float>(c, "fSplit", fs.size());
      toDevice(c, c->dFSplit, fs);
    }
    XB_CUDA(cudaStreamSynchronize(c->stream));
  });
  if(rc != XB_OK) {
    xb_ctx_destroy(c);
    return rc;
  }
  *out = c;
  return XB_OK;
}

int xb_ctx_destroy(xb_ctx* c) {
  if(!c) return XB_ERR_ARG;
  cudaSetDevice(c->device);
  if(c->stream) cudaStreamSynchronize(c->stream);
  destroyGraphs(c);
  for(auto& kv : c->pool)
    if(kv.second.p) cudaFree(kv.second.p);
  if(c->stream) cudaStreamDestroy(c->stream);
  delete c;
  return XB_OK;
}

const char* xb_last_error(const xb_ctx* c) { return c ? c->lastError.c_str() : "null context"; }

int xb_set_input_mask(xb_ctx* c, const uint8_t* mask, int w, int h) {
  return guarded(c, [&] {
    if(!mask) {
      c->inputMask = nullptr;  // the buffer stays in the pool
      c->inputMaskW = c->inputMaskH = 0;
      return;
    }
    if(w <= 0 || h <= 0) throw XbError{XB_ERR_ARG, "bad mask size"};
    const size_t n = (size_t)w * h;
    c->inputMask = buf<uint8_t>(c, "input_mask", n);
    XB_CUDA(cudaMemcpyAsync(c->inputMask, mask, n, cudaMemcpyHostToDevice, c->stream));
    XB_CUDA(cudaStreamSynchronize(c->stream));
    c->inputMaskW = w;
    c->inputMaskH = h;
  });
}

int xb_ctx_set_params(xb_ctx* c, const xb_params* p) {
  return guarded(c, [&] {
    if(!p) throw XbError{XB_ERR_ARG, "null parameters"};
    std::string why;
    const int rc = validate(*p, why);
    if(rc != XB_OK) throw XbError{rc, why};
    if(!sameFit(c->p, *p))
      throw XbError{XB_ERR_ARG, "the parameters change the basis or the fit's sizes (new context)"};
    c->p = *p;
    c->stage = 0;
  });
}

int xb_set_option(xb_ctx* c, const char* name, long long value) {
  if(!c || !name) return XB_ERR_ARG;
  std::string n(name);
  if(n == "trace") {
    c->trace = value != 0;
  } else if(n == "time_kernels") {
    c->timeKernels = value != 0;
    c->kt.total.clear();
  } else if(n == "gram_fp64") {
    c->gramFp64 = value != 0;
  } else if(n == "fill_gram") {
    c->fillGram = value != 0;
  } else if(n == "fill_gram_tma") {
    c->fillGramTma = value != 0;
  } else if(n == "test_wait_timeout") {
    c->testWaitTimeout = value != 0;
  } else if(n == "ldl_panel") {
    c->ldlPanel = value != 0;
  } else if(n == "ldl_cluster") {
    if(value != 8 && value != 16) return XB_ERR_ARG;
    c->ldlCluster = (int)value;
  } else if(n == "graph") {
    if(value != 0 && !mixedMode(c)) {
      c->lastError = "frame graphs are built for the mixed mode";
      return XB_ERR_UNSUPPORTED;
    }
    c->graph = value != 0;
  } else if(n == "rank") {
    if(value < 0 || value > 2) return XB_ERR_ARG;
    c->rank = (int)value;
  } else if(n == "autotune") {
    c->autotune = value != 0;
  } else if(n == "tune_variant") {
    c->tuneForce = value < 0 ? -1 : (int)value;
  } else if(n == "rank_candidates") {
    if(value < 0 || value > MAX_MAXSS) return XB_ERR_ARG;
    c->rankCandidates = (int)value;
  } else if(n == "rank_tau") {
    if(value <= 0 || value >= 1000) return XB_ERR_ARG;
    c->rankTau = (int)value;
  } else {
    return XB_ERR_ARG;
  }
  return XB_OK;
}

int xb_init(xb_ctx* c, const double* T, int tw, int th, const double* S, int sw, int sh) {
  return guarded(c, [&] {
    if(!T || !S || tw <= 0 || th <= 0) throw XbError{XB_ERR_ARG, "bad image"};
    if(tw != sw || th != sh)
      throw XbError{XB_ERR_SIZE_MISMATCH, "Template image and science image must be the same size!"};
    uploadImages<double>(c, T, S, tw, th, true);
    afterUpload(c);
  });
}

int xb_init_f32(xb_ctx* c, const float* T, int tw, int th, const float* S, int sw, int sh) {
  return guarded(c, [&] {
    if(!T || !S || tw <= 0 || th <= 0) throw XbError{XB_ERR_ARG, "bad image"};
    if(tw != sw || th != sh)
      throw XbError{XB_ERR_SIZE_MISMATCH, "Template image and science image must be the same size!"};
    uploadImages<float>(c, T, S, tw, th, false);
    afterUpload(c);
  });
}

int xb_init_device_f32(xb_ctx* c, const float* dT, const float* dS, int w, int h) {
  return guarded(c, [&] {
    if(!dT || !dS || w <= 0 || h <= 0) throw XbError{XB_ERR_ARG, "bad image"};
    c->w = w;
    c->h = h;
    c->imgIsF64 = 0;
    c->img[0] = (void*)dT;  // caller keeps them alive until the next init
    c->img[1] = (void*)dS;
    afterUpload(c);
  });
}

int xb_sss(xb_ctx* c) {
  return guarded(c, [&] {
    needStage(c, 1);
    stageSss(c);
    c->stage = 2;
  });
}

int xb_cmv(xb_ctx* c) {
  return guarded(c, [&] {
    needStage(c, 2);
    stageCmv(c);
    c->stage = 3;
  });
}

int xb_cd(xb_ctx* c, int* convTemplate) {
  return guarded(c, [&] {
    needStage(c, 3);
    stageCd(c);
    if(convTemplate) *convTemplate = c->convTemplate;
    c->stage = 4;
  });
}

int xb_ksc(xb_ctx* c) {
  return guarded(c, [&] {
    needStage(c, 4);
    stageKsc(c);
    c->stage = 5;
  });
}

int xb_conv(xb_ctx* c, double* kernSum) {
  return guarded(c, [&] {
    needStage(c, 5);
    stageConvSub(c, false);
    if(kernSum) *kernSum = c->kernSum;
    c->stage = 6;
  });
}

int xb_sub(xb_ctx* c) {
  return guarded(c, [&] {
    needStage(c, 6);
    stageConvSub(c, true);
    c->stage = 7;
  });
}

int xb_run_device(xb_ctx* c, const float* dT, const float* dS, int w, int h, float* dConv,
                  float* dDiff) {
  return guarded(c, [&] {
    if(!dT || !dS || w <= 0 || h <= 0) throw XbError{XB_ERR_ARG, "bad image"};
    runFrame(c, dT, dS, w, h, dConv, dDiff, false);
  });
}

int xb_run(xb_ctx* c, const float* T, const float* S, int w, int h, float* convOut,
           float* diffOut) {
  if(c && c->graph && mixedMode(c)) {
    // frame graph: inputs straight into the graph's images, one replay,
    // outputs straight back
    return guarded(c, [&] {
      if(!T || !S || w <= 0 || h <= 0) throw XbError{XB_ERR_ARG, "bad image"};
      runFrame(c, T, S, w, h, convOut, diffOut, true);
    });
  }
  int rc = xb_init_f32(c, T, w, h, S, w, h);
  if(rc == XB_OK) rc = xb_sss(c);
  if(rc == XB_OK) rc = xb_cmv(c);
  if(rc == XB_OK) rc = xb_cd(c, nullptr);
  if(rc == XB_OK) rc = xb_ksc(c);
  if(rc == XB_OK) rc = xb_conv(c, nullptr);
  if(rc == XB_OK) rc = xb_sub(c);
  if(rc == XB_OK && convOut) rc = xb_get_image(c, XB_IMG_CONV, convOut);
  if(rc == XB_OK && diffOut) rc = xb_get_image(c, XB_IMG_DIFF, diffOut);
  return rc;
}

int xb_get_image(xb_ctx* c, int which, float* out) {
  return guarded(c, [&] {
    if(!out) throw XbError{XB_ERR_ARG, "null output"};
    const size_t n = (size_t)c->w * c->h;
    if(which == XB_IMG_CONV) needStage(c, 6);
    else if(which == XB_IMG_DIFF) needStage(c, 7);
    else throw XbError{XB_ERR_ARG, "use xb_get_mask for the mask"};
    const float* d = which == XB_IMG_CONV ? c->convF : c->diffF;
    XB_CUDA(cudaMemcpyAsync(out, d, n * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
    XB_CUDA(cudaStreamSynchronize(c->stream));
  });
}

int xb_get_image_f64(xb_ctx* c, int which, double* out) {
  return guarded(c, [&] {
    if(!out) throw XbError{XB_ERR_ARG, "null output"};
    const size_t n = (size_t)c->w * c->h;
    if(which == XB_IMG_CONV) needStage(c, 6);
    else if(which == XB_IMG_DIFF) needStage(c, 7);
    else throw XbError{XB_ERR_ARG, "use xb_get_mask for the mask"};
    const double* d = which == XB_IMG_CONV ? c->convD : c->diffD;
    if(d) {
      XB_CUDA(cudaMemcpyAsync(out, d, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
      XB_CUDA(cudaStreamSynchronize(c->stream));
    } else {
      std::vector<float> f = toHost(c, which == XB_IMG_CONV ? c->convF : c->diffF, n);
      for(size_t i = 0; i < n; i++) out[i] = f[i];
    }
  });
}

int xb_get_mask(xb_ctx* c, uint16_t* out) {
  return guarded(c, [&] {
    needStage(c, 1);
    const size_t n = (size_t)c->w * c->h;
    XB_CUDA(cudaMemcpyAsync(out, c->mask, n * sizeof(uint16_t), cudaMemcpyDeviceToHost, c->stream));
    XB_CUDA(cudaStreamSynchronize(c->stream));
  });
}

int xb_get_device_images(xb_ctx* c, const float** dConv, const float** dDiff) {
  return guarded(c, [&] {
    needStage(c, 7);
    if(dConv) *dConv = c->convF;
    if(dDiff) *dDiff = c->diffF;
  });
}

int xb_get_solution(xb_ctx* c, double* out, int cap, int* n) {
  return guarded(c, [&] {
    needStage(c, 5);
    if(n) *n = (int)c->hSol.size();
    if(out)
      for(int i = 0; i < cap && i < (int)c->hSol.size(); i++) out[i] = c->hSol[i];
  });
}

int xb_get_array(xb_ctx* c, const char* name, void* out, size_t cap, size_t* nbytes) {
  if(!c || !name) return XB_ERR_ARG;
  auto it = c->arrays.find(name);
  if(it == c->arrays.end()) return XB_ERR_ARG;
  if(nbytes) *nbytes = it->second.size();
  if(out) std::memcpy(out, it->second.data(), std::min(cap, it->second.size()));
  return XB_OK;
}

int xb_get_scalar(xb_ctx* c, const char* name, double* out) {
  if(!c || !name || !out) return XB_ERR_ARG;
  const std::string nm(name);
  if(nm.rfind("kt:", 0) == 0) {  // kt:<kernel>:ms | kt:<kernel>:n
    int rc = guarded(c, [&] { ktCollect(c); });
    if(rc != XB_OK) return rc;
    const size_t colon = nm.rfind(':');
    auto kt = c->kt.total.find(nm.substr(3, colon - 3));
    if(kt == c->kt.total.end() || colon <= 3) return XB_ERR_ARG;
    *out = nm.substr(colon + 1) == "n" ? (double)kt->second.second : kt->second.first;
    return XB_OK;
  }
  auto it = c->scalars.find(name);
  if(it == c->scalars.end()) return XB_ERR_ARG;
  *out = it->second;
  return XB_OK;
}

long long xb_kernel_launches(const xb_ctx* c) { return c ? c->launches : 0; }

int xb_get_stream(xb_ctx* c, void** stream) {
  if(!c || !stream) return XB_ERR_ARG;
  *stream = (void*)c->stream;
  return XB_OK;
}

}  // extern "C"
