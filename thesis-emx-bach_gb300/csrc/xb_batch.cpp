// xb_batch.cpp — batches of independent frame pairs (xb_batch_* in
// include/xbach.h).
//
// Each frame pair is a complete difference-imaging problem; its stage
// sequence is host-driven (the ksc loop reads rejection counts back after
// every refit), so one frame keeps at most a few kernels in flight and most
// of the GPU idle.  A batch keeps nWorkers contexts, each with its own stream
// and its own host thread; the workers take frames from one queue in order,
// so the GPU interleaves the kernels of up to nWorkers frames.  Contexts keep
// their device buffers between frames (the buffer pool only grows), so a
// steady stream of frames allocates nothing.
//
// Frames may carry their own parameters (xb_batch_set_params): the stamp
// grid, thresholds and clipping of each pair, within the batch's basis and
// sizes.  When the workers replay frame graphs, frames are dealt to workers
// by a fixed schedule (largest first, to the least-loaded worker) instead of
// a shared queue, so the same list of frames meets the same worker, whose
// graph for that shape and parameter set is already captured.

#include <algorithm>
#include <atomic>
#include <numeric>
#include <string>
#include <thread>
#include <vector>

#include "xb_internal.h"

struct xb_batch {
  std::vector<xb_ctx*> workers;
  xb_params base{};                        // the batch's parameters
  std::vector<xb_params> frameParams;      // per frame (xb_batch_set_params), or empty
  std::string lastError;
  int device = 0;
  cudaStream_t join = nullptr;             // caller's stream (xb_batch_set_stream)
  cudaEvent_t start = nullptr;             // recorded on `join` before a run
  std::vector<cudaEvent_t> done;           // one per worker, recorded after its last frame
};

namespace {

// One frame on worker context c: device inputs, outputs copied to the
// caller's device buffers.
int runDeviceFrame(xb_ctx* c, const float* dT, const float* dS, int w, int h, float* dConv,
                   float* dDiff) {
  return xb_run_device(c, dT, dS, w, h, dConv, dDiff);
}

// Frames per worker for graph replays: largest first, each to the worker
// with the fewest pixels so far (lowest index on ties).
std::vector<std::vector<int>> fixedSchedule(int nFrames, int nW, const int* w, const int* h) {
  std::vector<int> order(nFrames);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
    return (long long)w[a] * h[a] > (long long)w[b] * h[b];
  });
  std::vector<long long> load(nW, 0);
  std::vector<std::vector<int>> per(nW);
  for(int i : order) {
    const int k = (int)(std::min_element(load.begin(), load.end()) - load.begin());
    per[k].push_back(i);
    load[k] += (long long)w[i] * h[i];
  }
  return per;
}

template <class F>
int runQueue(xb_batch* b, int nFrames, const int* fw, const int* fh, int* frameStatus,
             double* kernSum, F&& frame) {
  if(!b) return XB_ERR_ARG;
  if(nFrames < 0) {
    b->lastError = "negative frame count";
    return XB_ERR_ARG;
  }
  if(!b->frameParams.empty() && (int)b->frameParams.size() < nFrames) {
    b->lastError = "fewer frame parameter sets than frames";
    return XB_ERR_ARG;
  }
  std::vector<int> st(nFrames, XB_OK);
  std::vector<std::string> msg(nFrames);
  std::atomic<int> next{0};
  std::vector<std::thread> th;
  bool graphs = nFrames > 0;
  for(xb_ctx* c : b->workers) graphs = graphs && c->graph;
  // graph replays: every worker runs, on its fixed share of the frames
  const int nW = graphs ? (int)b->workers.size()
                        : std::min<int>((int)b->workers.size(), std::max(nFrames, 1));
  std::vector<std::vector<int>> fixed;
  if(graphs) fixed = fixedSchedule(nFrames, nW, fw, fh);
  if(b->join) {
    cudaSetDevice(b->device);
    const cudaError_t e = cudaEventRecord(b->start, b->join);
    if(e != cudaSuccess) {
      b->lastError = std::string("batch start event: ") + cudaGetErrorString(e);
      return XB_ERR_CUDA;
    }
  }
  for(int wi = 0; wi < nW; wi++)
    th.emplace_back([&, wi] {
      cudaSetDevice(b->device);
      xb_ctx* c = b->workers[wi];
      if(b->join) cudaStreamWaitEvent(c->stream, b->start, 0);
      for(size_t k = 0;; k++) {
        int i;
        if(graphs) {
          if(k >= fixed[wi].size()) break;
          i = fixed[wi][k];
        } else {
          i = next.fetch_add(1);
          if(i >= nFrames) break;
        }
        st[i] = xb_ctx_set_params(c, b->frameParams.empty() ? &b->base : &b->frameParams[i]);
        if(st[i] == XB_OK) st[i] = frame(c, i);
        if(st[i] != XB_OK) msg[i] = c->lastError;
        if(kernSum) kernSum[i] = st[i] == XB_OK ? c->kernSum : 0.0;
      }
      if(b->join) cudaEventRecord(b->done[wi], c->stream);
    });
  for(auto& t : th) t.join();
  if(b->join)
    for(int wi = 0; wi < nW; wi++) cudaStreamWaitEvent(b->join, b->done[wi], 0);
  int rc = XB_OK;
  for(int i = 0; i < nFrames; i++) {
    if(frameStatus) frameStatus[i] = st[i];
    if(rc == XB_OK && st[i] != XB_OK) {
      rc = st[i];
      b->lastError = "frame " + std::to_string(i) + ": " + msg[i];
    }
  }
  return rc;
}

}  // namespace

extern "C" {

int xb_batch_create(const xb_params* p, int device, int nWorkers, xb_batch** out) {
  if(!out || !p || nWorkers < 1 || nWorkers > 64) return XB_ERR_ARG;
  *out = nullptr;
  xb_batch* b = new xb_batch;
  b->device = device;
  b->base = *p;
  for(int i = 0; i < nWorkers; i++) {
    xb_ctx* c = nullptr;
    const int rc = xb_ctx_create(p, device, &c);
    if(rc != XB_OK) {
      for(xb_ctx* w : b->workers) xb_ctx_destroy(w);
      if(c) xb_ctx_destroy(c);
      delete b;
      return rc;
    }
    b->workers.push_back(c);
  }
  *out = b;
  return XB_OK;
}

int xb_batch_set_stream(xb_batch* b, void* stream) {
  if(!b) return XB_ERR_ARG;
  cudaSetDevice(b->device);
  if(!b->start) {
    if(cudaEventCreateWithFlags(&b->start, cudaEventDisableTiming) != cudaSuccess) return XB_ERR_CUDA;
    b->done.assign(b->workers.size(), nullptr);
    for(auto& e : b->done)
      if(cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return XB_ERR_CUDA;
  }
  b->join = (cudaStream_t)stream;
  return XB_OK;
}

int xb_batch_destroy(xb_batch* b) {
  if(!b) return XB_ERR_ARG;
  int rc = XB_OK;
  cudaSetDevice(b->device);
  if(b->start) cudaEventDestroy(b->start);
  for(cudaEvent_t e : b->done)
    if(e) cudaEventDestroy(e);
  for(xb_ctx* c : b->workers) {
    const int r = xb_ctx_destroy(c);
    if(rc == XB_OK) rc = r;
  }
  delete b;
  return rc;
}

const char* xb_batch_last_error(const xb_batch* b) {
  return b ? b->lastError.c_str() : "null batch";
}

int xb_batch_run(xb_batch* b, int nFrames, const float* const* T, const float* const* S,
                 const int* w, const int* h, float* const* conv, float* const* diff,
                 int* frameStatus, double* kernSum) {
  if(b && nFrames > 0 && (!T || !S || !w || !h)) {
    b->lastError = "null frame arrays";
    return XB_ERR_ARG;
  }
  return runQueue(b, nFrames, w, h, frameStatus, kernSum, [&](xb_ctx* c, int i) {
    return xb_run(c, T[i], S[i], w[i], h[i], conv ? conv[i] : nullptr, diff ? diff[i] : nullptr);
  });
}

int xb_batch_run_device(xb_batch* b, int nFrames, const float* const* dT,
                        const float* const* dS, const int* w, const int* h,
                        float* const* dConv, float* const* dDiff, int* frameStatus,
                        double* kernSum) {
  if(b && nFrames > 0 && (!dT || !dS || !w || !h)) {
    b->lastError = "null frame arrays";
    return XB_ERR_ARG;
  }
  return runQueue(b, nFrames, w, h, frameStatus, kernSum, [&](xb_ctx* c, int i) {
    return runDeviceFrame(c, dT[i], dS[i], w[i], h[i], dConv ? dConv[i] : nullptr,
                          dDiff ? dDiff[i] : nullptr);
  });
}

int xb_batch_set_params(xb_batch* b, int nFrames, const xb_params* params) {
  if(!b || nFrames < 0 || (nFrames > 0 && !params)) return XB_ERR_ARG;
  for(int i = 0; i < nFrames; i++)
    if(!xb::sameFit(b->base, params[i])) {
      b->lastError = "frame " + std::to_string(i) +
                     ": parameters change the basis or the fit's sizes of the batch";
      return XB_ERR_ARG;
    }
  b->frameParams.assign(params, params + nFrames);
  return XB_OK;
}

int xb_batch_worker(xb_batch* b, int i, xb_ctx** ctx) {
  if(!b || !ctx || i < 0 || i >= (int)b->workers.size()) return XB_ERR_ARG;
  *ctx = b->workers[i];
  return XB_OK;
}

}  // extern "C"
