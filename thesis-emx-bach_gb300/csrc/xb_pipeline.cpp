// xb_pipeline.cpp — streaming difference imaging over FITS files
// (xb_pipeline_* in include/xbach.h).
//
// The reference runs one pair per process: read both FITS files, run the
// stages, write conv and sub (src/main.cpp:16-159), so file decode and encode
// sit between GPU runs.  Here three thread groups overlap them across pairs:
//
//   readers  (nIo)      open both FITS files, decode the samples straight into
//                       a pinned slot (FP32 for unscaled BITPIX -32, which is
//                       exact; FP64 otherwise)
//   workers  (nWorkers) one context each: xb_run from the pinned slot
//                       (asynchronous H2D, the frame graph when option "graph"
//                       is on, D2H of conv and diff into the slot)
//   writers  (nIo)      encode conv and diff as BITPIX -32 and write them
//
// Slots circulate free -> read -> computed -> free; there are nWorkers + 2 nIo
// of them, so every worker can hold one while readers prefetch and writers
// drain.  Pinned buffers grow to the largest frame seen and are then reused,
// so a steady stream of same-sized pairs allocates nothing.  Each pair's
// result is the one xb_run gives on a single context.

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "xb_fits.h"
#include "xb_internal.h"

namespace {

using Clock = std::chrono::steady_clock;

double msSince(Clock::time_point t0) {
  return std::chrono::duration<double, std::milli>(Clock::now() - t0).count();
}

// Bounded hand-off between thread groups.
class SlotQueue {
 public:
  void push(int s) {
    {
      std::lock_guard<std::mutex> l(m_);
      q_.push_back(s);
    }
    cv_.notify_one();
  }
  // false once closed and drained
  bool pop(int& s) {
    std::unique_lock<std::mutex> l(m_);
    cv_.wait(l, [&] { return !q_.empty() || closed_; });
    if(q_.empty()) return false;
    s = q_.front();
    q_.pop_front();
    return true;
  }
  void close() {
    {
      std::lock_guard<std::mutex> l(m_);
      closed_ = true;
    }
    cv_.notify_all();
  }

 private:
  std::mutex m_;
  std::condition_variable cv_;
  std::deque<int> q_;
  bool closed_ = false;
};

struct PinnedBuf {
  void* p = nullptr;
  size_t cap = 0;
  // grows (dropping the contents); false when the allocation fails
  bool reserve(size_t bytes) {
    if(bytes <= cap) return true;
    if(p) cudaFreeHost(p);
    p = nullptr;
    cap = 0;
    if(cudaHostAlloc(&p, bytes, cudaHostAllocPortable) != cudaSuccess) {
      p = nullptr;
      return false;
    }
    cap = bytes;
    return true;
  }
  void release() {
    if(p) cudaFreeHost(p);
    p = nullptr;
    cap = 0;
  }
};

struct Slot {
  PinnedBuf in[2];   // template, science (FP32 or FP64 samples)
  PinnedBuf out[2];  // conv, diff (FP32)
  int pair = -1, w = 0, h = 0;
  bool f64 = false;
};

}  // namespace

struct xb_pipeline {
  int device = 0;
  int nIo = 1;
  std::vector<xb_ctx*> workers;
  std::vector<Slot> slots;
  std::string lastError;
  xb_pipeline_stats stats{};
  xb_params base{};                    // the pipeline's parameters
  std::vector<xb_params> pairParams;   // per pair (xb_pipeline_set_params), or empty
};

namespace {

// One pair on worker c from slot s.
int computePair(xb_ctx* c, Slot& s, bool wantConv, bool wantDiff) {
  float* conv = wantConv ? (float*)s.out[0].p : nullptr;
  float* diff = wantDiff ? (float*)s.out[1].p : nullptr;
  if(!s.f64) return xb_run(c, (const float*)s.in[0].p, (const float*)s.in[1].p, s.w, s.h, conv, diff);
  // FP64 samples: the plain path runs on them as read (the mixed path takes
  // FP32 images only)
  if(c->p.mode == XB_MODE_MIXED) {
    c->lastError = "mixed mode takes FP32 images (BITPIX -32 without BSCALE/BZERO)";
    return XB_ERR_UNSUPPORTED;
  }
  int rc = xb_init(c, (const double*)s.in[0].p, s.w, s.h, (const double*)s.in[1].p, s.w, s.h);
  if(rc == XB_OK) rc = xb_sss(c);
  if(rc == XB_OK) rc = xb_cmv(c);
  if(rc == XB_OK) rc = xb_cd(c, nullptr);
  if(rc == XB_OK) rc = xb_ksc(c);
  if(rc == XB_OK) rc = xb_conv(c, nullptr);
  if(rc == XB_OK) rc = xb_sub(c);
  if(rc == XB_OK && conv) rc = xb_get_image(c, XB_IMG_CONV, conv);
  if(rc == XB_OK && diff) rc = xb_get_image(c, XB_IMG_DIFF, diff);
  return rc;
}

// Decodes pair i into slot s; the status of the read.
int readPair(Slot& s, const char* tPath, const char* sPath, std::string& msg, double& bytes) {
  xb::FitsHeader hd[2];
  FILE* f[2] = {nullptr, nullptr};
  const char* path[2] = {tPath, sPath};
  int rc = XB_OK;
  for(int k = 0; k < 2 && rc == XB_OK; k++) {
    rc = path[k] ? xb::fitsOpen(path[k], hd[k], &f[k]) : XB_ERR_ARG;
    if(rc != XB_OK) msg = std::string("Unable to open file '") + (path[k] ? path[k] : "(null)") + "'";
  }
  if(rc == XB_OK && (hd[0].w != hd[1].w || hd[0].h != hd[1].h)) {
    rc = XB_ERR_SIZE_MISMATCH;
    msg = "Template image and science image must be the same size!";
  }
  if(rc == XB_OK) {
    s.w = hd[0].w;
    s.h = hd[0].h;
    s.f64 = !(hd[0].exactF32() && hd[1].exactF32());
    const size_t n = (size_t)s.w * s.h;
    for(int k = 0; k < 2 && rc == XB_OK; k++) {
      if(!s.in[k].reserve(n * (s.f64 ? 8 : 4)) || !s.out[k].reserve(n * 4)) {
        rc = XB_ERR_NOMEM;
        msg = "pinned host allocation failed";
      }
    }
    for(int k = 0; k < 2 && rc == XB_OK; k++) {
      rc = xb::fitsReadSamples(f[k], hd[k], s.in[k].p, s.f64);
      if(rc != XB_OK) msg = std::string("Unable to read file '") + path[k] + "'";
      else bytes += (double)n * (double)(-hd[k].bitpix / 8);
    }
  }
  for(FILE* x : f)
    if(x) std::fclose(x);
  return rc;
}

}  // namespace

extern "C" {

int xb_pipeline_create(const xb_params* p, int device, int nWorkers, int nIo, xb_pipeline** out) {
  if(!out || !p || nWorkers < 1 || nWorkers > 64 || nIo < 1 || nIo > 64) return XB_ERR_ARG;
  *out = nullptr;
  xb_pipeline* pl = new xb_pipeline;
  pl->device = device;
  pl->nIo = nIo;
  pl->base = *p;
  for(int i = 0; i < nWorkers; i++) {
    xb_ctx* c = nullptr;
    const int rc = xb_ctx_create(p, device, &c);
    if(rc != XB_OK) {
      for(xb_ctx* w : pl->workers) xb_ctx_destroy(w);
      if(c) xb_ctx_destroy(c);
      delete pl;
      return rc;
    }
    pl->workers.push_back(c);
  }
  pl->slots.resize((size_t)nWorkers + 2 * (size_t)nIo);
  *out = pl;
  return XB_OK;
}

int xb_pipeline_destroy(xb_pipeline* pl) {
  if(!pl) return XB_ERR_ARG;
  cudaSetDevice(pl->device);
  int rc = XB_OK;
  for(xb_ctx* c : pl->workers) {
    const int r = xb_ctx_destroy(c);
    if(rc == XB_OK) rc = r;
  }
  for(Slot& s : pl->slots)
    for(int k = 0; k < 2; k++) {
      s.in[k].release();
      s.out[k].release();
    }
  delete pl;
  return rc;
}

const char* xb_pipeline_last_error(const xb_pipeline* pl) {
  return pl ? pl->lastError.c_str() : "null pipeline";
}

int xb_pipeline_worker(xb_pipeline* pl, int i, xb_ctx** ctx) {
  if(!pl || !ctx || i < 0 || i >= (int)pl->workers.size()) return XB_ERR_ARG;
  *ctx = pl->workers[i];
  return XB_OK;
}

int xb_pipeline_set_params(xb_pipeline* pl, int nPairs, const xb_params* params) {
  if(!pl || nPairs < 0 || (nPairs > 0 && !params)) return XB_ERR_ARG;
  for(int i = 0; i < nPairs; i++)
    if(!xb::sameFit(pl->base, params[i])) {
      pl->lastError = "pair " + std::to_string(i) +
                      ": parameters change the basis or the fit's sizes of the pipeline";
      return XB_ERR_ARG;
    }
  pl->pairParams.assign(params, params + nPairs);
  return XB_OK;
}

int xb_pipeline_stats_get(const xb_pipeline* pl, xb_pipeline_stats* out) {
  if(!pl || !out) return XB_ERR_ARG;
  *out = pl->stats;
  return XB_OK;
}

int xb_pipeline_run_files(xb_pipeline* pl, int nPairs, const char* const* templatePath,
                          const char* const* sciencePath, const char* const* convPath,
                          const char* const* diffPath, int* pairStatus, double* kernSum) {
  if(!pl) return XB_ERR_ARG;
  if(nPairs < 0 || (nPairs > 0 && (!templatePath || !sciencePath))) {
    pl->lastError = "bad pair lists";
    return XB_ERR_ARG;
  }
  if(!pl->pairParams.empty() && (int)pl->pairParams.size() < nPairs) {
    pl->lastError = "fewer pair parameter sets than pairs";
    return XB_ERR_ARG;
  }
  const auto t0 = Clock::now();
  std::vector<int> st(nPairs, XB_OK);
  std::vector<double> ks(nPairs, 0.0);
  std::vector<std::string> msg(nPairs);
  SlotQueue freeQ, readyQ, doneQ;
  for(int s = 0; s < (int)pl->slots.size(); s++) freeQ.push(s);
  std::atomic<int> next{0}, readersLeft{pl->nIo}, workersLeft{(int)pl->workers.size()};
  std::mutex statMu;
  xb_pipeline_stats acc{};
  std::vector<std::thread> th;

  for(int r = 0; r < pl->nIo; r++)
    th.emplace_back([&] {
      cudaSetDevice(pl->device);
      double ms = 0, bytes = 0;
      int s;
      while(freeQ.pop(s)) {
        const int i = next.fetch_add(1);
        if(i >= nPairs) {
          freeQ.push(s);
          break;
        }
        Slot& sl = pl->slots[s];
        sl.pair = i;
        const auto tr = Clock::now();
        st[i] = readPair(sl, templatePath[i], sciencePath[i], msg[i], bytes);
        ms += msSince(tr);
        if(st[i] == XB_OK) readyQ.push(s);
        else freeQ.push(s);
      }
      {
        std::lock_guard<std::mutex> l(statMu);
        acc.read_ms += ms;
        acc.bytes_read += bytes;
      }
      if(readersLeft.fetch_sub(1) == 1) readyQ.close();
    });
  for(int wi = 0; wi < (int)pl->workers.size(); wi++)
    th.emplace_back([&, wi] {
      cudaSetDevice(pl->device);
      xb_ctx* c = pl->workers[wi];
      double ms = 0;
      int s;
      while(readyQ.pop(s)) {
        Slot& sl = pl->slots[s];
        const int i = sl.pair;
        const auto tc = Clock::now();
        st[i] = xb_ctx_set_params(c, pl->pairParams.empty() ? &pl->base : &pl->pairParams[i]);
        if(st[i] == XB_OK)
          st[i] = computePair(c, sl, convPath && convPath[i], diffPath && diffPath[i]);
        ms += msSince(tc);
        if(st[i] == XB_OK) ks[i] = c->kernSum;
        else msg[i] = c->lastError;
        doneQ.push(s);
      }
      {
        std::lock_guard<std::mutex> l(statMu);
        acc.compute_ms += ms;
      }
      if(workersLeft.fetch_sub(1) == 1) doneQ.close();
    });
  for(int r = 0; r < pl->nIo; r++)
    th.emplace_back([&] {
      double ms = 0, bytes = 0;
      int s;
      while(doneQ.pop(s)) {
        Slot& sl = pl->slots[s];
        const int i = sl.pair;
        const auto tw = Clock::now();
        for(int k = 0; k < 2 && st[i] == XB_OK; k++) {
          const char* path = k == 0 ? (convPath ? convPath[i] : nullptr) : (diffPath ? diffPath[i] : nullptr);
          if(!path) continue;
          if(xb::fitsWrite(path, (const float*)sl.out[k].p, nullptr, sl.w, sl.h) != XB_OK) {
            st[i] = XB_ERR_IO;
            msg[i] = std::string("Unable to save file '") + path + "'";
          } else {
            bytes += (double)sl.w * sl.h * 4;
          }
        }
        ms += msSince(tw);
        freeQ.push(s);
      }
      std::lock_guard<std::mutex> l(statMu);
      acc.write_ms += ms;
      acc.bytes_written += bytes;
    });
  for(auto& t : th) t.join();
  acc.wall_ms = msSince(t0);
  acc.pairs = nPairs;
  pl->stats = acc;
  int rc = XB_OK;
  for(int i = 0; i < nPairs; i++) {
    if(pairStatus) pairStatus[i] = st[i];
    if(kernSum) kernSum[i] = ks[i];
    if(rc == XB_OK && st[i] != XB_OK) {
      rc = st[i];
      pl->lastError = "pair " + std::to_string(i) + ": " + msg[i];
    }
  }
  return rc;
}

}  // extern "C"
