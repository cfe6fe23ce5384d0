// xb_graph.cu — whole frame pairs replayed as captured CUDA graphs (option
// "graph", mixed mode; no counterpart in the reference, whose host loop
// reads every decision back).
//
// Stage by stage, the host reads back the kept-stamp counts after sss, the
// test-list lengths and merits in cd and the rejection count after every ksc
// check, and sizes the next launches by them.  A frame graph moves every one
// of those decisions onto the device:
//   * launches are sized by the stamp-grid bound (nAll) and read the live
//     count from device memory (the liveN arguments of the stage kernels);
//   * the low-threshold sss retry is an IF node on the kept counts;
//   * the global test fit of each cd set is an IF node on its list length;
//   * the fit direction is a pair of IF nodes set from the two merits;
//   * the ksc reject-and-refit loop is a WHILE node whose condition the
//     check sets (refills pending, with an iteration bound).
// The same kernels run in the same order on the same data, so a replay
// writes the images of the stage-by-stage run bit for bit.  One graph is
// captured per frame shape (size and parameters) on first use and replayed
// for every later frame of that shape; a replay costs one launch, two input
// and two output copies and one synchronisation for the frame record.

#include <cstring>
#include <map>
#include <string>

#include "xb_internal.h"

namespace xb {

// Frame record, packed on the device at the end of a replay and copied to
// pinned host memory by the graph itself.
struct FrameRec {
  int nKept[2];
  int sssRetry;
  int nTest[2];
  int convTemplate;
  int kscIterations;
  int kscOverflow;
  int kscRefills;
  int singular;
  int timeout;
  double merit[2];
  double kernSum;
};

struct FrameGraph {
  cudaGraphExec_t exec = nullptr;
  float* in[2] = {nullptr, nullptr};  // the graph's input images
  float* conv = nullptr;
  float* diff = nullptr;
  uint16_t* mask = nullptr;
  FrameRec* rec = nullptr;            // pinned; followed by nSol doubles of solution
  int stampsx = 0, stampsy = 0, fStampWidth = 0, nAll = 0;
  // kernel launches of each part, for the launch count of a replay
  long long lTop = 0, lRetry = 0, lAny = 0, lCd[2] = {0, 0}, lBranch[2] = {0, 0},
            lKsc[2] = {0, 0};
};

struct FrameGraphs {
  std::map<std::string, FrameGraph> byShape;
};

namespace {

constexpr int REC_RETRY = 0, REC_CONVT = 1, REC_KSC_IT = 2, REC_KSC_OVER = 3, REC_REFILLS = 4;

__global__ void k_cond_sss_retry(const int* __restrict__ nKept, int nAll,
                                 cudaGraphConditionalHandle h, int* __restrict__ rec) {
  // bach.cpp:142-161 with the stage-by-stage expressions
  const double fT = (double)nKept[0] / nAll, fS = (double)nKept[1] / nAll;
  const int retry = (fT < 0.1 || fS < 0.1) ? 1 : 0;
  rec[REC_RETRY] = retry;
  cudaGraphSetConditional(h, retry);
}

__global__ void k_cond_positive(const int* __restrict__ v, int n, cudaGraphConditionalHandle h) {
  int any = 0;
  for(int i = 0; i < n; i++) any |= v[i] > 0 ? 1 : 0;
  cudaGraphSetConditional(h, any);
}

__global__ void k_set_double(double* p, double v) { *p = v; }

// cd's decision (bach.cpp:303-309): convolve the template when the science
// merit is larger; h0 runs the fit on set 0, h1 on set 1.
__global__ void k_cond_direction(const double* __restrict__ merit, cudaGraphConditionalHandle h0,
                                 cudaGraphConditionalHandle h1, int* __restrict__ rec) {
  const int convTemplate = merit[1] > merit[0] ? 1 : 0;
  rec[REC_CONVT] = convTemplate;
  cudaGraphSetConditional(h0, convTemplate);      // chosen = 0
  cudaGraphSetConditional(h1, 1 - convTemplate);  // chosen = 1
}

__global__ void k_cond_ksc(const int* __restrict__ outs, int limit, int* __restrict__ rec,
                           cudaGraphConditionalHandle h) {
  const int it = ++rec[REC_KSC_IT];
  rec[REC_REFILLS] += outs[0];
  int more = outs[0] > 0 ? 1 : 0;
  if(more && it > limit) {  // indices only grow, so this cannot happen
    rec[REC_KSC_OVER] = 1;
    more = 0;
  }
  cudaGraphSetConditional(h, more);
}

__global__ void k_frame_record(const int* __restrict__ nKept, const int* __restrict__ rec,
                               const int* __restrict__ nTest, const double* __restrict__ merit,
                               const double* __restrict__ kernSum,
                               const int* __restrict__ singular, int* __restrict__ status,
                               FrameRec* __restrict__ out) {
  out->nKept[0] = nKept[0];
  out->nKept[1] = nKept[1];
  out->sssRetry = rec[REC_RETRY];
  out->nTest[0] = nTest[0];
  out->nTest[1] = nTest[1];
  out->convTemplate = rec[REC_CONVT];
  out->kscIterations = rec[REC_KSC_IT];
  out->kscOverflow = rec[REC_KSC_OVER];
  out->kscRefills = rec[REC_REFILLS];
  out->singular = *singular;
  out->timeout = status[1];
  status[1] = 0;  // reported once, as checkSolveTimeout does
  out->merit[0] = merit[0];
  out->merit[1] = merit[1];
  out->kernSum = *kernSum;
}

cudaStream_t bodyStream(xb_ctx* c, int depth) {
  while((int)c->bodyStreams.size() <= depth) {
    cudaStream_t s;
    XB_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    c->bodyStreams.push_back(s);
  }
  return c->bodyStreams[depth];
}

}  // namespace

// ------------------------------------------------------ capture helpers ---

void uploadNow(xb_ctx* c, void* d, const void* h, size_t bytes) {
  if(!c->upStream) XB_CUDA(cudaStreamCreateWithFlags(&c->upStream, cudaStreamNonBlocking));
  XB_CUDA(cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, c->upStream));
  XB_CUDA(cudaStreamSynchronize(c->upStream));
}

cudaGraphConditionalHandle graphHandle(xb_ctx* c, unsigned dflt) {
  cudaStreamCaptureStatus st;
  cudaGraph_t g = nullptr;
  XB_CUDA(cudaStreamGetCaptureInfo(c->stream, &st, nullptr, &g, nullptr, nullptr, nullptr));
  if(st != cudaStreamCaptureStatusActive) throw XbError{XB_ERR_STATE, "no graph capture active"};
  cudaGraphConditionalHandle h;
  XB_CUDA(cudaGraphConditionalHandleCreate(&h, g, dflt, cudaGraphCondAssignDefault));
  return h;
}

// A conditional node (IF, or WHILE when loop) on h after the work captured
// so far on c->stream; body() is captured into it on a stream of its own
// nesting depth, then capture continues after the node.
long long graphBody(xb_ctx* c, cudaGraphConditionalHandle h, bool loop,
                    const std::function<void()>& body) {
  cudaStreamCaptureStatus st;
  cudaGraph_t g = nullptr;
  const cudaGraphNode_t* deps = nullptr;
  const cudaGraphEdgeData* edges = nullptr;
  size_t nDeps = 0;
  XB_CUDA(cudaStreamGetCaptureInfo(c->stream, &st, nullptr, &g, &deps, &edges, &nDeps));
  cudaGraphNodeParams np = {};
  np.type = cudaGraphNodeTypeConditional;
  np.conditional.handle = h;
  np.conditional.type = loop ? cudaGraphCondTypeWhile : cudaGraphCondTypeIf;
  np.conditional.size = 1;
  cudaGraphNode_t node;
  XB_CUDA(cudaGraphAddNode(&node, g, deps, edges, nDeps, &np));
  cudaGraph_t bodyGraph = np.conditional.phGraph_out[0];
  cudaStream_t outer = c->stream;
  cudaStream_t inner = bodyStream(c, c->bodyDepth);
  XB_CUDA(cudaStreamBeginCaptureToGraph(inner, bodyGraph, nullptr, nullptr, 0,
                                        cudaStreamCaptureModeRelaxed));
  c->stream = inner;
  c->bodyDepth++;
  const long long l0 = c->launches;
  try {
    body();
  } catch(...) {
    cudaGraph_t dummy;
    cudaStreamEndCapture(inner, &dummy);
    c->stream = outer;
    c->bodyDepth--;
    throw;
  }
  cudaGraph_t done;
  c->bodyDepth--;
  c->stream = outer;
  XB_CUDA(cudaStreamEndCapture(inner, &done));
  XB_CUDA(cudaStreamUpdateCaptureDependencies(outer, &node, nullptr, 1,
                                              cudaStreamSetCaptureDependencies));
  return c->launches - l0;
}

void graphSssRetry(xb_ctx* c, const int* nKept, int nAll, const std::function<void()>& body) {
  const cudaGraphConditionalHandle h = graphHandle(c, 0);
  k_cond_sss_retry<<<1, 1, 0, c->stream>>>(nKept, nAll, h, graphRec(c));
  XB_LAUNCHED(c);
  c->graphRetryLaunches = graphBody(c, h, false, body);
}

long long graphIfPositive(xb_ctx* c, const int* v, int n, const std::function<void()>& body) {
  const cudaGraphConditionalHandle h = graphHandle(c, 0);
  k_cond_positive<<<1, 1, 0, c->stream>>>(v, n, h);
  XB_LAUNCHED(c);
  return graphBody(c, h, false, body);
}

void graphSetDouble(xb_ctx* c, double* p, double v) {
  k_set_double<<<1, 1, 0, c->stream>>>(p, v);
  XB_LAUNCHED(c);
}

long long graphWhile(xb_ctx* c, const std::function<void(cudaGraphConditionalHandle)>& body) {
  const cudaGraphConditionalHandle h = graphHandle(c, 1);  // the first pass always runs
  return graphBody(c, h, true, [&] { body(h); });
}

void graphKscContinue(xb_ctx* c, cudaGraphConditionalHandle h, const int* outs, int limit) {
  k_cond_ksc<<<1, 1, 0, c->stream>>>(outs, limit, graphRec(c), h);
  XB_LAUNCHED(c);
}

int* graphRec(xb_ctx* c) { return buf<int>(c, "graph_rec", 8); }

// ---------------------------------------------------------- capture ------

namespace {

// Frame size plus every parameter a capture bakes in (field by field: the
// struct's padding bytes are not part of the key).
std::string shapeKey(const xb_ctx* c, int w, int h) {
  std::string k;
  auto put = [&](const auto& v) { k.append(reinterpret_cast<const char*>(&v), sizeof(v)); };
  const xb_params& p = c->p;
  put(w);
  put(h);
  put(p.stampsx);
  put(p.stampsy);
  put(p.threshLow);
  put(p.threshHigh);
  put(p.threshKernFit);
  put(p.sigKernFit);
  put(p.sigClipAlpha);
  put(p.iqRange);
  put(p.maxKSStamps);
  put(p.hSStampWidth);
  put(p.hKernelWidth);
  put(p.inSpreadMaskFactor);
  put(p.normalizeTemplate);
  put(p.backgroundOrder);
  put(p.kernelOrder);
  put(p.nGauss);
  for(int i = 0; i < p.nGauss; i++) {
    put(p.dg[i]);
    put(p.bg[i]);
  }
  put(p.mode);
  put(p.gain);
  put(p.readNoise);
  put(p.convPerPixel);
  put(p.fitWeighted);
  put(c->gramFp64);
  put(c->ldlPanel);
  put(c->ldlCluster);
  put(c->fillGram);
  put(c->fillGramTma);
  put(c->testWaitTimeout);
  const uintptr_t im = (uintptr_t)c->inputMask;  // the mask's content is read at replay
  put(im);
  const int rank = c->rankW ? c->rank : 0;  // the weights are read from the device at replay
  put(rank);
  put(c->rankTau);
  put(c->rankCandidates);
  return k;
}

// The stage sequence of one frame, captured on c->stream, with the kernel
// launches of each part for the launch count of a replay.
void captureStages(xb_ctx* c, FrameGraph& fg) {
  const Geo& g = c->g;
  const long long l0 = c->launches;
  c->graphRetryLaunches = 0;
  stageInitMask(c);
  stageSss(c);
  fg.lRetry = c->graphRetryLaunches;
  int* rec = graphRec(c);
  double* merit = buf<double>(c, "cd_merit", 2);
  // both sets empty: no fit (the host reports it)
  const long long lAnyAll = graphIfPositive(c, c->dIWork, 2, [&] {
    stageCmv(c);
    stageCdGraph(c, fg.lCd);
    const cudaGraphConditionalHandle h0 = graphHandle(c, 0), h1 = graphHandle(c, 0);
    k_cond_direction<<<1, 1, 0, c->stream>>>(merit, h0, h1, rec);
    XB_LAUNCHED(c);
    for(int si = 0; si < 2; si++) {
      const long long lb = graphBody(c, si == 0 ? h0 : h1, false, [&] {
        c->chosen = si;
        c->convTemplate = si == 0 ? 1 : 0;
        fg.lKsc[si] = stageKscGraph(c);
        stageConvSub(c, false);
      });
      fg.lBranch[si] = lb - fg.lKsc[si];
    }
  });
  fg.lAny = lAnyAll - fg.lCd[0] - fg.lCd[1] - fg.lBranch[0] - fg.lKsc[0] - fg.lBranch[1] -
            fg.lKsc[1];
  FrameRec* dRec = buf<FrameRec>(c, "frame_rec", 1);
  k_frame_record<<<1, 1, 0, c->stream>>>(c->dIWork, rec, buf<int>(c, "cd_ntest", 2), merit,
                                         buf<double>(c, "kernSum", 1),
                                         buf<int>(c, "fit_singular", 1), deviceStatus(c), dRec);
  XB_LAUNCHED(c);
  XB_CUDA(cudaMemcpyAsync(fg.rec, dRec, sizeof(FrameRec), cudaMemcpyDeviceToHost, c->stream));
  XB_CUDA(cudaMemcpyAsync((char*)fg.rec + sizeof(FrameRec), buf<double>(c, "solution", 1),
                          sizeof(double) * g.nSol, cudaMemcpyDeviceToHost, c->stream));
  fg.lTop = c->launches - l0 - fg.lRetry - lAnyAll;
}

}  // namespace

// The host view of a finished frame, kept across a capture (capture runs
// no work but reassigns the context's pointers and decisions).
struct CtxView {
  int w, h, imgIsF64, stage, stampsx, stampsy, fStampWidth, nAll, sssRetry;
  void* img[2];
  uint16_t* mask;
  float *convF, *diffF;
  double *convD, *diffD, *dSol;
  StampSetDev set[2];
  int convTemplate, chosen, kscIterations, singular;
  double merit[2], kernSum;
  std::map<std::string, double> scalars;
  std::vector<double> hSol;
  std::string lastError;
};

static CtxView saveView(const xb_ctx* c) {
  CtxView v;
  v.w = c->w;
  v.h = c->h;
  v.imgIsF64 = c->imgIsF64;
  v.stage = c->stage;
  v.stampsx = c->stampsx;
  v.stampsy = c->stampsy;
  v.fStampWidth = c->fStampWidth;
  v.nAll = c->nAll;
  v.sssRetry = c->sssRetry;
  v.img[0] = c->img[0];
  v.img[1] = c->img[1];
  v.mask = c->mask;
  v.convF = c->convF;
  v.diffF = c->diffF;
  v.convD = c->convD;
  v.diffD = c->diffD;
  v.dSol = c->dSol;
  v.set[0] = c->set[0];
  v.set[1] = c->set[1];
  v.convTemplate = c->convTemplate;
  v.chosen = c->chosen;
  v.kscIterations = c->kscIterations;
  v.singular = c->singular;
  v.merit[0] = c->merit[0];
  v.merit[1] = c->merit[1];
  v.kernSum = c->kernSum;
  v.scalars = c->scalars;
  v.hSol = c->hSol;
  v.lastError = c->lastError;
  return v;
}

static void restoreView(xb_ctx* c, const CtxView& v) {
  c->w = v.w;
  c->h = v.h;
  c->imgIsF64 = v.imgIsF64;
  c->stage = v.stage;
  c->stampsx = v.stampsx;
  c->stampsy = v.stampsy;
  c->fStampWidth = v.fStampWidth;
  c->nAll = v.nAll;
  c->sssRetry = v.sssRetry;
  c->img[0] = v.img[0];
  c->img[1] = v.img[1];
  c->mask = v.mask;
  c->convF = v.convF;
  c->diffF = v.diffF;
  c->convD = v.convD;
  c->diffD = v.diffD;
  c->dSol = v.dSol;
  c->set[0] = v.set[0];
  c->set[1] = v.set[1];
  c->convTemplate = v.convTemplate;
  c->chosen = v.chosen;
  c->kscIterations = v.kscIterations;
  c->singular = v.singular;
  c->merit[0] = v.merit[0];
  c->merit[1] = v.merit[1];
  c->kernSum = v.kernSum;
  c->scalars = v.scalars;
  c->hSol = v.hSol;
  c->lastError = v.lastError;
}

// Captures the frame graph of the current shape (images already in fg.in).
static void captureFrame(xb_ctx* c, FrameGraph& fg) {
  const Geo& g = c->g;
  c->keepBuffers = 1;
  c->img[0] = fg.in[0];
  c->img[1] = fg.in[1];
  c->imgIsF64 = 0;
  XB_CUDA(cudaStreamSynchronize(c->stream));
  cudaGraph_t graph = nullptr;
  // pass 0 sizes every pool buffer for the graph (its launches are sized by
  // the stamp-grid bound), pass 1 is the graph; a buffer that still grows in
  // pass 1 would leave an earlier node with a retired pointer
  for(int pass = 0; pass < 2; pass++) {
    const size_t grownBefore = c->retired.size();
    const long long launches0 = c->launches;
    c->capturing = 1;
    XB_CUDA(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeRelaxed));
    try {
      c->mask = buf<uint16_t>(c, "mask", (size_t)c->w * c->h + 2);
      captureStages(c, fg);
    } catch(...) {
      cudaGraph_t dummy = nullptr;
      cudaStreamEndCapture(c->stream, &dummy);
      if(dummy) cudaGraphDestroy(dummy);
      c->capturing = 0;
      throw;
    }
    c->capturing = 0;
    XB_CUDA(cudaStreamEndCapture(c->stream, &graph));
    c->launches = launches0;  // captured, not launched
    if(pass == 0) {
      cudaGraphDestroy(graph);
      graph = nullptr;
    } else if(c->retired.size() != grownBefore) {
      cudaGraphDestroy(graph);
      throw XbError{XB_ERR_STATE, "a buffer grew while the frame graph was captured"};
    }
  }
  cudaError_t e = cudaGraphInstantiate(&fg.exec, graph, 0);
  cudaGraphDestroy(graph);
  if(e != cudaSuccess) throw CudaError{e, "cudaGraphInstantiate"};
  XB_CUDA(cudaGraphUpload(fg.exec, c->stream));
  fg.conv = c->convF;
  fg.diff = c->diffF;
  fg.mask = c->mask;
  fg.stampsx = c->stampsx;
  fg.stampsy = c->stampsy;
  fg.fStampWidth = c->fStampWidth;
  fg.nAll = c->nAll;
  (void)g;
}

// One frame pair from T,S to conv,diff (device buffers, or host buffers
// when host is set; conv/diff may be null).  With c->graph set the frame
// goes through the graph of its shape (captured on first use), its inputs
// copied straight into the graph's input images.
void runFrame(xb_ctx* c, const float* T, const float* S, int w, int h, float* conv, float* diff,
              bool host) {
  const size_t n = (size_t)w * h, bytes = n * sizeof(float);
  const bool useGraph = c->graph && mixedMode(c) && !c->trace && !c->timeKernels;
  const cudaMemcpyKind kIn = host ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
  const cudaMemcpyKind kOut = host ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
  const float *dT = T, *dS = S;
  if(host && (!useGraph || !c->graphs || !c->graphs->byShape.count(shapeKey(c, w, h)))) {
    // stage by stage (or the capturing first frame) reads device images
    float* uT = buf<float>(c, "run_in0", n);
    float* uS = buf<float>(c, "run_in1", n);
    XB_CUDA(cudaMemcpyAsync(uT, T, bytes, kIn, c->stream));
    XB_CUDA(cudaMemcpyAsync(uS, S, bytes, kIn, c->stream));
    dT = uT;
    dS = uS;
  }
  if(!useGraph) {
    // stage by stage
    int rc = xb_init_device_f32(c, dT, dS, w, h);
    if(rc == XB_OK) rc = xb_sss(c);
    if(rc == XB_OK) rc = xb_cmv(c);
    if(rc == XB_OK) rc = xb_cd(c, nullptr);
    if(rc == XB_OK) rc = xb_ksc(c);
    if(rc == XB_OK) rc = xb_conv(c, nullptr);
    if(rc == XB_OK) rc = xb_sub(c);
    if(rc != XB_OK) throw XbError{rc, c->lastError};
    if(conv) XB_CUDA(cudaMemcpyAsync(conv, c->convF, bytes, kOut, c->stream));
    if(diff) XB_CUDA(cudaMemcpyAsync(diff, c->diffF, bytes, kOut, c->stream));
    XB_CUDA(cudaStreamSynchronize(c->stream));
    return;
  }
  if(!c->graphs) c->graphs = new FrameGraphs;
  const std::string key = shapeKey(c, w, h);
  auto it = c->graphs->byShape.find(key);
  if(it == c->graphs->byShape.end()) {
    // first frame of this shape: stage by stage (this also settles the
    // tuned launch shapes and sizes the buffers), then the capture; the
    // stage-by-stage results stay the frame's results
    c->graph = 0;
    try {
      runFrame(c, dT, dS, w, h, nullptr, nullptr, false);
    } catch(...) {
      c->graph = 1;
      throw;
    }
    c->graph = 1;
    if(conv) XB_CUDA(cudaMemcpyAsync(conv, c->convF, bytes, kOut, c->stream));
    if(diff) XB_CUDA(cudaMemcpyAsync(diff, c->diffF, bytes, kOut, c->stream));
    XB_CUDA(cudaStreamSynchronize(c->stream));
    CtxView keep = saveView(c);
    FrameGraph fg;
    fg.in[0] = buf<float>(c, "graph_in0", n);
    fg.in[1] = buf<float>(c, "graph_in1", n);
    XB_CUDA(cudaHostAlloc((void**)&fg.rec, sizeof(FrameRec) + sizeof(double) * c->g.nSol,
                          cudaHostAllocDefault));
    try {
      captureFrame(c, fg);
    } catch(...) {
      cudaFreeHost(fg.rec);
      if(fg.exec) cudaGraphExecDestroy(fg.exec);
      restoreView(c, keep);
      throw;
    }
    c->graphs->byShape[key] = fg;
    restoreView(c, keep);
    c->scalars["graph_captured"] = 1;
    return;
  }
  FrameGraph& fg = it->second;
  XB_CUDA(cudaMemcpyAsync(fg.in[0], T, bytes, kIn, c->stream));
  XB_CUDA(cudaMemcpyAsync(fg.in[1], S, bytes, kIn, c->stream));
  XB_CUDA(cudaGraphLaunch(fg.exec, c->stream));
  if(conv) XB_CUDA(cudaMemcpyAsync(conv, fg.conv, bytes, kOut, c->stream));
  if(diff) XB_CUDA(cudaMemcpyAsync(diff, fg.diff, bytes, kOut, c->stream));
  XB_CUDA(cudaStreamSynchronize(c->stream));
  const FrameRec& r = *fg.rec;
  c->w = w;
  c->h = h;
  c->imgIsF64 = 0;
  c->img[0] = fg.in[0];
  c->img[1] = fg.in[1];
  c->mask = fg.mask;
  c->convF = fg.conv;
  c->diffF = fg.diff;
  c->convD = c->diffD = nullptr;
  c->stampsx = fg.stampsx;
  c->stampsy = fg.stampsy;
  c->fStampWidth = fg.fStampWidth;
  c->nAll = fg.nAll;
  c->arrays.clear();
  c->scalars.clear();
  c->scalars["w"] = w;
  c->scalars["h"] = h;
  c->scalars["stampsx"] = c->stampsx;
  c->scalars["stampsy"] = c->stampsy;
  c->scalars["fStampWidth"] = c->fStampWidth;
  c->scalars["sss_retry"] = c->sssRetry = r.sssRetry;
  c->set[0].n = r.nKept[0];
  c->set[1].n = r.nKept[1];
  c->scalars["nstamps0"] = r.nKept[0];
  c->scalars["nstamps1"] = r.nKept[1];
  c->launches += fg.lTop + (r.sssRetry ? fg.lRetry : 0);
  if(r.nKept[0] == 0 && r.nKept[1] == 0) {
    c->stage = 2;
    throw XbError{XB_ERR_NO_SUBSTAMPS, "No substamps found"};
  }
  c->launches += fg.lAny + (r.nTest[0] > 0 ? fg.lCd[0] : 0) + (r.nTest[1] > 0 ? fg.lCd[1] : 0);
  c->merit[0] = r.nTest[0] > 0 ? r.merit[0] : 666;
  c->merit[1] = r.nTest[1] > 0 ? r.merit[1] : 666;
  c->convTemplate = r.convTemplate;
  c->chosen = r.convTemplate ? 0 : 1;
  c->launches += fg.lBranch[c->chosen] + (long long)r.kscIterations * fg.lKsc[c->chosen];
  c->scalars["merit0"] = c->merit[0];
  c->scalars["merit1"] = c->merit[1];
  c->scalars["convTemplate"] = c->convTemplate;
  c->scalars["ksc_iterations"] = c->kscIterations = r.kscIterations;
  c->scalars["ksc_refills"] = r.kscRefills;
  c->scalars["singular"] = c->singular = r.singular;
  c->scalars["kernSum"] = c->kernSum = r.kernSum;
  c->scalars["graph_replay"] = 1;
  c->hSol.assign((const double*)((const char*)fg.rec + sizeof(FrameRec)),
                 (const double*)((const char*)fg.rec + sizeof(FrameRec)) + c->g.nSol);
  c->stage = 7;
  if(r.timeout) throw XbError{XB_ERR_DEVICE_TIMEOUT, "a bounded device-side wait ran out of time"};
  if(r.kscOverflow) throw XbError{XB_ERR_STATE, "ksc did not converge"};
}

void destroyGraphs(xb_ctx* c) {
  if(c->graphs) {
    for(auto& kv : c->graphs->byShape) {
      if(kv.second.exec) cudaGraphExecDestroy(kv.second.exec);
      if(kv.second.rec) cudaFreeHost(kv.second.rec);
    }
    delete c->graphs;
    c->graphs = nullptr;
  }
  for(void* p : c->retired) cudaFree(p);
  c->retired.clear();
  for(cudaStream_t s : c->bodyStreams) cudaStreamDestroy(s);
  c->bodyStreams.clear();
  if(c->upStream) cudaStreamDestroy(c->upStream);
  c->upStream = nullptr;
}

}  // namespace xb
