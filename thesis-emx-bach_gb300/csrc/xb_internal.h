// xb_internal.h — context, geometry and helpers shared by the CUDA
// translation units of the GB300 X-BACH library.
//
// Data layout in HBM (one context = one frame pair):
//   img[2]      template / science, FP32 when the input was FP32 (exact
//               promotion to FP64 on load), FP64 otherwise; row-major w*h.
//   mask        uint16 per pixel (bit meanings of include/datatypeUtil.h:172).
//   per stamp set (0 = stamps found on the template, 1 = on the science):
//     count/cur/orig   int per kept stamp
//     ssxy/ssval       maxSS substamp slots per kept stamp (int2 / double)
//     W                [stamp][wRows][fSS*fSS]   FP64 (plain) or FP32 (mixed)
//     Q                [stamp][qCount][qCount]   FP64
//     B                [stamp][bCount]           FP64
//   conv/diff   FP32 output images (plain mode also keeps FP64 copies).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>
#include <functional>
#include <map>
#include <string>
#include <vector>

#include "xbach.h"

namespace xb {

constexpr uint16_t BAD_PIX_VAL = 1u << 0, SAT_PIXEL = 1u << 1,
                   LOW_PIXEL = 1u << 2, NAN_PIXEL = 1u << 3,
                   BAD_CONV = 1u << 4, INPUT_MASK = 1u << 5, OK_CONV = 1u << 6,
                   BAD_INPUT = 1u << 7, BAD_PIXEL_T = 1u << 8,
                   SKIP_T = 1u << 9, BAD_PIXEL_S = 1u << 10,
                   SKIP_S = 1u << 11, BAD_OUTPUT = 1u << 12,
                   MASK_ALL = (1u << 13) - 1u;

// Limits of this build (checked at context creation / sss).
constexpr int MAX_NPSF = 128;       // basis functions
constexpr int MAX_FK = 41;          // kernel width (hKernelWidth <= 20)
constexpr int MAX_FSS = 63;         // substamp width (hSStampWidth <= 31)
constexpr int MAX_SOL = 2048;       // solution length
constexpr int MAX_MAXSS = 16;       // substamp slots per stamp
constexpr int MAX_KORDER = 8;       // per-pixel kernel: spatial terms kept per thread

struct Geo {
  int fSS, hSS, fK, hK, nPSF, nComp1, nComp2, nComp, nBG, matSize, nSol;
  int wRows, wCols, qCount, bCount, maxSS;
};

inline int triNum(int t) { return t * (t + 1) / 2; }

Geo makeGeo(const xb_params& p);
// a and b give the same basis, widths, orders and mode (a context can switch
// between them; stamp grid, thresholds and clipping may differ)
bool sameFit(const xb_params& a, const xb_params& b);

// Basis tables built once on the host (createKernelFilter/createKernelVector,
// cl_kern/cmv.cl:1-68; the host Kernel struct of include/datatypeUtil.h).
struct Basis {
  std::vector<int> gauss, kx, ky;
  std::vector<double> fX, fY, vec;  // nPSF*fK, nPSF*fK, nPSF*fK*fK
  std::vector<int> bgX, bgY, kpX, kpY;
  // unique Y filters: yGroupOf[n] = group; groups list their members
  std::vector<int> yGroupStart, yGroupMembers;  // CSR
};
Basis buildBasis(const xb_params& p, const Geo& g);

struct StampSetDev {
  int n = 0;                 // kept stamps
  int* orig = nullptr;       // original stamp index
  int* count = nullptr;      // usable substamps (<= maxKSStamps)
  int* cur = nullptr;        // current substamp index
  int2* ssxy = nullptr;      // n * maxSS
  double* ssval = nullptr;   // n * maxSS
  void* W = nullptr;         // n * wRows * wCols (double or float)
  double* Q = nullptr;       // n * qCount^2
  double* B = nullptr;       // n * bCount
  float* Wf = nullptr;       // mixed mode: W [n][wRows][ld] as hi + lo floats, ld = wCols
  float* Wlo = nullptr;      //   padded to 32 (Wf the hi parts, Wlo the lo parts)
  double* dots = nullptr;    // mixed mode: per-stamp dot table of the global matrix
  double* omega = nullptr;   // plain mode, weighted fit: n * wCols pixel weights 1 / sigma^2
  const int* dN = nullptr;   // frame graphs: the kept count on the device (n is its bound)
};

// Optional per-kernel CUDA-event timing (option "time_kernels"): launches
// wrapped in KT_SCOPE record events on the context stream; totals are
// collected on request.
struct KTimers {
  std::vector<cudaEvent_t> pool;
  struct Open {
    std::string name;
    cudaEvent_t a, b;
  };
  std::vector<Open> pending;
  std::map<std::string, std::pair<double, long long>> total;  // ms, launches
};

struct DevBuf {  // simple grow-only device allocation
  void* p = nullptr;
  size_t bytes = 0;
};

struct FrameGraphs;  // xb_graph.cu

}  // namespace xb

struct xb_ctx {
  xb_params p{};
  xb::Geo g{};
  xb::Basis basis;
  int device = 0;
  int smCount = 0;
  cudaStream_t stream = nullptr;
  int w = 0, h = 0;
  int imgIsF64 = 0;
  void* img[2] = {nullptr, nullptr};
  uint16_t* mask = nullptr;
  int stage = 0;  // 0 none, 1 init, 2 sss, 3 cmv, 4 cd, 5 ksc, 6 conv, 7 sub
  // sss
  int stampsx = 0, stampsy = 0, fStampWidth = 0, nAll = 0, sssRetry = 0;
  int4* geomAll = nullptr;        // cx, cy, sx, sy for every grid stamp
  double* skyAll[2] = {nullptr, nullptr};
  double* fwhmAll[2] = {nullptr, nullptr};
  int* cntAll[2] = {nullptr, nullptr};
  int2* ssxyAll[2] = {nullptr, nullptr};
  double* ssvalAll[2] = {nullptr, nullptr};
  double* goodScratch = nullptr;  // nAll * fStampWidth^2 good pixels
  uint8_t* clipScratch = nullptr; // nAll * fStampWidth^2 clip flags
  xb::StampSetDev set[2];
  // basis on device
  double* dFX = nullptr;
  double* dFY = nullptr;
  double* dVec = nullptr;
  int* dYGroupStart = nullptr;
  int* dYGroupMembers = nullptr;
  int* dKx = nullptr;
  int* dKy = nullptr;
  // the filters as float pairs (hi = (float)f, lo = (float)(f - hi)) for the
  // fused fill: X filters [nPSF][fK] hi then lo, then the unique Y filters
  // [group][fK] hi then lo
  float* dFSplit = nullptr;
  // cd / ksc
  int convTemplate = 0, chosen = 0;
  double merit[2] = {0, 0};
  double* dSol = nullptr;          // nSol
  std::vector<double> hSol;
  double* dMat = nullptr;          // (matSize+1)^2
  double* dMatLU = nullptr;        // factor workspace
  int* dPiv = nullptr;
  double* dWts = nullptr;          // nStamps * nComp2
  double* dDots = nullptr;         // per-stamp dot products for the matrix
  double* dSig = nullptr;          // per-stamp chi^2
  double* dWork = nullptr;         // generic scratch (doubles)
  int* dIWork = nullptr;           // generic scratch (ints)
  size_t workDoubles = 0, workInts = 0;
  int kscIterations = 0;
  int singular = 0;
  // conv / sub
  double kernSum = 0.0;
  float* convF = nullptr;
  float* diffF = nullptr;
  double* convD = nullptr;
  double* diffD = nullptr;
  // bookkeeping
  long long launches = 0;
  int trace = 0;
  int timeKernels = 0;
  int gramFp64 = 0;  // mixed mode: FP64 CUDA-core Gram instead of the tensor cores (checks)
  int fillGram = 1;     // mixed mode: fused fill + tensor-core Gram where the shape allows
  int fillGramTma = 1;  // the fused kernel stages its windows by TMA tile copies
  int testWaitTimeout = 0;  // option "test_wait_timeout": one bounded wait per fused-kernel CTA runs out
  int rank = 0;          // learned substamp order after sss: 1 demote, 2 sort
  int rankTau = 500;     // demotion threshold of the accept probability, 1/1000
  int autotune = 1;      // time the variants of tunable kernels on first use
  int tuneForce = -1;    // >= 0: launch this variant of every tunable kernel
  uint16_t* rankW = nullptr;  // ranker parameters on the device as BF16 bits (xb_ranker_set)
  int rankCandidates = 0;     // option "rank_candidates": candidates per stamp ranked (0: all)
  int mxTables = 0;        // the mixed build's monomial tables are on the device
  int ldlPanel = 1;        // option "ldl_panel": panel LDL^T kernel (0: the column kernel)
  int ldlCluster = 16;     // option "ldl_cluster": CTAs of the LDL^T cluster (16, or 8)
  uint8_t* inputMask = nullptr;  // xb_set_input_mask (device, inputMaskW x inputMaskH) or none
  int inputMaskW = 0, inputMaskH = 0;
  // frame graphs (xb_graph.cu)
  int graph = 0;           // option "graph": whole frames replay as captured CUDA graphs
  int capturing = 0;       // stage code is being captured: no host reads, no timers
  int keepBuffers = 0;     // graphs hold pool pointers: a grown buffer is retired, not freed
  std::vector<void*> retired;
  cudaStream_t upStream = nullptr;              // uploads made while capturing
  std::vector<cudaStream_t> bodyStreams;        // conditional-body capture, one per depth
  int bodyDepth = 0;
  long long graphRetryLaunches = 0;             // launches of the captured sss retry
  xb::FrameGraphs* graphs = nullptr;            // instantiated graphs by frame shape
  xb::KTimers kt;
  std::string lastError;
  std::map<std::string, std::vector<uint8_t>> arrays;
  std::map<std::string, double> scalars;
  std::map<std::string, xb::DevBuf> pool;

  template <class T>
  void put(const std::string& k, const std::vector<T>& v) {
    std::vector<uint8_t> b(v.size() * sizeof(T));
    if(!v.empty()) memcpy(b.data(), v.data(), b.size());
    arrays[k] = std::move(b);
  }
};

namespace xb {

// ---- error handling --------------------------------------------------------
struct CudaError {
  cudaError_t code;
  const char* where;
};
#define XB_CUDA(call)                                          \
  do {                                                         \
    cudaError_t e_ = (call);                                   \
    if(e_ != cudaSuccess) throw ::xb::CudaError{e_, #call};    \
  } while(0)
#define XB_LAUNCHED(ctx)                                             \
  do {                                                               \
    (ctx)->launches++;                                               \
    cudaError_t e_ = cudaGetLastError();                             \
    if(e_ != cudaSuccess) throw ::xb::CudaError{e_, "kernel launch"}; \
  } while(0)

struct XbError {
  int code;
  std::string msg;
};

// Named, grow-only device buffers: a repeated run on the same context
// reuses its allocations, so steady-state runs allocate nothing.
void* poolGet(xb_ctx* c, const char* name, size_t bytes);

// Raises a kernel's dynamic shared-memory limit to the device's opt-in
// maximum.  The limit belongs to the function, process-wide, and concurrent
// contexts (batch workers) launch the same kernels with different sizes, so
// a per-launch setting could undercut another context's launch or captured
// graph; occupancy follows each launch's own request, not this limit.
cudaError_t allowMaxDynamicSmem(const void* func, int device);
template <class T>
T* buf(xb_ctx* c, const char* name, size_t n) {
  return static_cast<T*>(poolGet(c, name, (n ? n : 1) * sizeof(T)));
}
template <class T>
T* buf(xb_ctx* c, const std::string& name, size_t n) {
  return buf<T>(c, name.c_str(), n);
}

template <class T>
std::vector<T> toHost(xb_ctx* c, const T* d, size_t n) {
  std::vector<T> h(n);
  if(n) XB_CUDA(cudaMemcpyAsync(h.data(), d, n * sizeof(T),
                                cudaMemcpyDeviceToHost, c->stream));
  XB_CUDA(cudaStreamSynchronize(c->stream));
  return h;
}
// Host tables for the device.  While a frame graph is being captured the
// copy runs at once on a side stream (the tables are fixed for the frame
// shape, so replays need no copy node).
void uploadNow(xb_ctx* c, void* d, const void* h, size_t bytes);
template <class T>
void toDevice(xb_ctx* c, T* d, const std::vector<T>& h) {
  if(h.empty()) return;
  if(c->capturing) {
    uploadNow(c, d, h.data(), h.size() * sizeof(T));
    return;
  }
  XB_CUDA(cudaMemcpyAsync(d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, c->stream));
}

// ---- kernel timers --------------------------------------------------------
cudaEvent_t ktEvent(xb_ctx* c);
void ktCollect(xb_ctx* c);
struct KtScope {
  xb_ctx* c;
  const char* name;
  cudaEvent_t a = nullptr;
  KtScope(xb_ctx* ctx, const char* n) : c(ctx), name(n) {
    if(c->timeKernels && !c->capturing) {
      a = ktEvent(c);
      cudaEventRecord(a, c->stream);
    }
  }
  ~KtScope() {
    if(a) {
      cudaEvent_t b = ktEvent(c);
      cudaEventRecord(b, c->stream);
      c->kt.pending.push_back({name, a, b});
    }
  }
};
#define XB_CAT2(a, b) a##b
#define XB_CAT(a, b) XB_CAT2(a, b)
#define KT_SCOPE(ctx, name) ::xb::KtScope XB_CAT(kt_scope_, __LINE__)((ctx), (name))

// ---- stage implementations (host orchestration in the .cu files) ---------
void stageInitMask(xb_ctx* c);
void stageSss(xb_ctx* c);
void stageCmv(xb_ctx* c);
// liveN (device, optional): the live length of dList; nList bounds it.
void fillStamps(xb_ctx* c, int si, const int* dList, int nList, int imgConv,
                const int* liveN = nullptr);
void stageCd(xb_ctx* c);
void stageKsc(xb_ctx* c);
void stageConvSub(xb_ctx* c, bool doSub);

// mixed-precision stages (xb_mixed.cu)
int mixedLd(const Geo& g);
int mixedDotStride(const Geo& g);
void fillStampsMixed(xb_ctx* c, int si, const int* dList, int nList, int imgConv,
                     const int* liveN = nullptr);
void sigsMixed(xb_ctx* c, int si, const int* dList, int nList, const double* dSol, int convImg,
               double* dSig, const int* liveN = nullptr);
void luFallbackSolve(xb_ctx* c, const double* M, double* F, int n, double* rhs, int* piv,
                     int* singular, const int* status);
void convSubMixed(xb_ctx* c, double* dKernSum);
// Kernel images of the spatial terms, FP64 (nComp2 x fK^2): the kernel at
// (xf, yf) is sum_t xf^i yf^j Kt[t], t over the (i, j) of the kernel
// polynomial, x power outer.
double* kernelTermsLaunch(xb_ctx* c);
void buildSystemMixed(xb_ctx* c, int si, const int* dList, int nList, int bgBase, double* M,
                      double* rhs, const int* liveN = nullptr);

// global system of the mixed path (xb_ldl.cu): LDL^T on a cluster, refined
// solve, pivoted LU when a pivot fails.  M is kept; rhs becomes the solution.
void globalSolveMixed(xb_ctx* c, const double* M, int n, double* rhs, int* piv, int* singular);
// Device status words of the mixed path: [0] bit 0 = an LDL^T pivot failed
// (per solve), [1] bit 0 = a bounded device-side wait ran out (sticky until
// checkSolveTimeout reports it).  Zeroed when first allocated.
int* deviceStatus(xb_ctx* c);
// Throws XB_ERR_DEVICE_TIMEOUT when a bounded wait of the cluster solve or
// the tensor-core Gram ran out since the last call (synchronises the stream).
void checkSolveTimeout(xb_ctx* c);
// Autotuner (xb_tune.cpp): the variant of a tunable kernel to launch for
// (kernel, device, shape); times all nVariants through `launch` on first use.
int tunedVariant(xb_ctx* c, const char* kernel, long long shape, int nVariants,
                 const std::function<void(int)>& launch);
// Learned substamp ranking (xb_ranker.cu): reorder both sets' substamps.
void rankSubstamps(xb_ctx* c);
// Fused fill + tensor-core Gram of the mixed path (xb_fill_gram.cu): W (hi,
// lo) of the listed stamps and their Gram matrices G (nList x R x R), the
// results of fill + finish + gramTensorCores bit for bit; fillGramFits says
// whether the context's shape and options allow it.
bool fillGramFits(const xb_ctx* c);
void fillGramLaunch(xb_ctx* c, int si, const int* dList, int nList, int imgConv, double* G,
                    const int* liveN);
// Tensor-core Gram of the mixed path (xb_gram_tc.cu) into G (nList x R x R);
// false when the shape is outside its limits.
bool gramTensorCores(xb_ctx* c, int si, const int* dList, int nList, int other, double* G,
                     const int* liveN = nullptr);
inline bool mixedMode(const xb_ctx* c) { return c->p.mode == XB_MODE_MIXED; }
// Noise model of the stamp chi^2: sigma^2 = (|a| + |b|) * invGain + rn2x2,
// which is |a| + |b| exactly for the defaults (gain 1, no read noise).
inline double noiseInvGain(const xb_params& p) { return p.gain > 0.0 ? 1.0 / p.gain : 1.0; }
inline double noiseRn2x2(const xb_params& p) { return 2.0 * p.readNoise * p.readNoise; }
// Weight of a substamp pixel in the weighted fit: 1 / sigma^2 of the noise
// model (0 where the model's variance is not positive).
__host__ __device__ inline double fitWeight(double a, double b, double invGain, double rn2x2) {
  const double v = (fabs(a) + fabs(b)) * invGain + rn2x2;
  return v > 0.0 ? 1.0 / v : 0.0;
}

// ---- frame graphs (xb_graph.cu) -------------------------------------------
// Capture helpers for stage code running under c->capturing: a conditional
// handle of the graph being captured, a conditional node whose body is
// captured from body() (returns the launches captured in it), and the
// device-side setters of the stage decisions.
cudaGraphConditionalHandle graphHandle(xb_ctx* c, unsigned dflt);
long long graphBody(xb_ctx* c, cudaGraphConditionalHandle h, bool loop,
                    const std::function<void()>& body);
void graphSssRetry(xb_ctx* c, const int* nKept, int nAll, const std::function<void()>& body);
long long graphIfPositive(xb_ctx* c, const int* v, int n, const std::function<void()>& body);
void graphSetDouble(xb_ctx* c, double* p, double v);
long long graphWhile(xb_ctx* c, const std::function<void(cudaGraphConditionalHandle)>& body);
void graphKscContinue(xb_ctx* c, cudaGraphConditionalHandle h, const int* outs, int limit);
int* graphRec(xb_ctx* c);
// One frame pair, device or host buffers in and out (graph replay when
// c->graph is set).
void runFrame(xb_ctx* c, const float* T, const float* S, int w, int h, float* conv, float* diff,
              bool host);
void destroyGraphs(xb_ctx* c);
// cd and ksc as captured by a frame graph (xb_fit.cu): lCd gets the launches
// of each set's conditional test fit; stageKscGraph returns the launches of
// one refit pass.
void stageCdGraph(xb_ctx* c, long long lCd[2]);
long long stageKscGraph(xb_ctx* c);

// Kernel image at normalised position (xf, yf) and its sum into *dOut
// (device): tree = 1 sums in 32-wide groups (cl_kern/cd.cl:419-442), tree = 0
// sequentially (src/bachUtil.cpp:532-538).
void kernelSumLaunch(xb_ctx* c, const double* dSol, double xf, double yf, int tree, double* dOut);

}  // namespace xb
