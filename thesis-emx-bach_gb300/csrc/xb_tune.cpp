// xb_tune.cpp — the autotuner for launch shapes (no counterpart in the
// reference, whose work-group sizes are fixed in the host code).
//
// A tunable kernel is launched through tunedVariant() with a key (kernel
// name + device + a shape number) and a launcher for each of its variants.
// Variants of one kernel produce identical results and differ only in tile
// shape, so the choice is free.  The first call for a key times every
// variant on the context's stream (one warm-up launch of each, then five
// rounds timing two launches of each variant in turn with CUDA events; a
// variant's time is its best round) and keeps the fastest in a process-wide
// table;
// other threads that reach the same key meanwhile use the default variant.
// With XB_TUNE_CACHE set, the table is read from and appended to that file
// ("key variant" lines), so later processes skip the timing.  Option
// "autotune" (default on) turns the timing off: variant 0 is used; so does
// XB_AUTOTUNE=0 in the environment (for runs under a profiler, whose
// serialisation would make the timings meaningless).

#include <cstdlib>
#include <fstream>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "xb_internal.h"

namespace xb {

namespace {

std::mutex gMu;
std::map<std::string, int> gTable;  // key -> chosen variant (-1: being timed)
bool gLoaded = false;

void loadCacheLocked() {
  if(gLoaded) return;
  gLoaded = true;
  const char* path = std::getenv("XB_TUNE_CACHE");
  if(!path || !*path) return;
  std::ifstream in(path);
  std::string key;
  int v;
  while(in >> key >> v)
    if(v >= 0) gTable[key] = v;
}

void appendCache(const std::string& key, int v) {
  const char* path = std::getenv("XB_TUNE_CACHE");
  if(!path || !*path) return;
  std::ofstream out(path, std::ios::app);
  out << key << ' ' << v << '\n';
}

}  // namespace

int tunedVariant(xb_ctx* c, const char* kernel, long long shape, int nVariants,
                 const std::function<void(int)>& launch) {
  if(c->tuneForce >= 0) return c->tuneForce < nVariants ? c->tuneForce : nVariants - 1;
  static const bool envOff = [] {
    const char* e = std::getenv("XB_AUTOTUNE");
    return e && e[0] == '0';
  }();
  if(!c->autotune || envOff || nVariants <= 1) return 0;
  const std::string key = std::string(kernel) + "@dev" + std::to_string(c->device) + ":" +
                          std::to_string(shape);
  if(c->capturing) {  // a graph being captured cannot time: the table's choice or variant 0
    std::lock_guard<std::mutex> lk(gMu);
    loadCacheLocked();
    auto it = gTable.find(key);
    return it != gTable.end() && it->second >= 0 ? it->second : 0;
  }
  {
    std::lock_guard<std::mutex> lk(gMu);
    loadCacheLocked();
    auto it = gTable.find(key);
    if(it != gTable.end()) {
      const int v = it->second < 0 ? 0 : it->second;
      c->scalars["tune:" + std::string(kernel)] = v;
      return v;
    }
    gTable[key] = -1;  // this thread times it
  }
  // Every variant once (lazy loading, first-touch costs), then rounds that
  // time each variant in turn (two launches) and keep its best round, so a
  // clock still ramping up or a neighbour's burst of work does not decide
  // for one variant alone.
  cudaEvent_t e0, e1;
  XB_CUDA(cudaEventCreate(&e0));
  XB_CUDA(cudaEventCreate(&e1));
  for(int v = 0; v < nVariants; v++) launch(v);
  std::vector<float> bestOf(nVariants, 0.f);
  constexpr int kRounds = 5, kPerRound = 2;
  for(int round = 0; round < kRounds; round++)
    for(int v = 0; v < nVariants; v++) {
      XB_CUDA(cudaEventRecord(e0, c->stream));
      for(int r = 0; r < kPerRound; r++) launch(v);
      XB_CUDA(cudaEventRecord(e1, c->stream));
      XB_CUDA(cudaEventSynchronize(e1));
      float ms = 0.f;
      XB_CUDA(cudaEventElapsedTime(&ms, e0, e1));
      if(round == 0 || ms < bestOf[v]) bestOf[v] = ms;
    }
  int best = 0;
  for(int v = 0; v < nVariants; v++) {
    c->scalars["tune:" + std::string(kernel) + ":v" + std::to_string(v) + ":ms"] = bestOf[v] / kPerRound;
    if(bestOf[v] < bestOf[best]) best = v;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  {
    std::lock_guard<std::mutex> lk(gMu);
    gTable[key] = best;
  }
  appendCache(key, best);
  c->scalars["tune:" + std::string(kernel)] = best;
  return best;
}

}  // namespace xb
