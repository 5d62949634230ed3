// Per-kernel timing instrumentation (see timing.h).
#include <atomic>
#include <mutex>
#include <vector>

#include "common.h"
#include "timing.h"

namespace s2g {

namespace {
struct Rec {
  cudaEvent_t a = nullptr, b = nullptr;
  int cat = KC_OTHER;
  double flops = 0, bytes = 0;
};
std::atomic<bool> g_on{false};
std::mutex g_mu;
std::vector<Rec> g_recs;
size_t g_used = 0;
}  // namespace

bool timing_enabled() { return g_on.load(std::memory_order_relaxed); }

KTimer::KTimer(int cat, cudaStream_t st, double flops, double bytes) {
  if (!timing_enabled()) return;
  std::lock_guard<std::mutex> lk(g_mu);
  if (g_used == g_recs.size()) {
    Rec r;
    if (cudaEventCreate(&r.a) != cudaSuccess || cudaEventCreate(&r.b) != cudaSuccess) return;
    g_recs.push_back(r);
  }
  slot_ = (int)g_used++;
  Rec &r = g_recs[slot_];
  r.cat = cat;
  r.flops = flops;
  r.bytes = bytes;
  st_ = st;
  cudaEventRecord(r.a, st);
}

KTimer::~KTimer() {
  if (slot_ < 0) return;
  std::lock_guard<std::mutex> lk(g_mu);
  cudaEventRecord(g_recs[slot_].b, st_);
}

}  // namespace s2g

extern "C" {

// Switches timing on (clearing previous records) or off.
int s2let_gpu_timing_enable(int on) {
  std::lock_guard<std::mutex> lk(s2g::g_mu);
  s2g::g_used = 0;
  s2g::g_on = on != 0;
  return 0;
}

// out[c*4 + 0..3] = launches, total milliseconds, algorithmic flops, algorithmic
// bytes of category c (timing.h KCat), c < ncat.  Synchronises the recorded events.
int s2let_gpu_timing_report(double *out, int ncat) {
  std::lock_guard<std::mutex> lk(s2g::g_mu);
  for (int i = 0; i < ncat * 4; ++i) out[i] = 0.0;
  for (size_t i = 0; i < s2g::g_used; ++i) {
    s2g::Rec &r = s2g::g_recs[i];
    if (r.cat >= ncat) continue;
    float ms = 0.f;
    if (cudaEventSynchronize(r.b) != cudaSuccess) return s2g::ERR_CUDA;
    if (cudaEventElapsedTime(&ms, r.a, r.b) != cudaSuccess) return s2g::ERR_CUDA;
    out[r.cat * 4 + 0] += 1.0;
    out[r.cat * 4 + 1] += ms;
    out[r.cat * 4 + 2] += r.flops;
    out[r.cat * 4 + 3] += r.bytes;
  }
  return 0;
}

}  // extern "C"
