// Per-kernel timing instrumentation (see timing.h).
#include <algorithm>
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
// copy trace: one record per traced copy, events owned here
struct CopyRec {
  cudaEvent_t a = nullptr, b = nullptr;
  int d2h = 0;
  double bytes = 0;
};
std::atomic<bool> g_copy_on{false};
std::mutex g_copy_mu;
std::vector<CopyRec> g_copies;

void clear_copies() {
  for (CopyRec &r : g_copies) {
    cudaEventDestroy(r.a);
    cudaEventDestroy(r.b);
  }
  g_copies.clear();
}
}  // namespace

void copy_async(void *dst, size_t dpitch, const void *src, size_t spitch, size_t width, size_t height,
                cudaMemcpyKind kind, cudaStream_t st) {
  if (width == 0 || height == 0) return;
  CopyRec r;
  const bool on = g_copy_on.load(std::memory_order_relaxed);
  if (on) {
    S2G_CUDA(cudaEventCreate(&r.a));
    S2G_CUDA(cudaEventCreate(&r.b));
    r.d2h = kind == cudaMemcpyDeviceToHost;
    r.bytes = (double)width * (double)height;
    S2G_CUDA(cudaEventRecord(r.a, st));
  }
  if (height == 1)
    S2G_CUDA(cudaMemcpyAsync(dst, src, width, kind, st));
  else
    S2G_CUDA(cudaMemcpy2DAsync(dst, dpitch, src, spitch, width, height, kind, st));
  if (on) {
    S2G_CUDA(cudaEventRecord(r.b, st));
    std::lock_guard<std::mutex> lk(g_copy_mu);
    g_copies.push_back(r);
  }
}

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

// Copy trace of the host-pointer batch calls: on != 0 clears previous records
// and starts tracing, 0 stops.
int s2let_gpu_copy_trace_enable(int on) {
  std::lock_guard<std::mutex> lk(s2g::g_copy_mu);
  s2g::clear_copies();
  s2g::g_copy_on = on != 0;
  return 0;
}

// out[d*4 + 0..3] for d = 0 (host to device), 1 (device to host): copies,
// bytes, busy milliseconds (sum of the copies' own durations) and span
// milliseconds (first copy start to last copy end of that direction).
// Synchronises the recorded events; keeps the records.
int s2let_gpu_copy_trace_report(double *out) {
  std::lock_guard<std::mutex> lk(s2g::g_copy_mu);
  for (int i = 0; i < 8; ++i) out[i] = 0.0;
  if (s2g::g_copies.empty()) return 0;
  const cudaEvent_t t0 = s2g::g_copies[0].a;
  double lo[2] = {1e300, 1e300}, hi[2] = {-1e300, -1e300};
  for (const s2g::CopyRec &r : s2g::g_copies) {
    float ms = 0.f, sa = 0.f, sb = 0.f;
    if (cudaEventSynchronize(r.b) != cudaSuccess) return s2g::ERR_CUDA;
    if (cudaEventElapsedTime(&ms, r.a, r.b) != cudaSuccess || cudaEventElapsedTime(&sa, t0, r.a) != cudaSuccess ||
        cudaEventElapsedTime(&sb, t0, r.b) != cudaSuccess)
      return s2g::ERR_CUDA;
    double *o = out + 4 * r.d2h;
    o[0] += 1.0;
    o[1] += r.bytes;
    o[2] += ms;
    lo[r.d2h] = std::min(lo[r.d2h], (double)sa);
    hi[r.d2h] = std::max(hi[r.d2h], (double)sb);
  }
  for (int d = 0; d < 2; ++d)
    if (out[4 * d] > 0) out[4 * d + 3] = hi[d] - lo[d];
  return 0;
}

}  // extern "C"
