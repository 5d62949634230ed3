// Per-kernel timing instrumentation (see timing.h).
#include <algorithm>
#include <atomic>
#include <mutex>
#include <vector>

#include "common.h"
#include "runtime.h"
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
  int d2h = 0, by_kernel = 0;
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

CopyMark copy_trace_begin(cudaMemcpyKind kind, double bytes, cudaStream_t st) {
  CopyMark m;
  if (!g_copy_on.load(std::memory_order_relaxed)) return m;
  S2G_CUDA(cudaEventCreate(&m.a));
  S2G_CUDA(cudaEventCreate(&m.b));
  m.d2h = kind == cudaMemcpyDeviceToHost;
  m.bytes = bytes;
  S2G_CUDA(cudaEventRecord(m.a, st));
  return m;
}

void copy_trace_end(const CopyMark &m, bool by_kernel, cudaStream_t st) {
  if (!m.a) return;
  S2G_CUDA(cudaEventRecord(m.b, st));
  CopyRec r;
  r.a = m.a;
  r.b = m.b;
  r.d2h = m.d2h;
  r.by_kernel = by_kernel ? 1 : 0;
  r.bytes = m.bytes;
  std::lock_guard<std::mutex> lk(g_copy_mu);
  g_copies.push_back(r);
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

// FMA throughput probe: every thread runs 8 independent FMA chains (enough to
// hide the pipe latency at the occupancy launched), so the kernel is bound by
// the FMA issue rate of the type T.  The chains' sum is stored only when it
// equals an unreachable value, which keeps the compiler from removing them.
template <class T>
__global__ void __launch_bounds__(256) k_fma_chains(T *out, int iters, T a, T b) {
  T x[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) x[k] = (T)(threadIdx.x + k);
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = x[k] * a + b;  // one FMA (contraction on in device code)
  }
  T s = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += x[k];
  if (s == (T)-1.2345e30) out[0] = s;
}

namespace s2g {
namespace {
template <class T>
int fma_rate(int iters, double *tflops) {
  int dev = 0, nsm = 0;
  S2G_CUDA(cudaGetDevice(&dev));
  S2G_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  T *out = nullptr;
  S2G_CUDA(cudaMalloc(&out, sizeof(T)));
  cudaEvent_t e0, e1;
  S2G_CUDA(cudaEventCreate(&e0));
  S2G_CUDA(cudaEventCreate(&e1));
  const int blocks = nsm * 8, threads = 256;
  // |a| < 1 and b > 0: the chains converge to b / (1 - a), no overflow or subnormals
  k_fma_chains<T><<<blocks, threads>>>(out, 16, (T)0.999, (T)0.001);  // warm-up
  S2G_LAUNCHED();
  S2G_CUDA(cudaEventRecord(e0));
  k_fma_chains<T><<<blocks, threads>>>(out, iters, (T)0.999, (T)0.001);
  S2G_CUDA(cudaEventRecord(e1));
  S2G_CUDA(cudaEventSynchronize(e1));
  S2G_LAUNCHED();
  float ms = 0.f;
  S2G_CUDA(cudaEventElapsedTime(&ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  *tflops = 2.0 * 8.0 * (double)blocks * threads * iters / (ms * 1e-3) / 1e12;
  return 0;
}
}  // namespace
}  // namespace s2g

extern "C" {

// Measured FMA throughput of this GPU (the denominators of the FP64 and FP32
// roofline fractions): fp64 != 0 for FP64, else FP32; *tflops = 2 x FMAs / s
// over one launch of `iters` iterations of 8 chains per thread.
int s2let_gpu_fma_rate(int fp64, int iters, double *tflops) {
  return s2g::guarded("s2let_gpu_fma_rate", [&] {
    S2G_REQUIRE(iters > 0 && tflops != nullptr, s2g::ERR_INVALID, "iters must be positive, tflops not NULL");
    s2g::ensure_device();
    if (fp64)
      s2g::fma_rate<double>(iters, tflops);
    else
      s2g::fma_rate<float>(iters, tflops);
  });
}

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

// out[d*5 + 0..4] for d = 0 (host to device), 1 (device to host): copies,
// bytes, busy milliseconds (sum of the copies' own durations), span
// milliseconds (first copy start to last copy end of that direction) and the
// copies made by the copy kernel.  Synchronises the recorded events; keeps the
// records.
int s2let_gpu_copy_trace_report(double *out) {
  std::lock_guard<std::mutex> lk(s2g::g_copy_mu);
  for (int i = 0; i < 10; ++i) out[i] = 0.0;
  if (s2g::g_copies.empty()) return 0;
  const cudaEvent_t t0 = s2g::g_copies[0].a;
  double lo[2] = {1e300, 1e300}, hi[2] = {-1e300, -1e300};
  for (const s2g::CopyRec &r : s2g::g_copies) {
    float ms = 0.f, sa = 0.f, sb = 0.f;
    if (cudaEventSynchronize(r.b) != cudaSuccess) return s2g::ERR_CUDA;
    if (cudaEventElapsedTime(&ms, r.a, r.b) != cudaSuccess || cudaEventElapsedTime(&sa, t0, r.a) != cudaSuccess ||
        cudaEventElapsedTime(&sb, t0, r.b) != cudaSuccess)
      return s2g::ERR_CUDA;
    double *o = out + 5 * r.d2h;
    o[0] += 1.0;
    o[1] += r.bytes;
    o[2] += ms;
    o[4] += r.by_kernel;
    lo[r.d2h] = std::min(lo[r.d2h], (double)sa);
    hi[r.d2h] = std::max(hi[r.d2h], (double)sb);
  }
  for (int d = 0; d < 2; ++d)
    if (out[5 * d] > 0) out[5 * d + 3] = hi[d] - lo[d];
  return 0;
}

}  // extern "C"
