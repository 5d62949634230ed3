// Axisymmetric wavelet hard threshold that allocates no device memory.
//
// Same result as s2let_transform_axisym_wav_hardthreshold_real /
// _multires_real (src/c/s2let_transform_axisym_mw.c:1183-1225), but the host
// arrays are staged in one file-scope device array instead of stream-ordered
// scratch, so a call makes no cudaMalloc / cudaMallocAsync / cudaFree.  There
// is no counterpart of this entry point in the reference.
//
// Scratch contract
//   * capacity: kScratchBytes (8 MiB).  Larger requests fail with
//     S2LET_GPU_ERR_INVALID before any copy.
//   * every call shares the one array: two calls whose GPU work overlaps
//     (calls from two host threads at the same time) race on it and corrupt
//     each other's results.  A call returns after its copy back has finished,
//     so calls from one host thread never overlap.
//   * nothing has to start at zero: each call writes every byte the kernel
//     reads (scale offsets, thresholds, maps) before the kernel runs; bytes
//     past the request keep whatever earlier calls left and are not read.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "common.h"
#include "host_layer.h"
#include "kernels.h"
#include "runtime.h"

namespace {

constexpr size_t kScratchBytes = size_t(8) << 20;
constexpr int kMaxScales = 64;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

// Device address of g_scratch, looked up with that device current the first
// time a call runs on it.  Only a successful lookup is kept: a failed one
// raises ERR_CUDA for that call and is tried again by the next.
struct DeviceSlot {
  std::mutex mu;
  void *ptr = nullptr;
};
DeviceSlot g_slots[kMaxDevices];

unsigned char *scratch_on_current_device() {
  int dev = -1;
  S2G_CUDA(cudaGetDevice(&dev));
  S2G_REQUIRE(dev >= 0 && dev < kMaxDevices, s2g::ERR_UNSUPPORTED, "device ordinal out of range");
  DeviceSlot &s = g_slots[dev];
  std::lock_guard<std::mutex> lk(s.mu);
  if (s.ptr == nullptr) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
    if (e != cudaSuccess || p == nullptr)
      throw s2g::Error(s2g::ERR_CUDA, std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
    s.ptr = p;
  }
  return static_cast<unsigned char *>(s.ptr);
}

size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

}  // namespace

extern "C" int s2let_gpu_axisym_wav_hardthreshold_real_noalloc(double *g_wav, const double *threshold,
                                                               const s2let_parameters_t *parameters,
                                                               int multires) {
  return s2g::guarded("s2let_gpu_axisym_wav_hardthreshold_real_noalloc", [&] {
    S2G_REQUIRE(parameters != nullptr && g_wav != nullptr && threshold != nullptr, s2g::ERR_INVALID,
                "NULL argument");
    s2let_parameters_t q = *parameters;
    q.N = 1;
    q.spin = 0;
    s2g::validate(&q, false);
    s2g::ensure_device();
    const int L = q.L, J = s2g::j_max(q);
    const int nscale = J - q.J_min + 1;
    S2G_REQUIRE(nscale >= 1 && nscale <= kMaxScales, s2g::ERR_INVALID,
                "needs 1 to 64 wavelet scales, got " + std::to_string(nscale));
    int64_t off[kMaxScales];
    int64_t tot = 0;
    for (int k = 0; k < nscale; ++k) {
      const int64_t b = multires ? std::min(s2g::bandlimit(q.J_min + k, q), L) : L;
      off[k] = tot;
      tot += b * (2 * b - 1);
    }
    const size_t off_bytes = align256(sizeof(int64_t) * nscale);
    const size_t thr_bytes = align256(sizeof(double) * nscale);
    const size_t map_bytes = sizeof(double) * (size_t)tot;
    const size_t need = off_bytes + thr_bytes + map_bytes;
    S2G_REQUIRE(need <= kScratchBytes, s2g::ERR_INVALID,
                "wavelet maps need " + std::to_string(need) + " bytes of scratch; this entry point holds at most " +
                    std::to_string(kScratchBytes) + " bytes (8 MiB)");
    unsigned char *base = scratch_on_current_device();
    int64_t *d_off = reinterpret_cast<int64_t *>(base);
    double *d_thr = reinterpret_cast<double *>(base + off_bytes);
    double *d_g = reinterpret_cast<double *>(base + off_bytes + thr_bytes);
    cudaStream_t st = cudaStreamPerThread;
    S2G_CUDA(cudaMemcpyAsync(d_off, off, sizeof(int64_t) * nscale, cudaMemcpyHostToDevice, st));
    S2G_CUDA(cudaMemcpyAsync(d_thr, threshold, sizeof(double) * nscale, cudaMemcpyHostToDevice, st));
    S2G_CUDA(cudaMemcpyAsync(d_g, g_wav, map_bytes, cudaMemcpyHostToDevice, st));
    s2g::hard_threshold(d_g, d_thr, d_off, nscale, tot, st);
    S2G_CUDA(cudaMemcpyAsync(g_wav, d_g, map_bytes, cudaMemcpyDeviceToHost, st));
    S2G_CUDA(cudaStreamSynchronize(st));
  });
}
