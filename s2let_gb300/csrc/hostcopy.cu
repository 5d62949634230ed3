// Host <-> device copies of the host-pointer entry points.
//
// The GPU reaches host memory through its chip-to-chip link.  Measured on
// GB300 with page-locked buffers of 8.8 GB: copies issued by a kernel (SM
// loads and stores of host memory) held 193 GB/s device to host and 211 GB/s
// host to device in every sample, while the copy engines delivered the same
// rates only part of the time and dropped to 40-110 GB/s (device to host
// most often) for stretches of tens to hundreds of milliseconds, with or
// without other GPU activity.  So page-locked host memory is moved by
// k_copy_rows on the caller's stream; anything else (or every copy, with
// S2LET_GPU_HOST_COPY=engine) by the copy engines (see copy_policy).
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdlib>
#include <cstring>

#include "common.h"
#include "timing.h"

namespace s2g {

namespace {

// 64 CTAs of 256 threads: 1 MB in flight.  Measured against 128 CTAs of 128
// threads (which fit beside three ring-DFT CTAs on an SM): device-to-host
// copies overlapping the transforms held 180 against 151 GB/s.
constexpr int kCopyThreads = 256;
constexpr int kCopyUnroll = 4;    // loads in flight per thread (latency of host reads)
constexpr int kCopyBlocks = 64;   // CTAs per copy: enough bytes in flight for the link, few SMs taken

// `height` rows of n elements of T: row r of src at src + r * spitch bytes,
// of dst at dst + r * dpitch.  Rows run along blockIdx.y; each row is
// grid-strided by the x blocks with kCopyUnroll independent loads per thread.
template <class T>
__global__ void __launch_bounds__(kCopyThreads) k_copy_rows(char *__restrict__ dst, size_t dpitch,
                                                            const char *__restrict__ src, size_t spitch,
                                                            size_t n) {
  const T *s = (const T *)(src + (size_t)blockIdx.y * spitch);
  T *d = (T *)(dst + (size_t)blockIdx.y * dpitch);
  const size_t step = (size_t)gridDim.x * kCopyThreads * kCopyUnroll;
  for (size_t i0 = (size_t)blockIdx.x * kCopyThreads * kCopyUnroll + threadIdx.x; i0 < n; i0 += step) {
    T v[kCopyUnroll];
#pragma unroll
    for (int u = 0; u < kCopyUnroll; ++u) {
      const size_t i = i0 + (size_t)u * kCopyThreads;
      if (i < n) v[u] = s[i];
    }
#pragma unroll
    for (int u = 0; u < kCopyUnroll; ++u) {
      const size_t i = i0 + (size_t)u * kCopyThreads;
      if (i < n) d[i] = v[u];
    }
  }
}

// 0: the copy engines for every copy; 1 (default): a copy kernel for both
// directions where the host memory is addressable by the device; 2: the copy
// kernel device to host, the copy engines host to device.  Policy 2 frees the
// copy kernel's SM slots while a synthesis call's host-to-device copies
// overlap the next analysis call (118 against 130 ms per pipelined round trip
// of 32 maps at L=1024 in most steps), but over 20 steps the engines' slow
// stretches hit several synthesis calls (260-378 ms instead of 118) and it lost
// overall.  S2LET_GPU_HOST_COPY=engine selects 0, =d2h_kernel 2.
int copy_policy() {
  static const int p = [] {
    const char *e = getenv("S2LET_GPU_HOST_COPY");
    if (e && strcmp(e, "engine") == 0) return 0;
    if (e && strcmp(e, "d2h_kernel") == 0) return 2;
    return 1;
  }();
  return p;
}

// True when a kernel may dereference host address `h`: page-locked memory
// mapped into the device's address space at the same address (the unified
// address space of 64-bit hosts).  Pageable and managed memory go to the copy
// engines.
bool device_addressable(const void *h) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, h) != cudaSuccess) {
    cudaGetLastError();  // clear the non-sticky error of an unknown pointer
    return false;
  }
  return at.type == cudaMemoryTypeHost && at.devicePointer == h;
}

// CTAs per copy: kCopyBlocks, or S2LET_GPU_COPY_CTAS (1-1024).  Measured on
// the pipelined host batches at L=1024 (32 maps per call): 64 CTAs 239
// maps/s, 32 CTAs 232, 16 CTAs 201 (fewer copy CTAs slow the copies more than
// they help the transforms).
int copy_blocks() {
  static const int b = [] {
    const char *e = getenv("S2LET_GPU_COPY_CTAS");
    const int v = e ? atoi(e) : 0;
    return (v >= 1 && v <= 1024) ? v : kCopyBlocks;
  }();
  return b;
}

template <class T>
void launch_rows(void *dst, size_t dpitch, const void *src, size_t spitch, size_t width, size_t height,
                 cudaStream_t st) {
  const size_t n = width / sizeof(T);
  const size_t per = (size_t)kCopyThreads * kCopyUnroll;
  const size_t want = (n + per - 1) / per;
  const int nblk = copy_blocks();
  int bx = (int)(want < (size_t)nblk ? want : (size_t)nblk);
  if (height > 1) bx = (bx + (int)height - 1) / (int)height;  // about nblk CTAs in all
  if (bx < 1) bx = 1;
  k_copy_rows<T><<<dim3(bx, (unsigned)height), kCopyThreads, 0, st>>>((char *)dst, dpitch, (const char *)src,
                                                                       spitch, n);
  S2G_LAUNCHED();
}

// a copy kernel when the host side is addressable and the rows fit its grid
bool copy_by_kernel(void *dst, size_t dpitch, const void *src, size_t spitch, size_t width, size_t height,
                    cudaMemcpyKind kind, cudaStream_t st) {
  if (copy_policy() == 0 || height > 65535) return false;
  if (copy_policy() == 2 && kind == cudaMemcpyHostToDevice) return false;
  if (kind != cudaMemcpyHostToDevice && kind != cudaMemcpyDeviceToHost) return false;
  if (!device_addressable(kind == cudaMemcpyHostToDevice ? src : dst)) return false;
  if (height == 1) dpitch = spitch = width;
  const uintptr_t all = (uintptr_t)dst | (uintptr_t)src | dpitch | spitch | width;
  if (all % 16 == 0)
    launch_rows<uint4>(dst, dpitch, src, spitch, width, height, st);
  else if (all % 8 == 0)
    launch_rows<uint2>(dst, dpitch, src, spitch, width, height, st);
  else if (all % 4 == 0)
    launch_rows<uint32_t>(dst, dpitch, src, spitch, width, height, st);
  else
    launch_rows<uint8_t>(dst, dpitch, src, spitch, width, height, st);
  return true;
}

}  // namespace

void copy_async(void *dst, size_t dpitch, const void *src, size_t spitch, size_t width, size_t height,
                cudaMemcpyKind kind, cudaStream_t st) {
  if (width == 0 || height == 0) return;
  const CopyMark m = copy_trace_begin(kind, (double)width * (double)height, st);
  const bool by_kernel = copy_by_kernel(dst, dpitch, src, spitch, width, height, kind, st);
  if (!by_kernel) {
    if (height == 1)
      S2G_CUDA(cudaMemcpyAsync(dst, src, width, kind, st));
    else
      S2G_CUDA(cudaMemcpy2DAsync(dst, dpitch, src, spitch, width, height, kind, st));
  }
  copy_trace_end(m, by_kernel, st);
}

}  // namespace s2g
