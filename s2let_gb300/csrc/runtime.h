// Runtime helpers shared by the C-ABI translation units: per-thread status,
// stream-ordered scratch, host<->device staging of the drop-in entry points.
#pragma once

#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <new>
#include <string>
#include <utility>
#include <vector>

#include "common.h"

namespace s2g {

void set_status(int code, const std::string &msg);
void report_failure();  // prints the status; exits when S2LET_GPU_ABORT_ON_ERROR=1
int last_status();
void ensure_device();   // throws ERR_NO_DEVICE without a usable GPU
cudaStream_t host_stream();  // per-thread stream of the host-pointer entry points

// Runs `body`, turning exceptions into the thread's status (never exits unless asked to).
template <class F>
int guarded(const char *fn, F &&body) {
  try {
    body();
    set_status(OK, "");
    return OK;
  } catch (const Error &e) {
    set_status(e.code, std::string(fn) + ": " + e.what());
  } catch (const std::bad_alloc &) {
    set_status(ERR_NOMEM, std::string(fn) + ": host allocation failed");
  } catch (const std::exception &e) {
    set_status(ERR_CUDA, std::string(fn) + ": " + e.what());
  }
  report_failure();
  return last_status();
}

// Stream-ordered device scratch, released (stream-ordered) when it goes out of scope.
struct Scratch {
  cudaStream_t st;
  std::vector<void *> ptrs;
  explicit Scratch(cudaStream_t s) : st(s) {}
  Scratch(const Scratch &) = delete;
  Scratch &operator=(const Scratch &) = delete;
  template <class T>
  T *get(int64_t n) {
    void *p = nullptr;
    S2G_CUDA(cudaMallocAsync(&p, sizeof(T) * (size_t)(n > 0 ? n : 1), st));
    ptrs.push_back(p);
    return (T *)p;
  }
  ~Scratch() {
    for (void *p : ptrs) cudaFreeAsync(p, st);
  }
};

// Host <-> device staging for the host-pointer entry points.
struct Staged {
  Scratch &S;
  std::vector<std::pair<void *, std::pair<void *, size_t>>> outs;  // (host, (dev, bytes))
  explicit Staged(Scratch &s) : S(s) {}
  template <class T>
  T *in(const void *h, int64_t n) {
    T *d = S.get<T>(n);
    if (n > 0) S2G_CUDA(cudaMemcpyAsync(d, h, sizeof(T) * n, cudaMemcpyHostToDevice, S.st));
    return d;
  }
  template <class T>
  T *out(void *h, int64_t n) {
    T *d = S.get<T>(n);
    if (n > 0) outs.push_back({h, {d, sizeof(T) * (size_t)n}});
    return d;
  }
  template <class T>  // read-modify-write buffer
  T *inout(void *h, int64_t n) {
    T *d = in<T>(h, n);
    if (n > 0) outs.push_back({h, {d, sizeof(T) * (size_t)n}});
    return d;
  }
  void finish() {
    for (auto &o : outs)
      S2G_CUDA(cudaMemcpyAsync(o.first, o.second.first, o.second.second, cudaMemcpyDeviceToHost, S.st));
    S2G_CUDA(cudaStreamSynchronize(S.st));
  }
};

}  // namespace s2g
