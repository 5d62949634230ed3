// Shared infrastructure of libs2let_gpu.so: status reporting, CUDA checks,
// launch counting, small device math helpers.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <cstdio>
#include <stdexcept>
#include <string>

namespace s2g {

// Error carried from any depth of the host code to the C-ABI boundary, where it
// becomes the thread's status (s2let_gpu_last_error) instead of exit(1).
struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

enum Status {
  OK = 0,
  ERR_INVALID = 1,
  ERR_UNSUPPORTED = 2,
  ERR_CUDA = 3,
  ERR_NOMEM = 4,
  ERR_NO_DEVICE = 5,
};

#define S2G_CUDA(call)                                                                      \
  do {                                                                                      \
    cudaError_t e_ = (call);                                                                \
    if (e_ != cudaSuccess) {                                                                \
      int code_ = (e_ == cudaErrorMemoryAllocation) ? ::s2g::ERR_NOMEM : ::s2g::ERR_CUDA;   \
      throw ::s2g::Error(code_, std::string(#call) + ": " + cudaGetErrorString(e_));       \
    }                                                                                       \
  } while (0)

#define S2G_REQUIRE(cond, code, msg)                                                        \
  do {                                                                                      \
    if (!(cond)) throw ::s2g::Error((code), (msg));                                         \
  } while (0)

// Counts this library's kernel launches (instrumentation for the bench's
// gpu_launches field).
extern std::atomic<uint64_t> g_launches;

#define S2G_LAUNCHED()                                                                      \
  do {                                                                                      \
    ::s2g::g_launches.fetch_add(1, std::memory_order_relaxed);                              \
    cudaError_t e_ = cudaPeekAtLastError();                                                 \
    if (e_ != cudaSuccess)                                                                  \
      throw ::s2g::Error(::s2g::ERR_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e_)); \
  } while (0)

inline int ceil_div(int64_t a, int64_t b) { return (int)((a + b - 1) / b); }

constexpr double kPi = 3.141592653589793238462643383279502884197;

}  // namespace s2g
