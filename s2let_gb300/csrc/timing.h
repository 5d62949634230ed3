// Optional per-kernel timing: CUDA events recorded on the launching stream
// around each instrumented launch, with the launch's algorithmic work (flops,
// bytes) attached.  Off by default; s2let_gpu_timing_enable() switches it on.
#pragma once

#include <cuda_runtime.h>

namespace s2g {

enum KCat {
  KC_CONTRACT = 0,  // Wigner/Legendre contractions on stored tables (FP64; double-float at split precision)
  KC_RING = 1,      // Bluestein ring DFTs
  KC_GAMMA = 2,     // gamma DFTs
  KC_MERGE = 3,     // tiling merge / split / symmetrise
  KC_MIXED = 4,     // split-precision tensor-core contractions
  KC_OTHER = 5,
  KC_RECOMPUTE = 6,  // FP64 contractions regenerating the Wigner values (recomputed tables)
  KC_QUAD = 7,       // forward quadrature operator applied to ring spectra (recomputed tables)
  KC_SLICE = 8,      // digit slicing of the coefficients for the tensor-core contractions
  KC_N = 9
};

bool timing_enabled();

// Copy trace (s2let_gpu_copy_trace_enable): while tracing is on, begin/end
// record CUDA events on st around one host<->device copy of `bytes`; off, they
// do nothing.
struct CopyMark {
  cudaEvent_t a = nullptr, b = nullptr;
  int d2h = 0;
  double bytes = 0;
};
CopyMark copy_trace_begin(cudaMemcpyKind kind, double bytes, cudaStream_t st);
// by_kernel: the copy was made by the copy kernel (else by the copy engines)
void copy_trace_end(const CopyMark &m, bool by_kernel, cudaStream_t st);

// One host<->device copy of the host-pointer entry points (a plain copy when
// height == 1, else `height` rows of `width` bytes at the given pitches),
// asynchronous on st, traced as above (hostcopy.cu).  Host memory that the
// GPU can address (page-locked, or any memory where the device accesses
// pageable memory) is moved by a copy kernel; other memory by the copy engines.
void copy_async(void *dst, size_t dpitch, const void *src, size_t spitch, size_t width, size_t height,
                cudaMemcpyKind kind, cudaStream_t st);

class KTimer {
 public:
  KTimer(int cat, cudaStream_t st, double flops, double bytes);
  ~KTimer();

 private:
  int slot_ = -1;
  cudaStream_t st_ = nullptr;
};

}  // namespace s2g
