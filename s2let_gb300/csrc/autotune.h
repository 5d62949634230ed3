// Launch shapes picked by measurement: per kernel family and problem bucket,
// the candidates are timed once on the live call, the fastest is kept in
// memory and in a cache file (one line per choice, keyed by the GPU model),
// and later calls and processes launch it directly.
#pragma once

#include <cuda_runtime.h>

#include <functional>

namespace s2g {

enum TuneFamily {
  TF_CONTRACT = 1,  // FP64 contraction k_contract: maps per CTA
  TF_RC_L2T = 2,    // recomputed-table contraction l -> t: maps per CTA
  TF_RC_T2L = 3,    // recomputed-table contraction t -> l: maps per CTA
  TF_MIXED = 4,     // split-precision contraction: columns per table pass and map groups per launch
};

// Index of the candidate to launch, in [0, ncand).  Tuning on
// (s2let_gpu_autotune(1) or S2LET_GPU_AUTOTUNE=1): for a key (family, a, b, c)
// not seen before, on a stream that is not being captured, every candidate is
// run through trial(i) (which enqueues candidate i on st) once to warm up and
// kTuneReps times between CUDA events, the host waits for the events, and the
// fastest is recorded; the caller then launches the returned candidate as
// usual.  trial must be idempotent (every candidate writes the same outputs).
// Tuning off, or while st is being captured: the recorded choice for the key
// if there is one, else def.
int tuned(int family, int a, int b, int c, int ncand, int def, cudaStream_t st,
          const std::function<void(int)> &trial);

// current mode (0 off, 1 tuning on), for caches keyed by the launch shapes
int autotune_mode();

// power-of-two bucket of a size (the key's granularity)
inline int tune_bucket(int x) {
  int b = 1;
  while (b < x) b <<= 1;
  return b;
}

}  // namespace s2g
