// Split-precision Legendre/Wigner contraction on the tcgen05 tensor cores.
//
// Every FP64 operand row (a table row, a coefficient column) is written as
// 2^e * sum_{i<7} d_i 2^{-6-7i} with integer digits |d_i| <= 64 held exactly in
// bf16.  The 28 digit products with i + j <= 6 are accumulated in FP32 by
// tcgen05.mma; a class c = i + j sums at most c + 1 products of magnitude
// <= 2^12 over K <= 1024 terms, so classes 0..2 are exact integers and the
// rounding of the others sits below 2^-45 of the result.  The epilogue
// combines the classes in FP64.  Truncation error: about 2^-41 of
// max|row| * max|column| per term (measured 2.5e-12 normwise on adversarial
// synthetic rows; the FP64 oracle tolerance of the path is 1e-10).
#pragma once

#include <cuda_runtime.h>

#include "kernels.h"

namespace s2g {

// True when the contraction ran on the tensor cores; false when the problem is
// outside the split-precision kernel's domain (small band-limit, adjoint table
// orientation) and the caller must run the FP64 kernel.
// nparts (1 or 2) problems that differ only in their coefficients, weights,
// lmin and outputs (scales sharing one band-limit and n) share one pass over
// the table.
bool contract_l2t_mixed(const L2T *a, int nparts, cudaStream_t st);
bool contract_t2l_mixed(const T2L *a, int nparts, cudaStream_t st);

void release_sliced_tables();
size_t sliced_table_bytes();
// Reads and clears the device flag raised by a split-precision launch whose
// bounded wait expired (1: pipeline wait, 2: MMA drain); 0 when none did.
int mixed_error_flag_read_and_clear();

// Contraction precision of the calling host thread (0 FP64, 1 split precision).
extern thread_local int t_precision;

}  // namespace s2g
