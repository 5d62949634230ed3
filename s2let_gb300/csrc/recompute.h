// Contractions against recomputed (checkpointed) Wigner tables (WignerTable::rc),
// FP64: the same operators as contract_l2t / contract_t2l with the table values
// regenerated in the kernels instead of read from memory.
#pragma once

#include <cuda_runtime.h>

#include "kernels.h"

namespace s2g {

void contract_l2t_rc(const L2T &p, cudaStream_t st);
void contract_t2l_rc(const T2L &p, cudaStream_t st);

}  // namespace s2g
