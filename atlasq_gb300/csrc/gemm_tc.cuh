// Tensor-core (tcgen05, 3xTF32) batched complex64 GEMM over GemmProb problems.
#pragma once
#include "gemm.cuh"

// Device scratch of the tensor-core path for `count` problems bounded by
// maxM x maxN x maxK (the split operands live in shared memory only, so this
// is a small constant the dispatcher checks for).
size_t tc_gemm_scratch_bytes(int count, int maxM, int maxN, int maxK);
// The GEMM (operand split fused into the kernel).  `status` (device int)
// receives AGB_ERR_TIMEOUT if a bounded wait expired; it is not cleared here.
int launch_gemm_tc(const GemmProb* probs, int count, int maxM, int maxN, int maxK, void* scratch,
                   size_t scratch_bytes, int* status, cudaStream_t s);
