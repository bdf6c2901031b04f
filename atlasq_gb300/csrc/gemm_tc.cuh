// Tensor-core (tcgen05, 3xTF32) batched complex64 GEMM over GemmProb problems.
#pragma once
#include "gemm.cuh"

// Device scratch for the packed split operands of `count` problems bounded by
// maxM x maxN x maxK.
size_t tc_gemm_scratch_bytes(int count, int maxM, int maxN, int maxK);
// Pack + GEMM.  `status` (device int) receives AGB_ERR_TIMEOUT if a bounded
// wait expired; it is not cleared here.
int launch_gemm_tc(const GemmProb* probs, int count, int maxM, int maxN, int maxK, void* scratch,
                   size_t scratch_bytes, int* status, cudaStream_t s);
