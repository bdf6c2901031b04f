// Batched complex GEMM problems: D = alpha * op(A) op(B) + beta * Csrc.
// Each batch entry is a GemmProb in device memory, so kernels that build the
// problems on the device (from gate descriptors) and the host API share one
// launcher.  op: 0 = N, 1 = T, 2 = C (conjugate transpose).
#pragma once
#include "common.cuh"

struct GemmProb {
  const void* A;
  const void* B;
  void* D;
  const void* Csrc;  // may alias D; ignored when beta == 0
  int64_t lda, ldb, ldd, ldc;
  int M, N, K;
  int opA, opB;
  double alpha_re, alpha_im, beta_re, beta_im;
};

// Optional tensor-core context: the tensor-core path's scratch token and a
// device status word.  With a context whose scratch is large enough,
// complex64 problems of at least 64 x 64 x 32 run on tcgen05 (gemm_tc.cu);
// everything else runs on the SIMT kernel.
struct GemmCtx {
  void* tc_scratch = nullptr;
  size_t tc_bytes = 0;
  int* status = nullptr;
};

// Launch over `count` problems whose M, N, K are bounded by maxM, maxN, maxK
// (tiles beyond a problem's own extent exit early).
template <typename CX>
int launch_gemm_probs(const GemmProb* probs, int count, int maxM, int maxN, cudaStream_t s,
                      const GemmCtx* ctx = nullptr, int maxK = 0);
