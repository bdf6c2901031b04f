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

// Launch the SIMT tile kernel over `count` problems whose M, N are bounded by
// maxM, maxN (tiles beyond a problem's own extent exit early).
template <typename CX>
int launch_gemm_probs(const GemmProb* probs, int count, int maxM, int maxN, cudaStream_t s);
