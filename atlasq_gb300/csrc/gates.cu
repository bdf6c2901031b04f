// Single-site kernels: the single-qubit gate (reference convention U^T).
#include "common.cuh"

namespace {
// T'[a,t,b] = sum_s U[s,t] T[a,s,b]   (adaptive_mps.py:177, einsum "st,asb->atb")
template <typename CX>
__global__ void single_qubit_kernel(CX* T, const CX* __restrict__ U, int chiL, int chiR) {
  const int64_t n = (int64_t)chiL * chiR;
  const CX u00 = U[0], u01 = U[1], u10 = U[2], u11 = U[3];
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t a = i / chiR, b = i % chiR;
    CX* p0 = T + (a * 2 + 0) * chiR + b;
    CX* p1 = T + (a * 2 + 1) * chiR + b;
    const CX t0 = *p0, t1 = *p1;
    CX r0 = czero<CX>(), r1 = czero<CX>();
    cfma(r0, u00, t0);  // t = 0: U[0,0] T[.,0,.] + U[1,0] T[.,1,.]
    cfma(r0, u10, t1);
    cfma(r1, u01, t0);  // t = 1: U[0,1] T[.,0,.] + U[1,1] T[.,1,.]
    cfma(r1, u11, t1);
    *p0 = r0;
    *p1 = r1;
  }
}
}  // namespace

extern "C" int agb_single_qubit_gate(int dtype, void* T, const void* U, int chiL, int chiR, void* stream) {
  if (dtype != AGB_C64 && dtype != AGB_C128) return AGB_ERR_ARG;
  if (!T || !U || chiL <= 0 || chiR <= 0) return AGB_ERR_ARG;
  const int64_t n = (int64_t)chiL * chiR;
  int blocks = (int)((n + 255) / 256);
  if (blocks > 1184) blocks = 1184;
  cudaStream_t s = (cudaStream_t)stream;
  if (dtype == AGB_C64) single_qubit_kernel<float2><<<blocks, 256, 0, s>>>((float2*)T, (const float2*)U, chiL, chiR);
  else single_qubit_kernel<double2><<<blocks, 256, 0, s>>>((double2*)T, (const double2*)U, chiL, chiR);
  AGB_CHECK_LAUNCH();
  return AGB_OK;
}
