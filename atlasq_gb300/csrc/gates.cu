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

// Many single-qubit gates in one launch.  desc (device, int64):
//   [ngroups][5] = {T, chiL, chiR, first, count}, then the gate pointers
//   [sum of counts] (each a 2x2 matrix of the tensor's type).
// Group g applies its `count` gates to tensor T in order; gates of one site
// compose element-wise (each (a, b) fibre is transformed independently), so a
// thread applies the whole chain to its fibre in registers.
constexpr int SQ_CHUNK = 64;
template <typename CX>
__global__ void __launch_bounds__(256) single_qubit_batch_kernel(const int64_t* __restrict__ desc, int ngroups) {
  __shared__ CX su[SQ_CHUNK * 4];
  const int64_t* G = desc + (int64_t)blockIdx.y * 5;
  CX* T = (CX*)G[0];
  // chiL < 0: device-resident tensor; G[2] then points at its two bond
  // dimensions (left, right) in the instance's int32 dimension array
  const bool res = G[1] < 0;
  const int chiL = res ? ((const int*)G[2])[0] : (int)G[1];
  const int chiR = res ? ((const int*)G[2])[1] : (int)G[2];
  const int64_t first = G[3];
  const int cnt = (int)G[4];
  const int64_t* up = desc + (int64_t)ngroups * 5 + first;
  const int64_t n = (int64_t)chiL * chiR;
  for (int c0 = 0; c0 < cnt; c0 += SQ_CHUNK) {
    const int cc = min(SQ_CHUNK, cnt - c0);
    __syncthreads();
    for (int t = threadIdx.x; t < cc * 4; t += blockDim.x) su[t] = ((const CX*)up[c0 + t / 4])[t % 4];
    __syncthreads();
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
      const int64_t a = i / chiR, b = i % chiR;
      CX* p0 = T + (a * 2 + 0) * chiR + b;
      CX* p1 = T + (a * 2 + 1) * chiR + b;
      CX t0 = *p0, t1 = *p1;
      for (int g = 0; g < cc; ++g) {
        const CX* u = su + 4 * g;
        CX r0 = czero<CX>(), r1 = czero<CX>();
        cfma(r0, u[0], t0);
        cfma(r0, u[2], t1);
        cfma(r1, u[1], t0);
        cfma(r1, u[3], t1);
        t0 = r0;
        t1 = r1;
      }
      *p0 = t0;
      *p1 = t1;
    }
  }
}
}  // namespace

extern "C" int agb_single_qubit_batch(int dtype, int ngroups, const int64_t* desc, int max_elems, void* stream) {
  if (dtype != AGB_C64 && dtype != AGB_C128) return AGB_ERR_ARG;
  if (ngroups < 0 || ngroups > 65535 || max_elems < 0) return AGB_ERR_ARG;
  if (ngroups == 0) return AGB_OK;
  if (!desc || max_elems == 0) return AGB_ERR_ARG;
  int bx = (max_elems + 255) / 256;
  if (bx > 64) bx = 64;
  const dim3 grid(bx, ngroups);
  cudaStream_t s = (cudaStream_t)stream;
  if (dtype == AGB_C64) single_qubit_batch_kernel<float2><<<grid, 256, 0, s>>>(desc, ngroups);
  else single_qubit_batch_kernel<double2><<<grid, 256, 0, s>>>(desc, ngroups);
  AGB_CHECK_LAUNCH();
  return AGB_OK;
}

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
