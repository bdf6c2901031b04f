// Sampling and expectation helper kernels (sm_103a).
//
// Sampling (replaces _batch_sweep_sample, src/atlas_q/mps_pytorch.py:247-355):
// per site the host computes temp = L @ T.reshape(chiL, 2 chiR) with the GEMM;
// agb_sample_site then, per shot (one warp each),
//   p_s = sum |temp[shot, s*chiR : (s+1)*chiR]|^2 (double accumulation),
//   p_s += 1e-15 (the reference's floor, :313), pz = p0 / (p0 + p1),
//   u = Philox4x32-10((shot, shot>>32, site, 0), seed) word0 >> 8 * 2^-24,
//   outcome = u >= pz; bits = bits << 1 | outcome (qubit 0 = MSB, :321),
//   L_new = temp[shot, outcome*chiR : ...]  (left state kept unnormalised, :342-352).
//
// Expectations (replaces the einsum of expectation_value, src/atlas_q/mpo_ops.py:1145):
// E'[r,B] = sum E[a,b] conj(A[a,t,r]) W[L,s,t,R] A[b,s,B] is evaluated as
//   M_L = E_L @ A.reshape(chiA, 2 chiB)               (GEMM)
//   N_R[(a,t),B] = sum_{L,s} W[L,s,t,R] M_L[a,(s,B)]  (agb_mpo_mix, this file)
//   E'_R = A.reshape(2 chiA, chiB)^H @ N_R            (GEMM)
#include "common.cuh"

namespace {

template <typename CX>
__global__ void sample_site_kernel(const CX* __restrict__ temp, int shots, int chiR, int site,
                                   uint64_t seed, uint64_t shot_offset, int64_t* __restrict__ bits,
                                   CX* __restrict__ Lnew, double* __restrict__ pz_out) {
  const int lane = threadIdx.x & 31;
  const int s = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (s >= shots) return;
  const CX* row = temp + (int64_t)s * 2 * chiR;
  double p0 = 0, p1 = 0;
  for (int c = lane; c < chiR; c += 32) {
    p0 += (double)cabs2(row[c]);
    p1 += (double)cabs2(row[chiR + c]);
  }
  p0 = warp_sum(p0) + 1e-15;
  p1 = warp_sum(p1) + 1e-15;
  const double pz = p0 / (p0 + p1);
  const uint64_t shot = shot_offset + (uint64_t)s;
  const philox_out o = philox4x32_10((uint32_t)shot, (uint32_t)(shot >> 32), (uint32_t)site, 0u,
                                     (uint32_t)seed, (uint32_t)(seed >> 32));
  const double u = (double)(o.x >> 8) * (1.0 / 16777216.0);
  const int outc = (u >= pz) ? 1 : 0;
  if (lane == 0) {
    bits[s] = (bits[s] << 1) | outc;
    if (pz_out) pz_out[s] = pz;
  }
  if (Lnew) {
    const CX* src = row + outc * chiR;
    for (int c = lane; c < chiR; c += 32) Lnew[(int64_t)s * chiR + c] = src[c];
  }
}

// N[R][a][t][B] = sum_{L,s} W[L][s][t][R] * M[L][a][s][B]
template <typename CX>
__global__ void mpo_mix_kernel(const CX* __restrict__ M, const CX* __restrict__ W, CX* __restrict__ N,
                               int Lw, int Rw, int chiA, int chiB) {
  const int64_t per = (int64_t)chiA * 2 * chiB;
  const int64_t total = per * Rw;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int R = (int)(i / per);
    const int64_t rem = i % per;
    const int a = (int)(rem / (2 * chiB));
    const int t = (int)((rem / chiB) % 2);
    const int B = (int)(rem % chiB);
    CX acc = czero<CX>();
    for (int L = 0; L < Lw; ++L)
#pragma unroll
      for (int s = 0; s < 2; ++s) {
        const CX w = W[((L * 2 + s) * 2 + t) * Rw + R];
        if (w.x != 0 || w.y != 0)
          cfma(acc, w, M[(int64_t)L * per + ((int64_t)a * 2 + s) * chiB + B]);
      }
    N[i] = acc;
  }
}

// out = sum_{r,c} E[r,c] * Q[c,r]   (one block, double accumulation)
template <typename CX>
__global__ void trace_prod_kernel(const CX* __restrict__ E, const CX* __restrict__ Q, int n, double* out) {
  __shared__ double red[32];
  double re = 0, im = 0;
  for (int64_t i = threadIdx.x; i < (int64_t)n * n; i += blockDim.x) {
    const int r = (int)(i / n), c = (int)(i % n);
    const CX a = E[i], b = Q[(int64_t)c * n + r];
    re += (double)a.x * b.x - (double)a.y * b.y;
    im += (double)a.x * b.y + (double)a.y * b.x;
  }
  re = block_sum(re, red);
  im = block_sum(im, red);
  if (threadIdx.x == 0) {
    out[0] = re;
    out[1] = im;
  }
}

}  // namespace

extern "C" int agb_sample_site(int dtype, const void* temp, int shots, int chiR, int site, uint64_t seed,
                               uint64_t shot_offset, int64_t* bits, void* Lnew, double* pz_out,
                               void* stream) {
  if (dtype != AGB_C64 && dtype != AGB_C128) return AGB_ERR_ARG;
  if (shots < 0 || chiR <= 0 || !temp || !bits) return AGB_ERR_ARG;
  if (shots == 0) return AGB_OK;
  const int wpb = 8;
  dim3 grid((shots + wpb - 1) / wpb);
  cudaStream_t s = (cudaStream_t)stream;
  if (dtype == AGB_C64)
    sample_site_kernel<float2><<<grid, 32 * wpb, 0, s>>>((const float2*)temp, shots, chiR, site, seed,
                                                         shot_offset, bits, (float2*)Lnew, pz_out);
  else
    sample_site_kernel<double2><<<grid, 32 * wpb, 0, s>>>((const double2*)temp, shots, chiR, site, seed,
                                                          shot_offset, bits, (double2*)Lnew, pz_out);
  AGB_CHECK_LAUNCH();
  return AGB_OK;
}

extern "C" int agb_mpo_mix(int dtype, const void* M, const void* W, void* N, int Lw, int Rw, int chiA,
                           int chiB, void* stream) {
  if (dtype != AGB_C64 && dtype != AGB_C128) return AGB_ERR_ARG;
  if (!M || !W || !N || Lw <= 0 || Rw <= 0 || chiA <= 0 || chiB <= 0) return AGB_ERR_ARG;
  const int64_t total = (int64_t)Rw * chiA * 2 * chiB;
  int blocks = (int)((total + 255) / 256);
  if (blocks > 4096) blocks = 4096;
  cudaStream_t s = (cudaStream_t)stream;
  if (dtype == AGB_C64)
    mpo_mix_kernel<float2><<<blocks, 256, 0, s>>>((const float2*)M, (const float2*)W, (float2*)N, Lw, Rw, chiA, chiB);
  else
    mpo_mix_kernel<double2><<<blocks, 256, 0, s>>>((const double2*)M, (const double2*)W, (double2*)N, Lw, Rw, chiA, chiB);
  AGB_CHECK_LAUNCH();
  return AGB_OK;
}

extern "C" int agb_trace_prod(int dtype, const void* E, const void* Q, int n, double* out2, void* stream) {
  if (dtype != AGB_C64 && dtype != AGB_C128) return AGB_ERR_ARG;
  if (!E || !Q || !out2 || n <= 0) return AGB_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  if (dtype == AGB_C64) trace_prod_kernel<float2><<<1, 1024, 0, s>>>((const float2*)E, (const float2*)Q, n, out2);
  else trace_prod_kernel<double2><<<1, 1024, 0, s>>>((const double2*)E, (const double2*)Q, n, out2);
  AGB_CHECK_LAUNCH();
  return AGB_OK;
}
