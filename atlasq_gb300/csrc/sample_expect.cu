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
  typedef typename cx_traits<CX>::R R;
  const CX* row = temp + (int64_t)s * 2 * chiR;
  // both probabilities to double accuracy on the FP32 pipe; the decision
  // (double division, Philox) runs once per shot, in lane 0
  SumAcc<R> a0, a1;
  for (int c = lane; c < chiR; c += 32) {
    a0.add(cabs2(row[c]));
    a1.add(cabs2(row[chiR + c]));
  }
  a0.warp_reduce();
  a1.warp_reduce();
  int outc = 0;
  if (lane == 0) {
    const double p0 = a0.value() + 1e-15, p1 = a1.value() + 1e-15;
    const double pz = p0 / (p0 + p1);
    const uint64_t shot = shot_offset + (uint64_t)s;
    const philox_out o = philox4x32_10((uint32_t)shot, (uint32_t)(shot >> 32), (uint32_t)site, 0u,
                                       (uint32_t)seed, (uint32_t)(seed >> 32));
    const double u = (double)(o.x >> 8) * (1.0 / 16777216.0);
    outc = (u >= pz) ? 1 : 0;
    bits[s] = (bits[s] << 1) | outc;
    if (pz_out) pz_out[s] = pz;
  }
  outc = __shfl_sync(0xffffffffu, outc, 0);
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

// N[g][a][t][b] = sum_s W[g][s][t] M[g][a][s][b]   (W: one 2x2 operator per item)
template <typename CX>
__global__ void site_mix_kernel(const CX* __restrict__ M, const CX* __restrict__ W, CX* __restrict__ N, int count,
                                int chiA, int chiB) {
  const int64_t per = (int64_t)chiA * 2 * chiB;
  const int g = blockIdx.y;
  if (g >= count) return;
  const CX w00 = W[g * 4 + 0], w01 = W[g * 4 + 1], w10 = W[g * 4 + 2], w11 = W[g * 4 + 3];
  const CX* Mg = M + (int64_t)g * per;
  CX* Ng = N + (int64_t)g * per;
  const int64_t half = (int64_t)chiA * chiB;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < half; i += (int64_t)gridDim.x * blockDim.x) {
    const int a = (int)(i / chiB), b = (int)(i % chiB);
    const CX m0 = Mg[((int64_t)a * 2 + 0) * chiB + b], m1 = Mg[((int64_t)a * 2 + 1) * chiB + b];
    CX n0 = czero<CX>(), n1 = czero<CX>();
    cfma(n0, w00, m0);  // t = 0: W[0][0] M[s=0] + W[1][0] M[s=1]
    cfma(n0, w10, m1);
    cfma(n1, w01, m0);  // t = 1
    cfma(n1, w11, m1);
    Ng[((int64_t)a * 2 + 0) * chiB + b] = n0;
    Ng[((int64_t)a * 2 + 1) * chiB + b] = n1;
  }
}

// out = sum_{r,c} E[r,c] * Q[c,r]   (one block of 32 x 32 threads, double
// accuracy).  32 x 32 tiles, two in flight per barrier: thread (ty, tx) takes
// E[r0 + ty][c0 + tx] (coalesced) and Q[c0 + tx][r0 + ty] from a tile of Q
// staged row-wise (coalesced) in shared memory.
template <typename CX>
__global__ void __launch_bounds__(1024) trace_prod_kernel(const CX* __restrict__ E, const CX* __restrict__ Q,
                                                          int n, double* out) {
  typedef typename cx_traits<CX>::R R;
  __shared__ CX qs[2][32][33];
  __shared__ double red[32];
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const int nb = (n + 31) / 32, ntile = nb * nb;
  SumAcc<R> re, im;
  for (int t0 = 0; t0 < ntile; t0 += 2) {
    CX ev[2];
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      const int t = t0 + u;
      CX qv = czero<CX>();
      ev[u] = czero<CX>();
      if (t < ntile) {
        const int r0 = (t / nb) * 32, c0 = (t % nb) * 32;
        if (c0 + ty < n && r0 + tx < n) qv = Q[(int64_t)(c0 + ty) * n + r0 + tx];
        if (r0 + ty < n && c0 + tx < n) ev[u] = E[(int64_t)(r0 + ty) * n + c0 + tx];
      }
      qs[u][ty][tx] = qv;
    }
    __syncthreads();
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      const CX a = ev[u], b = qs[u][tx][ty];
      re.add_prod(a.x, b.x);
      re.add_prod(-a.y, b.y);
      im.add_prod(a.x, b.y);
      im.add_prod(a.y, b.x);
    }
    __syncthreads();
  }
  const double sre = block_sum(re.value(), red);
  const double sim = block_sum(im.value(), red);
  if (threadIdx.x == 0) {
    out[0] = sre;
    out[1] = sim;
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

extern "C" int agb_site_mix(int dtype, const void* M, const void* W, void* N, int count, int chiA, int chiB,
                            void* stream) {
  if (dtype != AGB_C64 && dtype != AGB_C128) return AGB_ERR_ARG;
  if (!M || !W || !N || count < 0 || count > 65535 || chiA <= 0 || chiB <= 0) return AGB_ERR_ARG;
  if (count == 0) return AGB_OK;
  const int64_t half = (int64_t)chiA * chiB;
  int bx = (int)((half + 255) / 256);
  if (bx > 256) bx = 256;
  const dim3 grid(bx, count);
  cudaStream_t s = (cudaStream_t)stream;
  if (dtype == AGB_C64)
    site_mix_kernel<float2><<<grid, 256, 0, s>>>((const float2*)M, (const float2*)W, (float2*)N, count, chiA, chiB);
  else
    site_mix_kernel<double2><<<grid, 256, 0, s>>>((const double2*)M, (const double2*)W, (double2*)N, count, chiA,
                                                  chiB);
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
