// MPO x MPS site products and the TDVP local-operator contraction (sm_103a).
//
//   mpo_apply_site   out[(l, a), s, (r, b)] = sum_t W[l, s, t, r] A[a, t, b]
//                    (the per-site contraction of apply_mpo_to_mps; bond
//                    dimensions multiply, nothing is truncated)
//   tdvp_local_h     H[i, t, j] = sum_{l,s,n} Lsum[l, i] W[l, s, t, n] A[i, s, j] Rsum[n, j],
//                    Lsum[l, i] = sum_q L[q, l, i], Rsum[n, j] = sum_u R[u, n, j]
//                    (the index pattern of the reference's local step,
//                    'qli, lstn, isj, unj -> itj': i and j are shared by the
//                    environments and the site tensor, q and u are summed)
// Both are bandwidth-bound elementwise passes (two or 2 Dl Dn terms per output).
#include "common.cuh"

namespace {

template <typename CX>
__global__ void mpo_apply_site_kernel(const CX* __restrict__ W, const CX* __restrict__ A, CX* __restrict__ out,
                                      int Dl, int Dr, int ca, int cb) {
  // output index: (((l * ca + a) * 2 + s) * Dr + r) * cb + b
  const int64_t total = (int64_t)Dl * ca * 2 * Dr * cb;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    int64_t q = idx;
    const int b = (int)(q % cb); q /= cb;
    const int r = (int)(q % Dr); q /= Dr;
    const int s = (int)(q % 2);  q /= 2;
    const int a = (int)(q % ca); q /= ca;
    const int l = (int)q;
    // W[l][s][t][r] at ((l * 2 + s) * 2 + t) * Dr + r ; A[a][t][b] at (a * 2 + t) * cb + b
    const CX w0 = W[((int64_t)(l * 2 + s) * 2 + 0) * Dr + r];
    const CX w1 = W[((int64_t)(l * 2 + s) * 2 + 1) * Dr + r];
    const CX a0 = A[((int64_t)a * 2 + 0) * cb + b];
    const CX a1 = A[((int64_t)a * 2 + 1) * cb + b];
    CX acc = cmul(w0, a0);
    cfma(acc, w1, a1);
    out[idx] = acc;
  }
}

// Lsum[l][i] = sum_q L[q][l][i]  (L: [cq][Dl][ci]);  Rsum[n][j] = sum_u R[u][n][j]  (R: [cu][Dn][cj])
template <typename CX>
__global__ void env_colsum_kernel(const CX* __restrict__ E, int rows, int cols, CX* __restrict__ out) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= cols) return;
  typedef typename cx_traits<CX>::R R;
  SumAcc<R> re, im;
  for (int q = 0; q < rows; ++q) {
    const CX v = E[(int64_t)q * cols + c];
    re.add(v.x);
    im.add(v.y);
  }
  out[c] = mk<CX>((R)re.value(), (R)im.value());
}

template <typename CX>
__global__ void tdvp_local_h_kernel(const CX* __restrict__ Ls, const CX* __restrict__ W, const CX* __restrict__ A,
                                    const CX* __restrict__ Rs, CX* __restrict__ H, int Dl, int Dn, int ci, int cj) {
  // H[i][t][j]; W[l][s][t][n]; Ls[l][i]; Rs[n][j]
  const int64_t total = (int64_t)ci * 2 * cj;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int j = (int)(idx % cj);
    const int t = (int)((idx / cj) % 2);
    const int i = (int)(idx / (2 * (int64_t)cj));
    CX acc = czero<CX>();
    for (int s = 0; s < 2; ++s) {
      const CX a = A[((int64_t)i * 2 + s) * cj + j];
      CX inner = czero<CX>();
      for (int l = 0; l < Dl; ++l) {
        const CX li = Ls[(int64_t)l * ci + i];
        CX wr = czero<CX>();
        for (int n = 0; n < Dn; ++n) cfma(wr, W[((int64_t)(l * 2 + s) * 2 + t) * Dn + n], Rs[(int64_t)n * cj + j]);
        cfma(inner, li, wr);
      }
      cfma(acc, inner, a);
    }
    H[idx] = acc;
  }
}

int grid_for(int64_t total) {
  int64_t b = (total + 255) / 256;
  if (b < 1) b = 1;
  if (b > 152 * 32) b = 152 * 32;
  return (int)b;
}

}  // namespace

extern "C" int agb_mpo_apply_site(int dtype, const void* W, const void* A, void* out, int Dl, int Dr, int chiA,
                                  int chiB, void* stream) {
  if (dtype != AGB_C64 && dtype != AGB_C128) return AGB_ERR_ARG;
  if (Dl <= 0 || Dr <= 0 || chiA <= 0 || chiB <= 0 || !W || !A || !out) return AGB_ERR_ARG;
  const int64_t total = (int64_t)Dl * chiA * 2 * Dr * chiB;
  cudaStream_t s = (cudaStream_t)stream;
  if (dtype == AGB_C64)
    mpo_apply_site_kernel<float2><<<grid_for(total), 256, 0, s>>>((const float2*)W, (const float2*)A, (float2*)out,
                                                                   Dl, Dr, chiA, chiB);
  else
    mpo_apply_site_kernel<double2><<<grid_for(total), 256, 0, s>>>((const double2*)W, (const double2*)A,
                                                                    (double2*)out, Dl, Dr, chiA, chiB);
  AGB_CHECK_LAUNCH();
  return AGB_OK;
}

extern "C" size_t agb_tdvp_local_h_workspace(int dtype, int Dl, int Dn, int chiI, int chiJ) {
  const size_t esz = dtype == AGB_C64 ? 8 : 16;
  return agb_align((size_t)Dl * chiI * esz) + agb_align((size_t)Dn * chiJ * esz);
}

extern "C" int agb_tdvp_local_h(int dtype, const void* L, const void* W, const void* A, const void* R, void* H,
                                int chiQ, int Dl, int chiI, int Dn, int chiU, int chiJ, void* ws, size_t ws_bytes,
                                void* stream) {
  if (dtype != AGB_C64 && dtype != AGB_C128) return AGB_ERR_ARG;
  if (chiQ <= 0 || Dl <= 0 || chiI <= 0 || Dn <= 0 || chiU <= 0 || chiJ <= 0) return AGB_ERR_ARG;
  if (!L || !W || !A || !R || !H || !ws) return AGB_ERR_ARG;
  if (ws_bytes < agb_tdvp_local_h_workspace(dtype, Dl, Dn, chiI, chiJ)) return AGB_ERR_WORKSPACE;
  const size_t esz = dtype == AGB_C64 ? 8 : 16;
  char* Ls = (char*)ws;
  char* Rs = Ls + agb_align((size_t)Dl * chiI * esz);
  cudaStream_t s = (cudaStream_t)stream;
  const int64_t total = (int64_t)chiI * 2 * chiJ;
  if (dtype == AGB_C64) {
    env_colsum_kernel<float2><<<(Dl * chiI + 127) / 128, 128, 0, s>>>((const float2*)L, chiQ, Dl * chiI, (float2*)Ls);
    AGB_CHECK_LAUNCH();
    env_colsum_kernel<float2><<<(Dn * chiJ + 127) / 128, 128, 0, s>>>((const float2*)R, chiU, Dn * chiJ, (float2*)Rs);
    AGB_CHECK_LAUNCH();
    tdvp_local_h_kernel<float2><<<grid_for(total), 256, 0, s>>>((const float2*)Ls, (const float2*)W,
                                                               (const float2*)A, (const float2*)Rs, (float2*)H,
                                                               Dl, Dn, chiI, chiJ);
  } else {
    env_colsum_kernel<double2><<<(Dl * chiI + 127) / 128, 128, 0, s>>>((const double2*)L, chiQ, Dl * chiI,
                                                                       (double2*)Ls);
    AGB_CHECK_LAUNCH();
    env_colsum_kernel<double2><<<(Dn * chiJ + 127) / 128, 128, 0, s>>>((const double2*)R, chiU, Dn * chiJ,
                                                                       (double2*)Rs);
    AGB_CHECK_LAUNCH();
    tdvp_local_h_kernel<double2><<<grid_for(total), 256, 0, s>>>((const double2*)Ls, (const double2*)W,
                                                                (const double2*)A, (const double2*)Rs,
                                                                (double2*)H, Dl, Dn, chiI, chiJ);
  }
  AGB_CHECK_LAUNCH();
  return AGB_OK;
}
