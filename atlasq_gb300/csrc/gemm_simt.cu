// SIMT batched complex GEMM for sm_103a: 64x64 output tiles, K-step 8,
// 256 threads, 4x4 complex accumulators per thread.  Used for small and ragged
// shapes, and for complex128.
#include "gemm.cuh"
#include "gemm_tc.cuh"

namespace {

constexpr int BM = 64, BN = 64, BK = 8;

template <typename CX>
AGB_DEV CX load_op(const CX* P, int64_t ld, int op, int row, int col, int rows, int cols) {
  // element (row, col) of op(P), where op(P) is rows x cols
  if (row >= rows || col >= cols) return czero<CX>();
  if (op == 0) return P[(int64_t)row * ld + col];
  if (op == 3) return cconj(P[(int64_t)row * ld + col]);
  CX v = P[(int64_t)col * ld + row];
  return op == 2 ? cconj(v) : v;
}

struct StridedBatch {
  GemmProb base;
  int64_t sA, sB, sC;  // element strides between batch entries
};

template <typename CX>
AGB_DEV GemmProb get_prob(const GemmProb* probs, const StridedBatch& sb) {
  if (probs) return probs[blockIdx.z];
  GemmProb p = sb.base;
  const int64_t z = blockIdx.z;
  p.A = (const CX*)sb.base.A + z * sb.sA;
  p.B = (const CX*)sb.base.B + z * sb.sB;
  p.D = (CX*)sb.base.D + z * sb.sC;
  p.Csrc = (const CX*)sb.base.Csrc + z * sb.sC;
  return p;
}

template <typename CX>
__global__ void __launch_bounds__(256) gemm_simt_kernel(const GemmProb* __restrict__ probs, StridedBatch sb) {
  const GemmProb p = get_prob<CX>(probs, sb);
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
  if (m0 >= p.M || n0 >= p.N) return;
  typedef typename cx_traits<CX>::R R;
  __shared__ CX As[BK][BM + 1];
  __shared__ CX Bs[BK][BN + 1];
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const CX* A = (const CX*)p.A;
  const CX* B = (const CX*)p.B;
  CX acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = czero<CX>();

  for (int k0 = 0; k0 < p.K; k0 += BK) {
    // A tile: BM x BK of op(A); B tile: BK x BN of op(B)
#pragma unroll
    for (int e = 0; e < 2; ++e) {
      const int idx = tid + e * 256;
      int r, c;
      if (p.opA == 0 || p.opA == 3) { r = idx / BK; c = idx % BK; } else { r = idx % BM; c = idx / BM; }
      As[c][r] = load_op(A, p.lda, p.opA, m0 + r, k0 + c, p.M, p.K);
      int kr, nc;
      if (p.opB == 0 || p.opB == 3) { kr = idx / BN; nc = idx % BN; } else { kr = idx % BK; nc = idx / BK; }
      Bs[kr][nc] = load_op(B, p.ldb, p.opB, k0 + kr, n0 + nc, p.K, p.N);
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < BK; ++k) {
      CX a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[k][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[k][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) cfma(acc[i][j], a[i], b[j]);
    }
    __syncthreads();
  }
  const CX alpha = mk<CX>((R)p.alpha_re, (R)p.alpha_im);
  const CX beta = mk<CX>((R)p.beta_re, (R)p.beta_im);
  const bool use_beta = (p.beta_re != 0.0 || p.beta_im != 0.0);
  CX* D = (CX*)p.D;
  const CX* C = (const CX*)p.Csrc;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int r = m0 + ty + 16 * i;
    if (r >= p.M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int c = n0 + tx + 16 * j;
      if (c >= p.N) continue;
      CX v = cmul(alpha, acc[i][j]);
      if (use_beta) v = cadd(v, cmul(beta, C[(int64_t)r * p.ldc + c]));
      D[(int64_t)r * p.ldd + c] = v;
    }
  }
}

}  // namespace

template <typename CX>
int launch_gemm_probs(const GemmProb* probs, int count, int maxM, int maxN, cudaStream_t s, const GemmCtx* ctx,
                      int maxK) {
  if (count <= 0 || maxM <= 0 || maxN <= 0) return AGB_OK;
  if (sizeof(CX) == 8 && ctx && ctx->tc_scratch && maxM >= 64 && maxN >= 64 && maxK >= 32 &&
      ctx->tc_bytes >= tc_gemm_scratch_bytes(count, maxM, maxN, maxK))
    return launch_gemm_tc(probs, count, maxM, maxN, maxK, ctx->tc_scratch, ctx->tc_bytes, ctx->status, s);
  dim3 grid((maxN + BN - 1) / BN, (maxM + BM - 1) / BM, count);
  StridedBatch sb = {};
  gemm_simt_kernel<CX><<<grid, 256, 0, s>>>(probs, sb);
  AGB_CHECK_LAUNCH();
  return AGB_OK;
}

template int launch_gemm_probs<float2>(const GemmProb*, int, int, int, cudaStream_t, const GemmCtx*, int);
template int launch_gemm_probs<double2>(const GemmProb*, int, int, int, cudaStream_t, const GemmCtx*, int);

namespace {
// 'N' as stored, 'T' transposed, 'C' conjugate-transposed, 'R' conjugated (not transposed)
int op_code(char c) {
  return (c == 'N' || c == 'n') ? 0 : (c == 'T' || c == 't') ? 1 : (c == 'C' || c == 'c') ? 2 : (c == 'R' || c == 'r') ? 3 : -1;
}
}  // namespace

// Strided-batch host entry (no allocation: the kernel derives each batch
// entry's pointers from the base problem and the element strides).
extern "C" int agb_cgemm_batched(int dtype, char opA, char opB, int batch, int M, int N, int K,
                                 const void* A, int64_t lda, int64_t strideA, const void* B,
                                 int64_t ldb, int64_t strideB, void* C, int64_t ldc, int64_t strideC,
                                 double alpha_re, double alpha_im, double beta_re, double beta_im,
                                 void* stream) {
  const int oa = op_code(opA), ob = op_code(opB);
  if (oa < 0 || ob < 0 || batch < 0 || M < 0 || N < 0 || K < 0) return AGB_ERR_ARG;
  if (dtype != AGB_C64 && dtype != AGB_C128) return AGB_ERR_ARG;
  if (batch == 0 || M == 0 || N == 0) return AGB_OK;
  if (batch > 65535) return AGB_ERR_UNSUPPORTED;
  StridedBatch sb;
  GemmProb& b = sb.base;
  b.A = A;
  b.B = B;
  b.D = C;
  b.Csrc = C;
  b.lda = lda;
  b.ldb = ldb;
  b.ldd = ldc;
  b.ldc = ldc;
  b.M = M;
  b.N = N;
  b.K = K;
  b.opA = oa;
  b.opB = ob;
  b.alpha_re = alpha_re;
  b.alpha_im = alpha_im;
  b.beta_re = beta_re;
  b.beta_im = beta_im;
  sb.sA = strideA;
  sb.sB = strideB;
  sb.sC = strideC;
  cudaStream_t s = (cudaStream_t)stream;
  dim3 grid((N + BN - 1) / BN, (M + BM - 1) / BM, batch);
  if (dtype == AGB_C64)
    gemm_simt_kernel<float2><<<grid, 256, 0, s>>>(nullptr, sb);
  else
    gemm_simt_kernel<double2><<<grid, 256, 0, s>>>(nullptr, sb);
  AGB_CHECK_LAUNCH();
  return AGB_OK;
}
