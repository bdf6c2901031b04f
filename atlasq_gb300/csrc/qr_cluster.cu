// Householder QR on a thread-block cluster (sm_103a), for the canonicalisation
// sweeps: the same factorisation as qr_kernel (zgeqr2-style reflectors, thin Q
// formed by applying them to [I; 0]) with the matrix in distributed shared
// memory instead of one CTA streaming it through L2.
//
// One cluster of C CTAs per matrix op(A) (M x N).  CTA q owns the columns
// c = q, q + C, ... and keeps them column-major in its shared memory.  Step j:
// the owner of column j forms the reflector (beta, tau, v) from its column and
// writes v and tau into every CTA's shared memory (DSMEM stores, double
// buffered by the parity of j); one cluster barrier; every CTA applies
// H_j^H = I - conj(tau) v v^H to its own columns > j (one warp per column).
// Double buffering makes one barrier per step enough: a buffer is rewritten
// two steps later, after every CTA has passed the barrier of the step between.
// The thin Q is formed the same way, backwards, with its columns in global
// memory (contiguous per column, so Q^T is written in place).
#include <cooperative_groups.h>

#include "common.cuh"

namespace cg = cooperative_groups;

namespace {

constexpr int QRC_THREADS = 512;
constexpr size_t kQrSmemBudget = 200 * 1024;

template <typename CX>
__global__ void __launch_bounds__(QRC_THREADS, 1)
    qr_cluster_kernel(const CX* __restrict__ Ain, int M, int N, int transA, CX* Q, CX* R, int trans_out, CX* Qw,
                      int C) {
  typedef typename cx_traits<CX>::R Rt;
  cg::cluster_group cluster = cg::this_cluster();
  const int q = (int)cluster.block_rank();
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5, nw = QRC_THREADS / 32;
  const int kk = M < N ? M : N;
  const int ncol = (q < N) ? (N - q + C - 1) / C : 0;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  CX* vbuf = (CX*)smem_raw;             // [2][M]  reflector of the current step (written remotely)
  CX* tauall = vbuf + 2 * (size_t)M;     // [kk]    every step's tau (own copy)
  CX* cols = tauall + kk;                // [ncol][M] own columns, column-major
  __shared__ CX taub[2];
  __shared__ Rt red[32];
  // ---- load own columns of op(A)
  for (int lc = wid; lc < ncol; lc += nw) {
    const int c = q + lc * C;
    CX* col = cols + (size_t)lc * M;
    for (int r = lane; r < M; r += 32) col[r] = transA ? Ain[(int64_t)c * M + r] : Ain[(int64_t)r * N + c];
  }
  __syncthreads();
  // ---- factorisation
  for (int j = 0; j < kk; ++j) {
    const int owner = j % C, b = j & 1;
    if (q == owner) {
      CX* col = cols + (size_t)(j / C) * M;
      Rt p = 0;
      for (int r = j + 1 + tid; r < M; r += QRC_THREADS) p += cabs2(col[r]);
      const Rt xn2 = block_sum(p, red);
      __shared__ CX sc_s;
      if (tid == 0) {
        const CX alpha = col[j];
        CX t = czero<CX>(), sc = czero<CX>();
        Rt beta;
        if (xn2 == Rt(0) && alpha.y == Rt(0)) {
          beta = alpha.x;
        } else {
          beta = -copysign(sqrt(alpha.x * alpha.x + alpha.y * alpha.y + xn2), alpha.x);
          t = mk<CX>((beta - alpha.x) / beta, -alpha.y / beta);
          sc = cinv(csub(alpha, mk<CX>(beta, 0)));
        }
        col[j] = mk<CX>(beta, 0);
        sc_s = sc;
        for (int k = 0; k < C; ++k) cluster.map_shared_rank(taub, k)[b] = t;
      }
      __syncthreads();
      const CX sc = sc_s;
      for (int r = j + tid; r < M; r += QRC_THREADS) {
        CX v;
        if (r == j) {
          v = mk<CX>(1, 0);
        } else {
          v = cmul(col[r], sc);
          col[r] = v;  // reflector stored below the diagonal
        }
        for (int k = 0; k < C; ++k) cluster.map_shared_rank(vbuf, k)[(size_t)b * M + r] = v;
      }
    }
    cluster.sync();
    const CX t = taub[b];
    if (tid == 0) tauall[j] = t;
    if (t.x != Rt(0) || t.y != Rt(0)) {
      const CX tc = cconj(t);
      const CX* v = vbuf + (size_t)b * M;
      const int lc0 = (j + 1 - q + C - 1) / C > 0 ? (j + 1 - q + C - 1) / C : 0;  // own columns c > j
      for (int lc = lc0 + wid; lc < ncol; lc += nw) {
        CX* col = cols + (size_t)lc * M;
        CX acc = czero<CX>();
        for (int r = j + lane; r < M; r += 32) cfmac(acc, v[r], col[r]);
        acc = warp_csum(acc);
        const CX tw = cmul(tc, acc);
        for (int r = j + lane; r < M; r += 32) col[r] = csub(col[r], cmul(v[r], tw));
      }
    }
    __syncthreads();
  }
  // ---- R = upper triangle of the factored columns (kk x N)
  for (int lc = wid; lc < ncol; lc += nw) {
    const int c = q + lc * C;
    const CX* col = cols + (size_t)lc * M;
    for (int r = lane; r < kk; r += 32) {
      const CX val = (r <= c) ? col[r] : czero<CX>();
      if (trans_out) R[(int64_t)c * kk + r] = val;
      else R[(int64_t)r * N + c] = val;
    }
  }
  cluster.sync();  // every CTA is done with the factorisation's reflector buffers
  // ---- thin Q: columns c < kk, owned cyclically, column-major in global memory
  CX* Qc = trans_out ? Q : Qw;  // element (r, c) at c * M + r
  const int nq = (q < kk) ? (kk - q + C - 1) / C : 0;
  for (int lc = wid; lc < nq; lc += nw) {
    const int c = q + lc * C;
    for (int r = lane; r < M; r += 32) Qc[(int64_t)c * M + r] = (r == c) ? mk<CX>(1, 0) : czero<CX>();
  }
  __syncthreads();
  for (int j = kk - 1; j >= 0; --j) {
    const int owner = j % C, b = j & 1;
    if (q == owner) {
      const CX* col = cols + (size_t)(j / C) * M;
      for (int r = j + tid; r < M; r += QRC_THREADS) {
        const CX v = (r == j) ? mk<CX>(1, 0) : col[r];
        for (int k = 0; k < C; ++k) cluster.map_shared_rank(vbuf, k)[(size_t)b * M + r] = v;
      }
    }
    cluster.sync();
    const CX t = tauall[j];
    if (t.x != Rt(0) || t.y != Rt(0)) {
      const CX* v = vbuf + (size_t)b * M;
      const int lc0 = (j - q + C - 1) / C > 0 ? (j - q + C - 1) / C : 0;  // own Q columns c >= j
      for (int lc = lc0 + wid; lc < nq; lc += nw) {
        CX* qc = Qc + (int64_t)(q + lc * C) * M;
        CX acc = czero<CX>();
        for (int r = j + lane; r < M; r += 32) cfmac(acc, v[r], qc[r]);
        acc = warp_csum(acc);
        const CX tw = cmul(t, acc);
        for (int r = j + lane; r < M; r += 32) qc[r] = csub(qc[r], cmul(v[r], tw));
      }
    }
    __syncthreads();
  }
  if (!trans_out) {
    // Q row-major (M x kk) from the column-major working copy
    for (int lc = wid; lc < nq; lc += nw) {
      const int c = q + lc * C;
      for (int r = lane; r < M; r += 32) Q[(int64_t)r * kk + c] = Qw[(int64_t)c * M + r];
    }
  }
  cluster.sync();  // keep every CTA's shared memory alive until remote writers are done
}

}  // namespace

// Smallest cluster (2, 4, 8, or 16 CTAs where the device allows it) whose
// shared memory holds its columns; 0 if none does.
int qr_cluster_size(int esz, int M, int N, size_t* smem_out) {
  const int kk = M < N ? M : N;
  for (int C : {2, 4, 8, 16}) {
    const int ncol = (N + C - 1) / C;
    const size_t smem = ((size_t)2 * M + kk + (size_t)ncol * M) * esz;
    if (smem <= kQrSmemBudget) {
      if (smem_out) *smem_out = smem;
      return C;
    }
  }
  return 0;
}

template <typename CX>
int launch_qr_cluster(const CX* A, int M, int N, int transA, CX* Q, CX* R, int trans_out, CX* Qw, cudaStream_t s) {
  size_t smem = 0;
  const int C = qr_cluster_size(sizeof(CX), M, N, &smem);
  if (C == 0) return AGB_ERR_UNSUPPORTED;
  if (C > 8 && cudaFuncSetAttribute(qr_cluster_kernel<CX>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) !=
                   cudaSuccess) {
    cudaGetLastError();
    return AGB_ERR_UNSUPPORTED;
  }
  if (cudaFuncSetAttribute(qr_cluster_kernel<CX>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
      cudaSuccess) {
    cudaGetLastError();
    return AGB_ERR_UNSUPPORTED;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(C, 1, 1);
  cfg.blockDim = dim3(QRC_THREADS, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = C;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  const cudaError_t err = cudaLaunchKernelEx(&cfg, qr_cluster_kernel<CX>, A, M, N, transA, Q, R, trans_out, Qw, C);
  agb_note_launch();
  if (err != cudaSuccess) {
    cudaGetLastError();
    return AGB_ERR_UNSUPPORTED;
  }
  return AGB_OK;
}

template int launch_qr_cluster<float2>(const float2*, int, int, int, float2*, float2*, int, float2*, cudaStream_t);
template int launch_qr_cluster<double2>(const double2*, int, int, int, double2*, double2*, int, double2*,
                                        cudaStream_t);
