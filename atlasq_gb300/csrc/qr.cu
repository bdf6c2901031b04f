// Householder QR for the MPS canonicalisation sweeps (sm_103a).
//
// Replaces robust_qr / torch.linalg.qr (src/atlas_q/linalg_robust.py:55-76) as
// used by to_left_canonical (adaptive_mps.py:310-339), canonicalize_right_to_left
// (mps_pytorch.py:123-152) and to_mixed_canonical (adaptive_mps.py:346-385).
//
// One CTA (1024 threads = 128 column lanes x 8 row groups) per matrix.  The
// matrix op(A) (M x N, op = N or T) is copied into the workspace, reduced with
// zgeqr2-style reflectors (H_j^H applied from the left), then the thin Q
// (M x kk, kk = min(M, N)) is formed by applying H_0 ... H_{kk-1} to [I; 0].
// Outputs: Q [M, kk] and R [kk, N] (upper triangular), or their transposes.
#include "common.cuh"

template <typename CX>
int launch_qr_cluster(const CX* A, int M, int N, int transA, CX* Q, CX* R, int trans_out, CX* Qw, cudaStream_t s);
template <typename CX>
int launch_qr_blocked(const CX* A, int M, int N, int transA, CX* Q, CX* R, int trans_out, void* ws, size_t ws_bytes,
                      cudaStream_t s);
size_t qr_blocked_workspace(int esz, int M, int N);

namespace {

constexpr int QR_CG = 128, QR_RG = 8;

template <typename CX>
__global__ void __launch_bounds__(1024) qr_kernel(const CX* __restrict__ Ain, int M, int N, int transA,
                                                  CX* W, CX* Q, CX* R, int trans_out, CX* tau, CX* Qw) {
  typedef typename cx_traits<CX>::R Rt;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  CX* v = (CX*)smem_raw;                 // [M]
  CX* part = v + M;                      // [QR_RG][QR_CG]
  __shared__ Rt red[32];
  __shared__ CX bc[2];
  const int tid = threadIdx.x, nt = blockDim.x;
  const int cg = tid % QR_CG, rg = tid / QR_CG;
  const int kk = M < N ? M : N;
  // W = op(A), row-major M x N
  for (int64_t i = tid; i < (int64_t)M * N; i += nt) {
    const int r = (int)(i / N), c = (int)(i % N);
    W[i] = transA ? Ain[(int64_t)c * M + r] : Ain[i];
  }
  __syncthreads();
  for (int j = 0; j < kk; ++j) {
    Rt p = 0;
    for (int r = j + 1 + tid; r < M; r += nt) p += cabs2(W[(int64_t)r * N + j]);
    const Rt xn2 = block_sum(p, red);
    if (tid == 0) {
      const CX alpha = W[(int64_t)j * N + j];
      CX t = czero<CX>(), sc = czero<CX>();
      Rt beta;
      if (xn2 == Rt(0) && alpha.y == Rt(0)) {
        beta = alpha.x;
      } else {
        beta = -copysign(sqrt(alpha.x * alpha.x + alpha.y * alpha.y + xn2), alpha.x);
        t = mk<CX>((beta - alpha.x) / beta, -alpha.y / beta);
        sc = cinv(csub(alpha, mk<CX>(beta, 0)));
      }
      bc[0] = t;
      bc[1] = sc;
      tau[j] = t;
      W[(int64_t)j * N + j] = mk<CX>(beta, 0);
      v[j] = mk<CX>(1, 0);
    }
    __syncthreads();
    const CX t = bc[0], sc = bc[1];
    for (int r = j + 1 + tid; r < M; r += nt) {
      const CX x = cmul(W[(int64_t)r * N + j], sc);
      v[r] = x;
      W[(int64_t)r * N + j] = x;
    }
    __syncthreads();
    if (t.x == Rt(0) && t.y == Rt(0)) continue;
    const CX tc = cconj(t);
    // apply H^H = I - conj(tau) v v^H to columns c > j
    for (int c0 = j + 1; c0 < N; c0 += QR_CG) {
      const int c = c0 + cg;
      CX acc = czero<CX>();
      if (c < N)
        for (int r = j + rg; r < M; r += QR_RG) cfmac(acc, v[r], W[(int64_t)r * N + c]);
      part[rg * QR_CG + cg] = acc;
      __syncthreads();
      if (c < N) {
        CX w = czero<CX>();
#pragma unroll
        for (int g = 0; g < QR_RG; ++g) w = cadd(w, part[g * QR_CG + cg]);
        const CX tw = cmul(tc, w);
        for (int r = j + rg; r < M; r += QR_RG) {
          CX* a = W + (int64_t)r * N + c;
          *a = csub(*a, cmul(v[r], tw));
        }
      }
      __syncthreads();
    }
  }
  // R = upper triangle of W[:kk, :]
  for (int64_t i = tid; i < (int64_t)kk * N; i += nt) {
    const int r = (int)(i / N), c = (int)(i % N);
    const CX val = (c >= r) ? W[(int64_t)r * N + c] : czero<CX>();
    if (trans_out) R[(int64_t)c * kk + r] = val;
    else R[i] = val;
  }
  // Q = H_0 ... H_{kk-1} [I; 0]: apply the reflectors (stored below the diagonal
  // of W, unit leading entry) in reverse order to the first kk identity columns.
  // Q is formed row-major (element (r, c) at r*kk + c, column lanes coalesced);
  // a transposed output is formed in the workspace and copied out at the end.
  CX* Qf = trans_out ? Qw : Q;
  const int64_t qs_r = kk, qs_c = 1;
  for (int64_t i = tid; i < (int64_t)M * kk; i += nt) {
    const int r = (int)(i / kk), c = (int)(i % kk);
    Qf[r * qs_r + c * qs_c] = (r == c) ? mk<CX>(1, 0) : czero<CX>();
  }
  __syncthreads();
  for (int j = kk - 1; j >= 0; --j) {
    const CX t = tau[j];
    if (t.x == Rt(0) && t.y == Rt(0)) continue;
    for (int r = j + tid; r < M; r += nt) v[r] = (r == j) ? mk<CX>(1, 0) : W[(int64_t)r * N + j];
    __syncthreads();
    for (int c0 = j; c0 < kk; c0 += QR_CG) {
      const int c = c0 + cg;
      CX acc = czero<CX>();
      if (c < kk)
        for (int r = j + rg; r < M; r += QR_RG) cfmac(acc, v[r], Qf[r * qs_r + c * qs_c]);
      part[rg * QR_CG + cg] = acc;
      __syncthreads();
      if (c < kk) {
        CX w = czero<CX>();
#pragma unroll
        for (int g = 0; g < QR_RG; ++g) w = cadd(w, part[g * QR_CG + cg]);
        const CX tw = cmul(t, w);
        for (int r = j + rg; r < M; r += QR_RG) {
          CX* a = Qf + r * qs_r + c * qs_c;
          *a = csub(*a, cmul(v[r], tw));
        }
      }
      __syncthreads();
    }
  }
  if (trans_out) {
    __syncthreads();
    for (int64_t i = tid; i < (int64_t)M * kk; i += nt) {
      const int c = (int)(i / M), r = (int)(i % M);  // coalesced writes of Q^T
      Q[i] = Qf[(int64_t)r * kk + c];
    }
  }
}

}  // namespace

// working copy of op(A), tau, column-major Q (single-CTA and unblocked cluster kernels)
static size_t qr_unblocked_workspace(int dtype, int M, int N) {
  const int esz = dtype == AGB_C64 ? 8 : 16;
  const int kk = M < N ? M : N;
  return agb_align((size_t)M * N * esz) + agb_align((size_t)kk * esz) + agb_align((size_t)M * kk * esz);
}

extern "C" size_t agb_qr_workspace(int dtype, int M, int N) {
  const size_t unblocked = qr_unblocked_workspace(dtype, M, N);
  const size_t blocked = qr_blocked_workspace(dtype == AGB_C64 ? 8 : 16, M, N);
  return unblocked > blocked ? unblocked : blocked;
}

extern "C" int agb_qr(int dtype, const void* A, int M, int N, int transA, void* Q, void* R,
                      int trans_out, void* ws, size_t ws_bytes, void* stream) {
  if (dtype != AGB_C64 && dtype != AGB_C128) return AGB_ERR_ARG;
  if (M <= 0 || N <= 0 || !A || !Q || !R || !ws) return AGB_ERR_ARG;
  if (M > 8192) return AGB_ERR_UNSUPPORTED;
  if (ws_bytes < agb_qr_workspace(dtype, M, N)) return AGB_ERR_WORKSPACE;
  const int esz = dtype == AGB_C64 ? 8 : 16;
  const int kk = M < N ? M : N;
  char* base = (char*)ws;
  void* W = base;
  void* tau = base + agb_align((size_t)M * N * esz);
  void* Qw = (char*)tau + agb_align((size_t)kk * esz);
  const size_t smem = (size_t)M * esz + (size_t)QR_RG * QR_CG * esz;
  cudaStream_t s = (cudaStream_t)stream;
  // large matrices: the blocked cluster kernel (panels of reflectors, one
  // cluster barrier per panel), else the unblocked one (columns in distributed
  // shared memory)
  if ((int64_t)M * N >= 64 * 64) {
    const int rb = dtype == AGB_C64
                       ? launch_qr_blocked<float2>((const float2*)A, M, N, transA, (float2*)Q, (float2*)R, trans_out,
                                                   ws, ws_bytes, s)
                       : launch_qr_blocked<double2>((const double2*)A, M, N, transA, (double2*)Q, (double2*)R,
                                                    trans_out, ws, ws_bytes, s);
    if (rb == AGB_OK) return AGB_OK;
    const int rc = dtype == AGB_C64
                       ? launch_qr_cluster<float2>((const float2*)A, M, N, transA, (float2*)Q, (float2*)R, trans_out,
                                                   (float2*)Qw, s)
                       : launch_qr_cluster<double2>((const double2*)A, M, N, transA, (double2*)Q, (double2*)R,
                                                    trans_out, (double2*)Qw, s);
    if (rc == AGB_OK) return AGB_OK;
  }
  if (dtype == AGB_C64) {
    if (agb_smem_optin(qr_kernel<float2>, smem) != cudaSuccess) return AGB_ERR_CUDA;
    qr_kernel<float2><<<1, 1024, smem, s>>>((const float2*)A, M, N, transA, (float2*)W, (float2*)Q,
                                             (float2*)R, trans_out, (float2*)tau, (float2*)Qw);
  } else {
    if (agb_smem_optin(qr_kernel<double2>, smem) != cudaSuccess) return AGB_ERR_CUDA;
    qr_kernel<double2><<<1, 1024, smem, s>>>((const double2*)A, M, N, transA, (double2*)W,
                                              (double2*)Q, (double2*)R, trans_out, (double2*)tau, (double2*)Qw);
  }
  (void)kk;
  AGB_CHECK_LAUNCH();
  return AGB_OK;
}

// ---------------------------------------------------------------------------
// Allocation-free QR.
//
// Some callers of this library cannot allocate device memory: a host runtime
// that reaches the library only through this C ABI and is handed device
// pointers by the component that owns the GPU memory, or code running while
// another allocator owns every device allocation.  agb_qr_noalloc computes the
// same factorisation as agb_qr without a caller-supplied workspace: its scratch
// (the working copy of op(A) and the reflector scalars) is the file-scope
// device array below, AGB_QR_NOALLOC_MAX_BYTES bytes, which every GPU that
// loads this library holds until the process exits.
//
// * The array's host-side name is not a device address.  The first call on
//   each device, with that device current, looks the address up with
//   cudaGetSymbolAddress and caches it; make that first call before any
//   stream capture begins.
// * Every call shares the one array and it keeps the previous call's
//   contents.  The kernel overwrites everything it reads (the working copy is
//   filled from A, each scalar is written before use), so nothing has to be
//   cleared first.  Calls that overlap on the GPU (e.g. on two streams) race
//   on the array; issue them on one stream or serialise them.
// * Problems whose scratch exceeds AGB_QR_NOALLOC_MAX_BYTES are rejected with
//   AGB_ERR_TOO_LARGE before anything is launched.
// * No cudaMalloc, cudaFree or allocating library call is made.
#include <mutex>

static __device__ __align__(256) unsigned char g_qr_noalloc_scratch[AGB_QR_NOALLOC_MAX_BYTES];

namespace {
constexpr int kMaxDevices = 64;
void* g_qr_noalloc_ptr[kMaxDevices] = {nullptr};
std::mutex g_qr_noalloc_mu;
}  // namespace

extern "C" int agb_qr_noalloc(int dtype, const void* A, int M, int N, int transA, void* Q, void* R,
                              int trans_out, void* stream) {
  if (dtype != AGB_C64 && dtype != AGB_C128) return AGB_ERR_ARG;
  if (M <= 0 || N <= 0 || !A || !Q || !R) return AGB_ERR_ARG;
  if (M > 8192) return AGB_ERR_UNSUPPORTED;
  const size_t need = qr_unblocked_workspace(dtype, M, N);
  if (need > (size_t)AGB_QR_NOALLOC_MAX_BYTES) return AGB_ERR_TOO_LARGE;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return AGB_ERR_CUDA;
  void* base = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_qr_noalloc_mu);
    if (!g_qr_noalloc_ptr[dev]) {
      void* p = nullptr;
      if (cudaGetSymbolAddress(&p, g_qr_noalloc_scratch) != cudaSuccess || !p) return AGB_ERR_CUDA;
      g_qr_noalloc_ptr[dev] = p;
    }
    base = g_qr_noalloc_ptr[dev];
  }
  const int esz = dtype == AGB_C64 ? 8 : 16;
  void* W = base;
  void* tau = (char*)base + agb_align((size_t)M * N * esz);
  const int kk = M < N ? M : N;
  void* Qw = (char*)tau + agb_align((size_t)kk * esz);
  const size_t smem = (size_t)M * esz + (size_t)QR_RG * QR_CG * esz;
  cudaStream_t s = (cudaStream_t)stream;
  if (dtype == AGB_C64) {
    if (agb_smem_optin(qr_kernel<float2>, smem) != cudaSuccess) return AGB_ERR_CUDA;
    qr_kernel<float2><<<1, 1024, smem, s>>>((const float2*)A, M, N, transA, (float2*)W, (float2*)Q,
                                             (float2*)R, trans_out, (float2*)tau, (float2*)Qw);
  } else {
    if (agb_smem_optin(qr_kernel<double2>, smem) != cudaSuccess) return AGB_ERR_CUDA;
    qr_kernel<double2><<<1, 1024, smem, s>>>((const double2*)A, M, N, transA, (double2*)W,
                                              (double2*)Q, (double2*)R, trans_out, (double2*)tau, (double2*)Qw);
  }
  AGB_CHECK_LAUNCH();
  return AGB_OK;
}
