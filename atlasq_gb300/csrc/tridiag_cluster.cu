// Householder tridiagonalisation of a Hermitian matrix held in the distributed
// shared memory of a thread-block cluster (sm_103a).
//
// One cluster of C CTAs (C = 1, 2, 4 or 8) per matrix.  CTA q owns the rows
// r = q, q + C, q + 2C, ... and keeps their lower-triangular entries packed in
// its shared memory, so the whole reduction runs on chip.  Step j (zhetd2
// formulation, lower):
//   A. every CTA publishes its entries of column j (rows > j) and a partial
//      norm to all CTAs (DSMEM stores); cluster barrier; each CTA forms the
//      reflector (beta, tau, v) redundantly.
//   B. fused pass over the CTA's rows: apply the previous step's rank-2 update
//      A -= v' w'^H + w' v'^H (columns > j) and accumulate the partial matvec
//      A v (row-wise and, through the Hermitian symmetry, column-wise with
//      shared-memory atomics); cluster barrier; each CTA sums the C partials
//      (DSMEM loads), forms w = tau A v - 1/2 tau (p^H v) tau ... and updates
//      column j+1 of its rows for the next reflector.
// Outputs match the single-CTA kernel: d, e (real), tau (complex), reflector v_j
// in row j of H (columns j+2 .. n-1, v_j[j+1] = 1 implicit), scale.
//
// Rows that do not fit (matrices above ~700 for complex64 at 8 CTAs) stay in
// place in the lower triangle of H (L2-resident): a CTA keeps its first
// `isplit` rows (the short ones) in shared memory and addresses the rest as
// H[r][0..r].  The reflectors are written to the strictly upper part of H
// (row j, columns >= j+2), which the overflow rows never touch.  Overflow rows
// are read and written only by their owning CTA, between block barriers.
#include <cooperative_groups.h>

#include <type_traits>

#include "heevd.cuh"
#include "prof.cuh"

namespace cg = cooperative_groups;

namespace {

AGB_DEV int row_offset(int i, int q, int C) { return i * (q + 1) + C * (i * (i - 1) / 2); }

template <typename CX, bool OVERFLOW>
__global__ void __launch_bounds__(512, 1) tridiag_cluster_kernel(const HeevdProb* __restrict__ probs, int C,
                                                                 int cap_elems) {
  typedef typename cx_traits<CX>::R R;
  cg::cluster_group cluster = cg::this_cluster();
  const int q = (int)cluster.block_rank();
  const HeevdProb P = probs[blockIdx.x / C];
  const int n = P.n;
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, wid = tid >> 5, nw = nt >> 5;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int nrows = (n - q + C - 1) / C;  // rows owned (q < n)
  const int nown = (q < n) ? nrows : 0;
  // The exchange vectors sit at the same shared-memory offset in every CTA of
  // the cluster (map_shared_rank maps an address to the same offset in the
  // peer CTA); the packed rows, whose size differs per CTA, come after them.
  CX* xbuf = (CX*)smem_raw;  // column j, written remotely by the owners
  CX* pp = xbuf + n;         // partial matvec, read remotely
  CX* v = pp + n;
  CX* w = v + n;
  CX* vprev = w + n;
  CX* wprev = vprev + n;
  CX* rows = wprev + n;
  __shared__ R normp[16];
  __shared__ R red[64];
  __shared__ CX sc[4];
  __shared__ R mxp[16];
  CX* H = (CX*)P.H;
  const int64_t ld = P.ldh;
  // own rows [0, isplit) are packed in shared memory, the rest live in H
  int isplit = 0;
  if (OVERFLOW)
    while (isplit < nown && row_offset(isplit + 1, q, C) <= cap_elems) ++isplit;
  auto rowp = [&](int i) -> CX* {
    if (!OVERFLOW) return rows + row_offset(i, q, C);  // every row in shared memory
    return (i < isplit) ? rows + row_offset(i, q, C) : H + (int64_t)(q + i * C) * ld;
  };
  R* d = (R*)P.d;
  R* e = (R*)P.e;
  CX* tau = (CX*)P.tau;

  // ---- scale by the largest diagonal magnitude
  R mx = 0;
  for (int i = tid; i < nown; i += nt) {
    const int r = q + i * C;
    mx = fmax(mx, fabs(H[(int64_t)r * ld + r].x));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if (lane == 0) red[wid] = mx;
  __syncthreads();
  if (tid == 0) {
    R m = 0;
    for (int i = 0; i < nw; ++i) m = fmax(m, red[i]);
    for (int k = 0; k < C; ++k) *cluster.map_shared_rank(&mxp[q], k) = m;
  }
  cluster.sync();
  mx = 0;
  for (int k = 0; k < C; ++k) mx = fmax(mx, mxp[k]);
  if (mx == R(0)) mx = R(1);
  if (q == 0 && tid == 0) *((R*)P.scale) = mx;
  const R inv = R(1) / mx;
  // ---- load own rows (lower triangle, scaled)
  for (int i = wid; i < nown; i += nw) {
    const int r = q + i * C;
    CX* dst = rowp(i);
    const CX* src = H + (int64_t)r * ld;  // dst == src for an overflow row (scaled in place)
    for (int c = lane; c <= r; c += 32) dst[c] = cscale(src[c], inv);
  }
  __syncthreads();
  if (n == 1) {
    if (tid == 0) {
      d[0] = rowp(0)[0].x;
      e[0] = 0;
      tau[0] = czero<CX>();
    }
    return;
  }
  bool prev_active = false;
  for (int j = 0; j <= n - 2; ++j) {
    // ---------------- A: publish column j (rows >= j+1) and the partial norm
    if (q == (j % C) && tid == 0) d[j] = rowp(j / C)[j].x;
    R part = 0;
    {
      // own rows r >= j+1: local index i >= i0
      const int i0 = (j + 1 - q + C - 1) / C > 0 ? (j + 1 - q + C - 1) / C : 0;
      for (int i = i0 + tid; i < nown; i += nt) {
        const int r = q + i * C;
        const CX x = rowp(i)[j];
        for (int k = 0; k < C; ++k) cluster.map_shared_rank(xbuf, k)[r] = x;
        if (r >= j + 2) part += cabs2(x);
      }
    }
    part = block_sum(part, red);
    if (tid == 0)
      for (int k = 0; k < C; ++k) *cluster.map_shared_rank(&normp[q], k) = part;
    cluster.sync();
    if (tid == 0) {
      R xn2 = 0;
      for (int k = 0; k < C; ++k) xn2 += normp[k];
      const CX alpha = xbuf[j + 1];
      CX t = czero<CX>(), s = czero<CX>();
      R beta;
      if (xn2 == R(0) && alpha.y == R(0)) {
        beta = alpha.x;
      } else {
        beta = -copysign(sqrt(alpha.x * alpha.x + alpha.y * alpha.y + xn2), alpha.x);
        t = mk<CX>((beta - alpha.x) / beta, -alpha.y / beta);
        s = cinv(csub(alpha, mk<CX>(beta, 0)));
      }
      sc[0] = t;
      sc[1] = s;
      if (q == 0) {
        e[j] = beta;
        tau[j] = t;
      }
    }
    __syncthreads();
    const CX t = sc[0], s = sc[1];
    const bool active = (t.x != R(0) || t.y != R(0));
    for (int r = j + 1 + tid; r < n; r += nt) {
      const CX vr = (r == j + 1) ? mk<CX>(1, 0) : cmul(xbuf[r], s);
      v[r] = vr;
      pp[r] = czero<CX>();
      if (q == 0 && r >= j + 2) H[(int64_t)j * ld + r] = vr;  // reflector storage
    }
    __syncthreads();
    // ---------------- B: fused previous update + partial matvec over own rows
    // Row pass (warp per row): apply the pending rank-2 update of the previous
    // step to columns > j and accumulate sum_{c <= r} A[r][c] v_c.
    {
      const int i0 = (j + 1 - q + C - 1) / C > 0 ? (j + 1 - q + C - 1) / C : 0;
      // the four (update, matvec) cases as separate loops: no per-element branch
      auto row_pass = [&](auto upd, auto mv) {
        for (int i = i0 + wid; i < nown; i += nw) {
          const int r = q + i * C;
          CX* row = rowp(i);
          const CX vr = vprev[r], wr = wprev[r];
          CX acc = czero<CX>();
          for (int c = j + 1 + lane; c <= r; c += 32) {
            CX a = row[c];
            if constexpr (decltype(upd)::value) {  // column j itself was updated at the end of the previous step
              a = csub(a, cmul(vr, cconj(wprev[c])));
              a = csub(a, cmul(wr, cconj(vprev[c])));
              row[c] = a;
            }
            if constexpr (decltype(mv)::value) cfma(acc, a, v[c]);
          }
          if constexpr (decltype(mv)::value) {
            acc = warp_csum(acc);
            if (lane == 0) pp[r] = acc;  // rows are owned by one warp: plain store
          }
        }
      };
      using T_ = std::true_type;
      using F_ = std::false_type;
      if (prev_active && active) row_pass(T_{}, T_{});
      else if (active) row_pass(F_{}, T_{});
      else if (prev_active) row_pass(T_{}, F_{});
      __syncthreads();
      // Column pass (thread per column): the strictly-lower entries of the own
      // rows contribute conj(A[r][c]) v_r to p[c] through Hermitian symmetry.
      // No atomics: one thread owns each column.
      if (active) {
        for (int c = j + 1 + tid; c < n; c += nt) {
          const int ic = (c + 1 - q + C - 1) / C > 0 ? (c + 1 - q + C - 1) / C : 0;  // own rows r > c
          CX acc = czero<CX>();
          int i = ic > i0 ? ic : i0;
          if constexpr (!OVERFLOW) {
            // walk the packed rows: offset(i + 1) - offset(i) = q + 1 + C i
            const CX* a = rows + row_offset(i, q, C) + c;
            const CX* vr = v + q + i * C;
            int stride = q + 1 + C * i;
            for (; i < nown; ++i) {
              cfma(acc, cconj(*a), *vr);
              a += stride;
              stride += C;
              vr += C;
            }
          } else {
            for (; i < nown; ++i) {
              const int r = q + i * C;
              cfma(acc, cconj(rowp(i)[c]), v[r]);
            }
          }
          pp[c] = cadd(pp[c], acc);
        }
      }
    }
    cluster.sync();
    // p = tau * sum_k pp_k ; K = -1/2 tau (p^H v) ; w = p + K v   (rows >= j+1, full length)
    CX kpart = czero<CX>();
    for (int r = j + 1 + tid; r < n; r += nt) {
      CX acc = czero<CX>();
      for (int k = 0; k < C; ++k) acc = cadd(acc, cluster.map_shared_rank(pp, k)[r]);
      const CX pr = cmul(t, acc);
      w[r] = pr;
      cfmac(kpart, pr, v[r]);
    }
    R kr = kpart.x, ki = kpart.y;
    block_sum2(kr, ki, red);
    const CX K = cscale(cmul(t, mk<CX>(kr, ki)), R(-0.5));
    for (int r = j + 1 + tid; r < n; r += nt) w[r] = cadd(w[r], cmul(K, v[r]));
    __syncthreads();
    // update column j+1 of own rows r >= j+1 (next reflector's column)
    if (active) {
      const CX vc = v[j + 1], wc = w[j + 1];
      const int i0 = (j + 1 - q + C - 1) / C > 0 ? (j + 1 - q + C - 1) / C : 0;
      for (int i = i0 + tid; i < nown; i += nt) {
        const int r = q + i * C;
        CX* a = rowp(i) + (j + 1);
        CX val = *a;
        val = csub(val, cmul(v[r], cconj(wc)));
        val = csub(val, cmul(w[r], cconj(vc)));
        *a = val;
      }
    }
    // keep (v, w) for the fused update of the next step (columns >= j+2)
    for (int r = j + 1 + tid; r < n; r += nt) {
      vprev[r] = v[r];
      wprev[r] = w[r];
    }
    prev_active = active;
    __syncthreads();
  }
  if (q == ((n - 1) % C) && tid == 0) {
    d[n - 1] = rowp((n - 1) / C)[n - 1].x;
    e[n - 1] = 0;
  }
  cluster.sync();  // keep every CTA's shared memory alive until remote readers finish
}

}  // namespace

// Shared memory bytes for cluster size C and matrix size n when every row fits.
size_t tridiag_cluster_smem(int esz, int n, int C) {
  size_t best = 0;
  for (int q = 0; q < C && q < n; ++q) {
    const int nown = (n - q + C - 1) / C;
    const size_t elems = (size_t)nown * (q + 1) + (size_t)C * ((size_t)nown * (nown - 1) / 2);
    if (elems > best) best = elems;
  }
  return (best + 6 * (size_t)n) * esz;
}

namespace {
constexpr size_t kSmemBudget = 224 * 1024;

// Largest cluster the device can co-schedule with `smem` bytes per CTA (16 needs
// the non-portable opt-in); 0 if none.
template <typename CX>
int max_cluster(size_t smem) {
  static int cached[2][2] = {{-1, -1}, {-1, -1}};
  const int big = smem > 160 * 1024;
  int& c = cached[sizeof(CX) == 16][big];
  if (c >= 0) return c;
  c = 8;
  if (cudaFuncSetAttribute(tridiag_cluster_kernel<CX, true>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) ==
      cudaSuccess) {
    cudaFuncSetAttribute(tridiag_cluster_kernel<CX, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)kSmemBudget);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(16, 1, 1);
    cfg.blockDim = dim3(512, 1, 1);
    cfg.dynamicSmemBytes = kSmemBudget;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = 16;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int nclusters = 0;
    if (cudaOccupancyMaxActiveClusters(&nclusters, tridiag_cluster_kernel<CX, true>, &cfg) == cudaSuccess &&
        nclusters > 0)
      c = 16;
  }
  cudaGetLastError();
  return c;
}
}  // namespace

// Autotuned cluster sizes: [complex128][n bucket of 32][batch-count class], 0 = untuned.
static int g_tuned_C[2][33][3] = {};
static int g_tuned_T[2][33][3] = {};  // threads per CTA (256 or 512), 0 = 512

static int count_class(int count) { return count <= 8 ? 0 : (count <= 32 ? 1 : 2); }

static bool cluster_fits(int esz, int n, int C) {
  if (C <= 8) return tridiag_cluster_smem(esz, n, C) <= kSmemBudget || C == 8;
  return 6 * (size_t)n * esz + 64 * 1024 <= kSmemBudget;
}

// Pick the cluster size for a matrix of size n: the autotuned choice for this
// size and batch class if there is one; otherwise the smallest of 1..8 CTAs
// whose shared memory holds every row (at least 8 above n = 256, where the
// per-step work, not the barriers, dominates); else the largest cluster the
// device schedules, with the overflow rows in L2.
int tridiag_cluster_size_for(int esz, int n, int count) {
  const int t = g_tuned_C[esz == 16][(n + 31) / 32][count_class(count)];
  if (t > 0 && cluster_fits(esz, n, t)) return t;
  return tridiag_cluster_size(esz, n);
}

int tridiag_cluster_size(int esz, int n) {
  const int lo = n > 256 ? 8 : 1;
  for (int C = lo; C <= 8; ++C)
    if (tridiag_cluster_smem(esz, n, C) <= kSmemBudget) return C;
  if (6 * (size_t)n * esz + 64 * 1024 > kSmemBudget) return 0;
  return esz == 8 ? max_cluster<float2>(kSmemBudget) : max_cluster<double2>(kSmemBudget);
}

template <typename CX>
int launch_tridiag_cluster_C(const HeevdProb* probs, int count, int maxn, int C, cudaStream_t s, int threads = 512);

template <typename CX>
int launch_tridiag_cluster(const HeevdProb* probs, int count, int maxn, cudaStream_t s) {
  const int C = tridiag_cluster_size_for(sizeof(CX), maxn, count);
  const int tb = g_tuned_C[sizeof(CX) == 16][(maxn + 31) / 32][count_class(count)] == C
                     ? g_tuned_T[sizeof(CX) == 16][(maxn + 31) / 32][count_class(count)]
                     : 0;
  return launch_tridiag_cluster_C<CX>(probs, count, maxn, C, s, tb > 0 ? tb : 512);
}

template <typename CX>
int launch_tridiag_cluster_C(const HeevdProb* probs, int count, int maxn, int C, cudaStream_t s, int threads) {
  const int esz = sizeof(CX);
  if (C == 0) return AGB_ERR_UNSUPPORTED;
  size_t smem = tridiag_cluster_smem(esz, maxn, C);
  const bool overflow = smem > kSmemBudget;
  if (overflow) smem = kSmemBudget;
  const int cap_elems = (int)(smem / esz) - 6 * maxn;
  auto kern = overflow ? tridiag_cluster_kernel<CX, true> : tridiag_cluster_kernel<CX, false>;
  if (C > 8) cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(count * C, 1, 1);
  cfg.blockDim = dim3(threads, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = C;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cudaError_t err = cudaLaunchKernelEx(&cfg, kern, probs, C, cap_elems);
  agb_note_launch();
  if (err != cudaSuccess) {
    agb_note_error(__FILE__, __LINE__, err);
    return AGB_ERR_CUDA;
  }
  return AGB_OK;
}

template int launch_tridiag_cluster<float2>(const HeevdProb*, int, int, cudaStream_t);
template int launch_tridiag_cluster<double2>(const HeevdProb*, int, int, cudaStream_t);

// ---------------------------------------------------------------------------
// Autotuner: time every admissible cluster size on `count` synthetic Hermitian
// n x n problems (Philox Gaussian entries, the batch shape the pipeline will
// launch) and remember the fastest for this size bucket and batch class.
namespace {
template <typename CX>
__global__ void tune_fill_kernel(HeevdProb* probs, char* base, int count, int n, size_t stride, int esz,
                                 uint64_t seed) {
  const int b = blockIdx.y;
  if (b >= count) return;
  char* slab = base + (size_t)b * stride;
  CX* H = (CX*)slab;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    HeevdProb p = {};
    p.H = H;
    p.ldh = n;
    p.n = n;
    p.ell = 1;
    p.nvec = 1;
    heevd_assign_scratch_dev(p, slab + agb_align((size_t)n * n * esz), esz);
    probs[b] = p;
  }
  typedef typename cx_traits<CX>::R R;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < (int64_t)n * n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int r = (int)(i / n), c = (int)(i % n);
    const int lo = r < c ? r : c, hi = r < c ? c : r;
    const uint64_t ctr = ((uint64_t)b * n + hi) * n + lo;
    R re = (R)philox_normal(seed, ctr, 0x21u), im = (R)philox_normal(seed, ctr, 0x22u);
    if (r == c) im = 0;
    if (r < c) im = -im;
    H[i] = mk<CX>(re, im);
  }
}

template <typename CX>
int tune_impl(int n, int count, void* ws, size_t ws_bytes, cudaStream_t s, int* best_C, float* best_ms) {
  const int esz = sizeof(CX);
  const size_t stride = agb_align((size_t)n * n * esz) + agb_align(heevd_scratch_bytes(esz, n, 1));
  const size_t need = agb_align((size_t)count * sizeof(HeevdProb)) + (size_t)count * stride;
  if (ws_bytes < need) return AGB_ERR_WORKSPACE;
  HeevdProb* probs = (HeevdProb*)ws;
  char* base = (char*)ws + agb_align((size_t)count * sizeof(HeevdProb));
  int cands[8], nc = 0;
  const int all[] = {1, 2, 4, 6, 8, 16};
  const int maxC = tridiag_cluster_size(esz, n) > 8 ? 16 : 8;
  for (int C : all)
    if (C <= maxC && C <= n && cluster_fits(esz, n, C)) cands[nc++] = C;
  cudaEvent_t e0, e1;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) return AGB_ERR_CUDA;
  int bC = 0, bT = 512;
  float bms = 1e30f;
  for (int k = 0; k < 2 * nc; ++k) {
    const int thr = (k & 1) ? 256 : 512;
    float tot = 0;
    for (int rep = 0; rep < 3; ++rep) {
      tune_fill_kernel<CX><<<dim3(64, count), 256, 0, s>>>(probs, base, count, n, stride, esz, 1234 + rep);
      cudaEventRecord(e0, s);
      const int rc = launch_tridiag_cluster_C<CX>(probs, count, n, cands[k / 2], s, thr);
      cudaEventRecord(e1, s);
      if (rc != AGB_OK) {
        cudaGetLastError();
        tot = 1e30f;
        break;
      }
      cudaEventSynchronize(e1);
      float ms = 0;
      cudaEventElapsedTime(&ms, e0, e1);
      if (rep > 0) tot += ms;  // first repetition warms up
    }
    if (tot < bms) {
      bms = tot;
      bC = cands[k / 2];
      bT = thr;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (cudaGetLastError() != cudaSuccess || bC == 0) return AGB_ERR_CUDA;
  g_tuned_C[esz == 16][(n + 31) / 32][count_class(count)] = bC;
  g_tuned_T[esz == 16][(n + 31) / 32][count_class(count)] = bT;
  if (best_C) *best_C = bC;
  if (best_ms) *best_ms = bms / 2;
  return AGB_OK;
}
}  // namespace

extern "C" size_t agb_tune_tridiag_workspace(int dtype, int n, int count) {
  const int esz = dtype == AGB_C64 ? 8 : 16;
  if (n <= 0 || count <= 0) return 0;
  return agb_align((size_t)count * sizeof(HeevdProb)) +
         (size_t)count * (agb_align((size_t)n * n * esz) + agb_align(heevd_scratch_bytes(esz, n, 1)));
}

extern "C" int agb_tune_tridiag(int dtype, int n, int count, void* ws, size_t ws_bytes, void* stream, int* best_C,
                                float* best_ms) {
  if (dtype != AGB_C64 && dtype != AGB_C128) return AGB_ERR_ARG;
  if (n <= 1 || n > 1024 || count <= 0 || !ws) return AGB_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  if (dtype == AGB_C64) return tune_impl<float2>(n, count, ws, ws_bytes, s, best_C, best_ms);
  return tune_impl<double2>(n, count, ws, ws_bytes, s, best_C, best_ms);
}

extern "C" int agb_tuned_tridiag_cluster(int dtype, int n, int count) {
  if (dtype != AGB_C64 && dtype != AGB_C128) return -1;
  if (n <= 0 || n > 1024 || count <= 0) return -1;
  const int esz = dtype == AGB_C64 ? 8 : 16;
  return tridiag_cluster_size_for(esz, n, count);
}

extern "C" int agb_set_tridiag_cluster(int dtype, int n, int count, int C, int threads) {
  if (dtype != AGB_C64 && dtype != AGB_C128) return AGB_ERR_ARG;
  if (n <= 0 || n > 1024 || count <= 0 || C < 0 || C > 16 || (threads != 256 && threads != 512)) return AGB_ERR_ARG;
  const int esz = dtype == AGB_C64 ? 8 : 16;
  if (C > 0 && (C > n || !cluster_fits(esz, n, C))) return AGB_ERR_UNSUPPORTED;
  if (C > tridiag_cluster_size(esz, n) && C > 8) {
    // a non-portable size must be one the device schedules
    const int maxC = esz == 8 ? max_cluster<float2>(kSmemBudget) : max_cluster<double2>(kSmemBudget);
    if (C > maxC) return AGB_ERR_UNSUPPORTED;
  }
  g_tuned_C[esz == 16][(n + 31) / 32][count_class(count)] = C;
  g_tuned_T[esz == 16][(n + 31) / 32][count_class(count)] = C > 0 ? threads : 0;
  return AGB_OK;
}
