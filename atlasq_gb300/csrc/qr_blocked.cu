// Blocked Householder QR on a thread-block cluster (sm_103a), for the
// canonicalisation sweeps (QR of a site tensor, up to ~1000 x 512).
//
// Same factorisation as qr_kernel (zgeqr2 reflectors H_i = I - tau_i v_i v_i^H,
// beta = -sign(Re alpha) ||x||, thin Q = H_0 H_1 ... applied to [I; 0]),
// reorganised in panels of QB columns (zgeqrf / zlarft / zlarfb):
//
// * Columns are dealt to the C CTAs of one cluster in panels, block-cyclically
//   (panel p -> CTA p mod C); each CTA keeps its panels column-major in shared
//   memory.
// * Panel p is factored by its owner alone: warp w holds panel column w; per
//   column the owner warp forms the reflector and one block barrier publishes
//   it to the warps that apply it to their columns.  The owner then forms the
//   triangular factor T_p of H_pb ... H_pb+QB-1 = I - V T V^H (forward,
//   columnwise) and writes V_p (explicit zeros above the unit diagonal) and
//   T_p to global memory (L2).
// * One cluster barrier per panel; every CTA then applies Q_p^H = I - V T^H V^H
//   to its later panels from a shared-memory copy of V_p:
//   W = V^H Y, W = T^H W, Y -= V W.
// * The thin Q is formed backwards, Z = Q_p Z from Z = [I; 0], each CTA on its
//   own columns with V_p, T_p read back from L2: no barrier between CTAs.
//
// One cluster barrier per QB columns (the unblocked cluster kernel needs two
// per column), and the trailing updates are QB-wide instead of rank-1.
#include <cooperative_groups.h>

#include "common.cuh"

namespace cg = cooperative_groups;

namespace {

constexpr int QBT = 512;  // threads per CTA (16 warps)
constexpr size_t kQrbSmemBudget = 220 * 1024;
constexpr int kQrbMaxCols = 256;  // own columns per CTA (npo * QB)

template <typename CX> struct QrbCfg;
template <> struct QrbCfg<float2> { static constexpr int QB = 16; };
template <> struct QrbCfg<double2> { static constexpr int QB = 8; };

struct QrbLayout {
  int QB, C, P, PF, npo, ld;
  size_t panels, vloc, w, w2, t, vb, total;  // byte offsets
};

AGB_HD QrbLayout qrb_layout(int esz, int QB, int M, int N, int C) {
  QrbLayout L;
  L.QB = QB;
  L.C = C;
  const int kk = M < N ? M : N;
  L.P = (N + QB - 1) / QB;
  L.PF = (kk + QB - 1) / QB;
  L.npo = (L.P + C - 1) / C;
  L.ld = M + 1;  // odd column stride: lanes reading one row of different columns hit different banks
  size_t o = 0;
  L.panels = o; o += (size_t)L.npo * QB * L.ld * esz;
  L.vloc = o;   o += (size_t)QB * L.ld * esz;
  L.w = o;      o += (size_t)QB * L.npo * QB * esz;
  L.w2 = o;     o += (size_t)QB * L.npo * QB * esz;
  L.t = o;      o += (size_t)QB * QB * esz;
  L.vb = o;     o += (size_t)2 * M * esz;
  L.total = o;
  return L;
}

// Y <- (I - V op(T) V^H) Y on rows [r0, M) of ncol local columns (column j of
// Y at Y + ycols[j] * ld).  op(T) = T^H when herm (Q_p^H), T otherwise (Q_p).
// V (QB columns, stride ld, rows r0..M-1 valid) and T are in shared memory;
// QB and ncol are multiples of 4.  Register tiles of 4 x 4 keep the
// shared-memory traffic at two loads per four complex FMAs.
template <typename CX>
AGB_DEV void qrb_apply(CX* Y, const int* ycols, int ncol, const CX* V, const CX* T, CX* W, CX* W2, int r0, int M,
                       int ld, int QB, bool herm) {
  typedef typename cx_traits<CX>::R Rt;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  constexpr int NW = QBT / 32;
  if (ncol == 0) return;
  // W = V^H Y: a warp per 4 x 4 tile of W, lanes split the rows; the 32 partial
  // sums (16 complex) are reduced so that lane l ends with sum number l
  const int ti_n = QB / 4, tj_n = ncol / 4;
  for (int tile = wid; tile < ti_n * tj_n; tile += NW) {
    const int i0 = (tile / tj_n) * 4, y0 = (tile % tj_n) * 4;
    const CX* vc[4];
    const CX* yc[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      vc[k] = V + (size_t)(i0 + k) * ld;
      yc[k] = Y + (size_t)ycols[y0 + k] * ld;
    }
    Rt a[32];
#pragma unroll
    for (int k = 0; k < 32; ++k) a[k] = 0;
    for (int r = r0 + lane; r < M; r += 32) {
      CX v[4], y[4];
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        v[k] = vc[k][r];
        y[k] = yc[k][r];
      }
#pragma unroll
      for (int ii = 0; ii < 4; ++ii)
#pragma unroll
        for (int jj = 0; jj < 4; ++jj) {
          // conj(v) * y
          a[(ii * 4 + jj) * 2] = fma(v[ii].x, y[jj].x, fma(v[ii].y, y[jj].y, a[(ii * 4 + jj) * 2]));
          a[(ii * 4 + jj) * 2 + 1] = fma(v[ii].x, y[jj].y, fma(-v[ii].y, y[jj].x, a[(ii * 4 + jj) * 2 + 1]));
        }
    }
#pragma unroll
    for (int o = 16, n = 32; o >= 1; o >>= 1, n >>= 1) {
      const bool up = (lane & o) != 0;
#pragma unroll
      for (int k = 0; k < n / 2; ++k) {
        const Rt send = up ? a[k] : a[k + n / 2];
        const Rt keep = up ? a[k + n / 2] : a[k];
        a[k] = keep + __shfl_xor_sync(0xffffffffu, send, o);
      }
    }
    // lane l holds value l = ((ii * 4 + jj) * 2 + component)
    const int comp = lane & 1, jj = (lane >> 1) & 3, ii = lane >> 3;
    Rt* wp = (Rt*)&W[(i0 + ii) * ncol + y0 + jj];
    wp[comp] = a[0];
  }
  __syncthreads();
  // W2 = op(T) W   (T upper triangular)
  for (int pr = tid; pr < QB * ncol; pr += QBT) {
    const int i = pr / ncol, y = pr % ncol;
    CX acc = czero<CX>();
    if (herm) {
      for (int k = 0; k <= i; ++k) cfmac(acc, T[k * QB + i], W[k * ncol + y]);  // conj(T[k][i]) W[k][y]
    } else {
      for (int k = i; k < QB; ++k) cfma(acc, T[i * QB + k], W[k * ncol + y]);
    }
    W2[pr] = acc;
  }
  __syncthreads();
  // Y -= V W2: a warp per block of 128 rows x 4 columns, lane rows r, r+32, r+64, r+96
  const int L = M - r0;
  const int rb_n = (L + 127) / 128;
  for (int task = wid; task < rb_n * tj_n; task += NW) {
    const int rbase = r0 + (task / tj_n) * 128 + lane, y0 = (task % tj_n) * 4;
    CX acc[4][4];
#pragma unroll
    for (int jr = 0; jr < 4; ++jr)
#pragma unroll
      for (int jc = 0; jc < 4; ++jc) acc[jr][jc] = czero<CX>();
    for (int i = 0; i < QB; ++i) {
      CX v[4], w[4];
#pragma unroll
      for (int jr = 0; jr < 4; ++jr) {
        const int r = rbase + 32 * jr;
        v[jr] = (r < M) ? V[(size_t)i * ld + r] : czero<CX>();
      }
#pragma unroll
      for (int jc = 0; jc < 4; ++jc) w[jc] = W2[i * ncol + y0 + jc];
#pragma unroll
      for (int jr = 0; jr < 4; ++jr)
#pragma unroll
        for (int jc = 0; jc < 4; ++jc) cfma(acc[jr][jc], v[jr], w[jc]);
    }
#pragma unroll
    for (int jc = 0; jc < 4; ++jc) {
      CX* yc = Y + (size_t)ycols[y0 + jc] * ld;
#pragma unroll
      for (int jr = 0; jr < 4; ++jr) {
        const int r = rbase + 32 * jr;
        if (r < M) yc[r] = csub(yc[r], acc[jr][jc]);
      }
    }
  }
  __syncthreads();
}

template <typename CX, int NK>
__global__ void __launch_bounds__(QBT, 1)
    qr_blocked_kernel(const CX* __restrict__ Ain, int M, int N, int transA, CX* Q, CX* R, int trans_out, CX* Vg,
                      CX* Tg, int C) {
  typedef typename cx_traits<CX>::R Rt;
  constexpr int QB = QrbCfg<CX>::QB;
  cg::cluster_group cluster = cg::this_cluster();
  const int q = (int)cluster.block_rank();
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int kk = M < N ? M : N;
  const QrbLayout Lo = qrb_layout(sizeof(CX), QB, M, N, C);
  const int ld = Lo.ld;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  CX* pan = (CX*)(smem_raw + Lo.panels);  // own panels: local column s * QB + jj
  CX* Vl = (CX*)(smem_raw + Lo.vloc);
  CX* W = (CX*)(smem_raw + Lo.w);
  CX* W2 = (CX*)(smem_raw + Lo.w2);
  CX* Tl = (CX*)(smem_raw + Lo.t);
  CX* vbuf = (CX*)(smem_raw + Lo.vb);  // [2][M] the current reflector, double-buffered
  __shared__ int ycols[kQrbMaxCols];
  __shared__ int ycount;
  __shared__ CX taus[QB];
  __shared__ CX Ssh[QB * QB];
  // own panels: p = q + s * C
  const int nown = (q < Lo.P) ? (Lo.P - q + C - 1) / C : 0;
  // ---- load own columns of op(A)
  for (int s = 0; s < nown; ++s) {
    const int p = q + s * C;
    for (int jj = wid; jj < QB; jj += QBT / 32) {
      const int c = p * QB + jj;
      CX* col = pan + (size_t)(s * QB + jj) * ld;
      for (int r = lane; r < M; r += 32)
        col[r] = (c < N) ? (transA ? Ain[(int64_t)c * M + r] : Ain[(int64_t)r * N + c]) : czero<CX>();
    }
  }
  __syncthreads();
  // ---- factorisation, panel by panel
  for (int p = 0; p < Lo.PF; ++p) {
    const int pb = p * QB;
    const int owner = p % C;
    if (q == owner) {
      const int s = p / C;
      CX* P0 = pan + (size_t)(s * QB) * ld;
      const int pw = min(QB, N - pb);  // columns in the panel
      const int bw = min(QB, kk - pb);  // columns factored
      // The panel in registers: warp w holds column w, lane `lane` its rows
      // lane + 32 k.  Per column the owner warp forms the reflector and writes
      // v to a shared vector (double-buffered by column parity: the next
      // owner cannot overwrite it before every warp has passed the barrier of
      // the column in between); one block barrier; the later warps apply it.
      CX x[NK];
      if (wid < pw) {
        const CX* col = P0 + (size_t)wid * ld;
#pragma unroll
        for (int k = 0; k < NK; ++k) {
          const int r = lane + 32 * k;
          x[k] = (r < M) ? col[r] : czero<CX>();
        }
      }
      for (int jj = 0; jj < bw; ++jj) {
        const int c = pb + jj;
        CX* vb = vbuf + (size_t)(jj & 1) * M;
        if (wid == jj) {
          Rt part = 0;
          CX am = czero<CX>();
#pragma unroll
          for (int k = 0; k < NK; ++k) {
            const int r = lane + 32 * k;
            if (r > c && r < M) part += cabs2(x[k]);
            if (r == c) am = x[k];
          }
          const Rt xn2 = warp_sum(part);
          CX alpha;
          alpha.x = __shfl_sync(0xffffffffu, am.x, c & 31);
          alpha.y = __shfl_sync(0xffffffffu, am.y, c & 31);
          CX t = czero<CX>(), sc = czero<CX>();
          Rt beta;
          if (xn2 == Rt(0) && alpha.y == Rt(0)) {
            beta = alpha.x;
          } else {
            beta = -copysign(sqrt(alpha.x * alpha.x + alpha.y * alpha.y + xn2), alpha.x);
            t = mk<CX>((beta - alpha.x) / beta, -alpha.y / beta);
            sc = cinv(csub(alpha, mk<CX>(beta, 0)));
          }
#pragma unroll
          for (int k = 0; k < NK; ++k) {
            const int r = lane + 32 * k;
            if (r < M) {
              CX v = czero<CX>();
              if (r == c) {
                v = mk<CX>(1, 0);
                x[k] = mk<CX>(beta, 0);
              } else if (r > c) {
                x[k] = cmul(x[k], sc);  // v below the diagonal
                v = x[k];
              }
              vb[r] = v;
            }
          }
          if (lane == 0) taus[jj] = t;
        }
        __syncthreads();
        // H_c^H = I - conj(tau) v v^H on the panel's later columns
        if (wid > jj && wid < pw) {
          const CX t = taus[jj];
          if (t.x != Rt(0) || t.y != Rt(0)) {
            CX a0 = czero<CX>(), a1 = czero<CX>();
#pragma unroll
            for (int k = 0; k < NK; ++k) {
              const int r = lane + 32 * k;
              if (r >= c && r < M) {
                if (k & 1) cfmac(a1, vb[r], x[k]);
                else cfmac(a0, vb[r], x[k]);
              }
            }
            const CX acc = warp_csum(cadd(a0, a1));
            const CX tw = cmul(cconj(t), acc);
#pragma unroll
            for (int k = 0; k < NK; ++k) {
              const int r = lane + 32 * k;
              if (r >= c && r < M) x[k] = csub(x[k], cmul(vb[r], tw));
            }
          }
        }
      }
      if (wid < pw) {
        CX* col = P0 + (size_t)wid * ld;
#pragma unroll
        for (int k = 0; k < NK; ++k) {
          const int r = lane + 32 * k;
          if (r < M) col[r] = x[k];
        }
      }
      __syncthreads();
      // V_p to global (explicit zeros above the unit diagonal; zero columns past bw)
      CX* Vp = Vg + (size_t)p * QB * M;
      for (int idx = tid; idx < QB * M; idx += QBT) {
        const int jj = idx / M, r = idx % M;
        const int c = pb + jj;
        CX v = czero<CX>();
        if (jj < bw) v = (r < c) ? czero<CX>() : (r == c ? mk<CX>(1, 0) : P0[(size_t)jj * ld + r]);
        Vp[idx] = v;
      }
      // S[k][i] = v_k^H v_i (k < i), pairs round-robin over the warps
      for (int pr = wid; pr < QB * QB; pr += QBT / 32) {
        const int k = pr / QB, i = pr % QB;
        if (k < i && i < bw) {
          const CX* vk = P0 + (size_t)k * ld;
          const CX* vi = P0 + (size_t)i * ld;
          const int ci = pb + i;
          CX acc = czero<CX>();
          for (int r = ci + lane; r < M; r += 32)
            cfmac(acc, vk[r], (r == ci) ? mk<CX>(1, 0) : vi[r]);  // v_k[ci] is below v_k's diagonal
          acc = warp_csum(acc);
          if (lane == 0) Ssh[pr] = acc;
        }
      }
      __syncthreads();
      // T (forward, columnwise): T[i][i] = tau_i, T[0:i][i] = -tau_i T[0:i][0:i] S[0:i][i];
      // lane k of warp 0 holds row k of T in registers
      if (wid == 0) {
        CX trow[QB];
#pragma unroll
        for (int m = 0; m < QB; ++m) trow[m] = czero<CX>();
#pragma unroll
        for (int i = 0; i < QB; ++i) {
          if (i < bw) {
            const CX ti = taus[i];
            CX acc = czero<CX>();
#pragma unroll
            for (int m = 0; m < i; ++m)
              if (m >= lane) cfma(acc, trow[m], Ssh[m * QB + i]);
            if (lane < i) trow[i] = cmul(mk<CX>(-ti.x, -ti.y), acc);
            else if (lane == i) trow[i] = ti;
          }
        }
        CX* Tp = Tg + (size_t)p * QB * QB;
        if (lane < QB)
#pragma unroll
          for (int m = 0; m < QB; ++m) Tp[lane * QB + m] = trow[m];
      }
      __threadfence();  // V_p, T_p visible to the cluster before the barrier
    }
    cluster.sync();
    // Q_p^H on own later panels (p' > p)
    if (tid == 0) {
      int nc = 0;
      for (int s = 0; s < nown; ++s) {
        const int pp = q + s * C;
        if (pp > p)
          for (int jj = 0; jj < QB; ++jj) ycols[nc++] = s * QB + jj;
      }
      ycount = nc;
    }
    __syncthreads();
    const int ncol = ycount;
    if (ncol > 0) {
      const CX* Vp = Vg + (size_t)p * QB * M;
      for (int idx = tid; idx < QB * (M - pb); idx += QBT) {
        const int jj = idx / (M - pb), r = pb + idx % (M - pb);
        Vl[(size_t)jj * ld + r] = __ldcg(Vp + (size_t)jj * M + r);
      }
      for (int e = tid; e < QB * QB; e += QBT) Tl[e] = __ldcg(Tg + (size_t)p * QB * QB + e);
      __syncthreads();
      qrb_apply(pan, ycols, ncol, Vl, Tl, W, W2, pb, M, ld, QB, true);
    }
  }
  // ---- R = upper triangle of the factored columns (kk x N)
  for (int s = 0; s < nown; ++s) {
    const int p = q + s * C;
    for (int jj = wid; jj < QB; jj += QBT / 32) {
      const int c = p * QB + jj;
      if (c >= N) continue;
      const CX* col = pan + (size_t)(s * QB + jj) * ld;
      for (int r = lane; r < kk; r += 32) {
        const CX val = (r <= c) ? col[r] : czero<CX>();
        if (trans_out) R[(int64_t)c * kk + r] = val;
        else R[(int64_t)r * N + c] = val;
      }
    }
  }
  __syncthreads();
  // ---- thin Q: own columns c < kk, Z = [I; 0] in the panel storage, Z <- Q_p Z backwards
  for (int s = 0; s < nown; ++s) {
    const int p = q + s * C;
    for (int jj = wid; jj < QB; jj += QBT / 32) {
      const int c = p * QB + jj;
      CX* col = pan + (size_t)(s * QB + jj) * ld;
      for (int r = lane; r < M; r += 32) col[r] = (r == c && c < kk) ? mk<CX>(1, 0) : czero<CX>();
    }
  }
  __syncthreads();
  for (int p = Lo.PF - 1; p >= 0; --p) {
    const int pb = p * QB;
    if (tid == 0) {
      int nc = 0;
      for (int s = 0; s < nown; ++s) {
        const int pp = q + s * C;
        if (pp >= p && pp < Lo.PF)  // columns c < pb are e_c, untouched by Q_p
          for (int jj = 0; jj < QB; ++jj) ycols[nc++] = s * QB + jj;
      }
      ycount = nc;
    }
    __syncthreads();
    const int ncol = ycount;
    if (ncol == 0) continue;
    const CX* Vp = Vg + (size_t)p * QB * M;
    for (int idx = tid; idx < QB * (M - pb); idx += QBT) {
      const int jj = idx / (M - pb), r = pb + idx % (M - pb);
      Vl[(size_t)jj * ld + r] = __ldcg(Vp + (size_t)jj * M + r);
    }
    for (int e = tid; e < QB * QB; e += QBT) Tl[e] = __ldcg(Tg + (size_t)p * QB * QB + e);
    __syncthreads();
    qrb_apply(pan, ycols, ncol, Vl, Tl, W, W2, pb, M, ld, QB, false);
  }
  // ---- write Q (M x kk, or its transpose)
  for (int s = 0; s < nown; ++s) {
    const int p = q + s * C;
    if (trans_out) {
      for (int jj = wid; jj < QB; jj += QBT / 32) {
        const int c = p * QB + jj;
        if (c >= kk) continue;
        const CX* col = pan + (size_t)(s * QB + jj) * ld;
        for (int r = lane; r < M; r += 32) Q[(int64_t)c * M + r] = col[r];
      }
    } else {
      const int nc = min(QB, kk - p * QB);
      for (int idx = tid; idx < M * (nc > 0 ? nc : 0); idx += QBT) {
        const int r = idx / nc, jj = idx % nc;
        Q[(int64_t)r * kk + p * QB + jj] = pan[(size_t)(s * QB + jj) * ld + r];
      }
    }
  }
  cluster.sync();
}

template <typename CX>
using QrbKernel = void (*)(const CX*, int, int, int, CX*, CX*, int, CX*, CX*, int);

// The instance whose per-lane register column (NK rows per lane) covers M rows;
// nullptr above 1024 rows (512 for complex128, whose columns would spill).
template <typename CX>
QrbKernel<CX> qrb_kernel_for(int M) {
  if (M <= 128) return qr_blocked_kernel<CX, 4>;
  if (M <= 256) return qr_blocked_kernel<CX, 8>;
  if (M <= 512) return qr_blocked_kernel<CX, 16>;
  if constexpr (sizeof(CX) == 8) {
    if (M <= 1024) return qr_blocked_kernel<CX, 32>;
  }
  return nullptr;
}

// Cluster size for the blocked kernel: the largest of 16, 8, 4, 2 CTAs not
// above the panel count whose shared memory fits; 0 if none.
template <typename CX>
int qrb_cluster_size(int M, int N, size_t* smem_out) {
  const QrbKernel<CX> kern = qrb_kernel_for<CX>(M);
  if (!kern) return 0;
  constexpr int QB = QrbCfg<CX>::QB;
  const int P = (N + QB - 1) / QB;
  static int allow16 = -1;
  for (int C : {16, 8, 4, 2}) {
    if (C > P) continue;
    const QrbLayout L = qrb_layout(sizeof(CX), QB, M, N, C);
    if (L.total > kQrbSmemBudget || L.npo * QB > kQrbMaxCols) continue;
    if (C == 16) {
      if (allow16 < 0) {
        allow16 = 0;
        if (cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) ==
                cudaSuccess &&
            cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)kQrbSmemBudget) == cudaSuccess) {
          cudaLaunchConfig_t cfg = {};
          cfg.gridDim = dim3(16, 1, 1);
          cfg.blockDim = dim3(QBT, 1, 1);
          cfg.dynamicSmemBytes = kQrbSmemBudget;
          cudaLaunchAttribute attr[1];
          attr[0].id = cudaLaunchAttributeClusterDimension;
          attr[0].val.clusterDim.x = 16;
          attr[0].val.clusterDim.y = 1;
          attr[0].val.clusterDim.z = 1;
          cfg.attrs = attr;
          cfg.numAttrs = 1;
          int ncl = 0;
          if (cudaOccupancyMaxActiveClusters(&ncl, kern, &cfg) == cudaSuccess && ncl > 0)
            allow16 = 1;
        }
        cudaGetLastError();
      }
      if (!allow16) continue;
    }
    if (smem_out) *smem_out = L.total;
    return C;
  }
  return 0;
}

}  // namespace

// Workspace of the blocked kernel: reflector panels (M x QB each) and T factors.
size_t qr_blocked_workspace(int esz, int M, int N) {
  const int QB = esz == 8 ? QrbCfg<float2>::QB : QrbCfg<double2>::QB;
  const int kk = M < N ? M : N;
  const int PF = (kk + QB - 1) / QB;
  return agb_align((size_t)PF * QB * M * esz) + agb_align((size_t)PF * QB * QB * esz);
}

template <typename CX>
int launch_qr_blocked(const CX* A, int M, int N, int transA, CX* Q, CX* R, int trans_out, void* ws, size_t ws_bytes,
                      cudaStream_t s) {
  if (ws_bytes < qr_blocked_workspace(sizeof(CX), M, N)) return AGB_ERR_WORKSPACE;
  size_t smem = 0;
  const int C = qrb_cluster_size<CX>(M, N, &smem);
  if (C == 0) return AGB_ERR_UNSUPPORTED;
  const QrbKernel<CX> kern = qrb_kernel_for<CX>(M);
  if (C > 8 && cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess) {
    cudaGetLastError();
    return AGB_ERR_UNSUPPORTED;
  }
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) {
    cudaGetLastError();
    return AGB_ERR_UNSUPPORTED;
  }
  constexpr int QB = QrbCfg<CX>::QB;
  const int kk = M < N ? M : N;
  const int PF = (kk + QB - 1) / QB;
  CX* Vg = (CX*)ws;
  CX* Tg = (CX*)((char*)ws + agb_align((size_t)PF * QB * M * sizeof(CX)));
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(C, 1, 1);
  cfg.blockDim = dim3(QBT, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = C;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  const cudaError_t err = cudaLaunchKernelEx(&cfg, kern, A, M, N, transA, Q, R, trans_out, Vg, Tg, C);
  agb_note_launch();
  if (err != cudaSuccess) {
    cudaGetLastError();
    return AGB_ERR_UNSUPPORTED;
  }
  return AGB_OK;
}

template int launch_qr_blocked<float2>(const float2*, int, int, int, float2*, float2*, int, void*, size_t,
                                       cudaStream_t);
template int launch_qr_blocked<double2>(const double2*, int, int, int, double2*, double2*, int, void*, size_t,
                                        cudaStream_t);
