// Two-stage Householder tridiagonalisation of the Gram matrices (sm_103a).
//
// The one-stage reduction (tridiag_cluster.cu) needs n - 1 dependent steps,
// each a BLAS-2 pass over the trailing matrix with two cluster barriers.  Here
// the same reduction is split in two:
//
//   stage 1  band_reduce_kernel   H -> B, bandwidth BW (16 for n <= 512),
//            one cluster of C CTAs per matrix, ceil((n-1)/BW) - 1 panel steps.
//            Step p: CTA 0 factors the panel A[(p+1)BW:, pBW:(p+1)BW] = Q_p R_p
//            (Householder, in shared memory) and forms the block-reflector
//            factor T_p (Q_p = I - V T V^H); every CTA then updates its rows of
//            the trailing matrix,  A22 <- Q_p^H A22 Q_p = A22 - V Y^H - Y V^H,
//            X = A22 V T, Y = X - 1/2 V (T^H V^H X)  (four cluster barriers
//            per panel; the matrix stays in H, in L2).  R_p and V_p are left in
//            the panel (LAPACK's packed storage), T_p in the band scratch.
//   stage 2  band_to_tridiag_kernel  B -> T (real symmetric tridiagonal),
//            one CTA per matrix with the band (and room for the bulge) in
//            shared memory.  Sweep s annihilates column s below the first
//            subdiagonal with a reflector of length <= BW and chases the
//            resulting bulge down the band (task k of sweep s acts on rows
//            s+1+k BW .. s+(k+1) BW).  Warp w runs sweeps w, w+16, ...; task
//            (s, k) starts once task (s-1, k+2) has finished (the only
//            overlapping neighbour), signalled through a progress word per
//            warp in shared memory (bounded waits).
//   back-transformation  bt_two_stage_kernel  V = Q1 Q2 Y: the stage-2
//            reflectors in reverse sweep order (the tasks of one sweep act on
//            disjoint rows, so a sweep is one parallel step), then the stage-1
//            block reflectors in reverse panel order; each CTA owns 32
//            eigenvector columns held in shared memory.
//
// d, e, scale and the eigenvector layout are those of the one-stage path, so
// bisection and inverse iteration are unchanged.
#include <cooperative_groups.h>

#include "heevd.cuh"
#include "prof.cuh"

namespace cg = cooperative_groups;

namespace {

constexpr int NWARP2 = 16;              // stage-2 workers (warps) per CTA
constexpr unsigned SPIN_LIMIT = 1u << 24;  // bounded wait of a stage-2 worker (polls)

template <typename CX>
struct TwoStage {
  CX* T1;   // [npanel][BW][BW]
  CX* Yx;   // [n][BW]
  CX* RV;   // [n][kmax][BW] stage-2 reflectors (v[0] = 1 stored)
  CX* RT;   // [n][kmax]     stage-2 taus
  int kmax;
};

template <typename CX>
AGB_DEV TwoStage<CX> two_stage_layout(void* band, int n, int bw) {
  TwoStage<CX> t;
  const size_t np = (size_t)(n + bw - 1) / bw;
  const int kmax = (n - 1 + bw - 1) / bw > 0 ? (n - 1 + bw - 1) / bw : 1;
  char* b = (char*)band;
  t.T1 = (CX*)b;  b += agb_align(np * bw * bw * sizeof(CX));
  t.Yx = (CX*)b;  b += agb_align((size_t)n * bw * sizeof(CX));
  t.RV = (CX*)b;  b += agb_align((size_t)n * kmax * bw * sizeof(CX));
  t.RT = (CX*)b;
  t.kmax = kmax;
  return t;
}

// zlarfg on (alpha, x) with ||x||^2 = xn2: beta, tau, and the scale of v = x / (alpha - beta).
template <typename CX>
AGB_DEV void householder(CX alpha, typename cx_traits<CX>::R xn2, typename cx_traits<CX>::R& beta, CX& tau,
                         CX& scale) {
  typedef typename cx_traits<CX>::R R;
  if (xn2 == R(0) && alpha.y == R(0)) {
    beta = alpha.x;
    tau = czero<CX>();
    scale = czero<CX>();
    return;
  }
  beta = -copysign(sqrt(alpha.x * alpha.x + alpha.y * alpha.y + xn2), alpha.x);
  tau = mk<CX>((beta - alpha.x) / beta, -alpha.y / beta);
  scale = cinv(csub(alpha, mk<CX>(beta, 0)));
}

// =========================================================================== stage 1
template <typename CX, int BW>
__global__ void __launch_bounds__(512, 1) band_reduce_kernel(const HeevdProb* __restrict__ probs, int C) {
  typedef typename cx_traits<CX>::R R;
  cg::cluster_group cluster = cg::this_cluster();
  const int q = (int)cluster.block_rank();
  const HeevdProb P = probs[blockIdx.x / C];
  const int n = P.n;
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, wid = tid >> 5, nw = nt >> 5;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int rows_max = (n + C - 1) / C;
  // exchange buffers first, at the same offset in every CTA (remote reads)
  CX* Wp = (CX*)smem_raw;              // [BW][BW] partial V^H X of this CTA
  R* mxp = (R*)(Wp + BW * BW);         // [16]
  CX* Tp = (CX*)(mxp + 32);            // [BW][BW]
  CX* Wt = Tp + BW * BW;               // [BW][BW]
  CX* Wsum = Wt + BW * BW;             // [BW][BW]
  CX* tauS = Wsum + BW * BW;           // [BW]
  CX* Vs = tauS + BW;                  // [n][BW] panel, then V
  CX* Ws = Vs + (size_t)n * BW;        // [n][BW] V T, then Y
  CX* Xs = Ws + (size_t)n * BW;        // [rows_max][BW] own rows of X, then Y
  __shared__ R red[64];
  __shared__ CX bc[2];
  CX* H = (CX*)P.H;
  const int64_t ld = P.ldh;
  const TwoStage<CX> S = two_stage_layout<CX>(P.band, n, BW);

  // ---- scale by the largest diagonal magnitude (as the one-stage kernels)
  R mx = 0;
  for (int i = q + tid * C; i < n; i += nt * C) mx = fmax(mx, fabs(H[(int64_t)i * ld + i].x));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if (lane == 0) red[wid] = mx;
  __syncthreads();
  if (tid == 0) {
    R m = 0;
    for (int i = 0; i < nw; ++i) m = fmax(m, red[i]);
    for (int k = 0; k < C; ++k) cluster.map_shared_rank(mxp, k)[q] = m;
  }
  cluster.sync();
  mx = 0;
  for (int k = 0; k < C; ++k) mx = fmax(mx, mxp[k]);
  if (mx == R(0)) mx = R(1);
  if (q == 0 && tid == 0) *((R*)P.scale) = mx;
  const R inv = R(1) / mx;
  for (int r = q + wid * C; r < n; r += nw * C)
    for (int c = lane; c < n; c += 32) {
      CX* a = H + (int64_t)r * ld + c;
      *a = cscale(*a, inv);
    }
  cluster.sync();

  for (int p = 0;; ++p) {
    const int c0 = p * BW, r0 = c0 + BW, m = n - r0;
    if (m < 2) break;
    // ------------------------------------------------ (a) panel factorisation on CTA 0
    if (q == 0) {
      for (int e = tid; e < m * BW; e += nt) {
        const int i = e / BW, c = e % BW;
        Vs[e] = H[(int64_t)(r0 + i) * ld + c0 + c];
      }
      __syncthreads();
      for (int c = 0; c < BW; ++c) {
        R part = 0;
        for (int i = c + 1 + tid; i < m; i += nt) part += cabs2(Vs[i * BW + c]);
        const R xn2 = block_sum(part, red);
        if (tid == 0) {
          R beta;
          CX t, sc;
          if (c < m) {
            householder(Vs[c * BW + c], xn2, beta, t, sc);
            Vs[c * BW + c] = mk<CX>(beta, 0);
          } else {
            t = czero<CX>();
            sc = czero<CX>();
          }
          tauS[c] = t;
          bc[0] = sc;
        }
        __syncthreads();
        const CX sc = bc[0], t = tauS[c];
        for (int i = c + 1 + tid; i < m; i += nt) Vs[i * BW + c] = cmul(Vs[i * BW + c], sc);
        __syncthreads();
        if (t.x != R(0) || t.y != R(0)) {
          // columns k > c: a_k -= conj(tau) v (v^H a_k), one warp per column
          for (int k = c + 1 + wid; k < BW; k += nw) {
            CX dot = czero<CX>();
            for (int i = c + lane; i < m; i += 32) {
              const CX vi = (i == c) ? mk<CX>(1, 0) : Vs[i * BW + c];
              cfmac(dot, vi, Vs[i * BW + k]);
            }
            dot = warp_csum(dot);
            const CX f = cmul(cconj(t), dot);
            for (int i = c + lane; i < m; i += 32) {
              const CX vi = (i == c) ? mk<CX>(1, 0) : Vs[i * BW + c];
              Vs[i * BW + k] = csub(Vs[i * BW + k], cmul(vi, f));
            }
          }
        }
        __syncthreads();
      }
      // R (upper) and V (strictly lower) back to the panel; Gram of V's columns
      for (int e = tid; e < m * BW; e += nt) {
        const int i = e / BW, c = e % BW;
        H[(int64_t)(r0 + i) * ld + c0 + c] = Vs[e];
      }
      // Wsum[r][c] = V(:, r)^H v_c for r < c (v_c = 0 above row c, 1 at c)
      for (int pr = wid; pr < BW * BW; pr += nw) {
        const int r = pr / BW, c = pr % BW;
        if (r >= c) continue;
        CX dot = czero<CX>();
        for (int i = c + lane; i < m; i += 32) {
          const CX vr = Vs[i * BW + r];                        // i >= c > r: V part
          const CX vc = (i == c) ? mk<CX>(1, 0) : Vs[i * BW + c];
          cfmac(dot, vr, vc);
        }
        dot = warp_csum(dot);
        if (lane == 0) Wsum[pr] = dot;
      }
      __syncthreads();
      // T (upper triangular, zlarft forward columnwise): T[c][c] = tau_c,
      // T[0:c, c] = -tau_c T[0:c, 0:c] Wsum[0:c, c]
      for (int c = 0; c < BW; ++c) {
        if (tid < c) {
          CX acc = czero<CX>();
          for (int j = tid; j < c; ++j) cfma(acc, Tp[tid * BW + j], Wsum[j * BW + c]);
          Tp[tid * BW + c] = cscale(cmul(tauS[c], acc), R(-1));
        } else if (tid == c) {
          Tp[c * BW + c] = tauS[c];
        } else if (tid < BW) {
          Tp[tid * BW + c] = czero<CX>();
        }
        __syncthreads();
      }
      for (int e = tid; e < BW * BW; e += nt) S.T1[(size_t)p * BW * BW + e] = Tp[e];
      __syncthreads();
    }
    cluster.sync();  // (b) panel, V and T visible to the cluster
    // ------------------------------------------------ (c) V and T in every CTA
    for (int e = tid; e < m * BW; e += nt) {
      const int i = e / BW, c = e % BW;
      Vs[e] = (i > c) ? H[(int64_t)(r0 + i) * ld + c0 + c] : (i == c ? mk<CX>(1, 0) : czero<CX>());
    }
    if (q != 0)
      for (int e = tid; e < BW * BW; e += nt) Tp[e] = S.T1[(size_t)p * BW * BW + e];
    __syncthreads();
    // ------------------------------------------------ (d) V T
    for (int e = tid; e < m * BW; e += nt) {
      const int i = e / BW, c = e % BW;
      CX acc = czero<CX>();
      for (int k = 0; k <= c; ++k) cfma(acc, Vs[i * BW + k], Tp[k * BW + c]);
      Ws[e] = acc;
    }
    __syncthreads();
    // ------------------------------------------------ (e) X = A22 (V T), own rows i = q + u C
    const int nown = (m - q + C - 1) / C > 0 ? (m - q + C - 1) / C : 0;
    for (int u = wid; u < nown; u += nw) {
      const int i = q + u * C;
      const CX* arow = H + (int64_t)(r0 + i) * ld + r0;
      CX acc[BW];
#pragma unroll
      for (int c = 0; c < BW; ++c) acc[c] = czero<CX>();
      for (int j = lane; j < m; j += 32) {
        const CX a = arow[j];
#pragma unroll
        for (int c = 0; c < BW; ++c) cfma(acc[c], a, Ws[j * BW + c]);
      }
#pragma unroll
      for (int c = 0; c < BW; ++c) {
        const CX s = warp_csum(acc[c]);
        if (lane == 0) Xs[u * BW + c] = s;
      }
    }
    __syncthreads();
    // ------------------------------------------------ (f) partial W = V^H X over own rows
    for (int e = tid; e < BW * BW; e += nt) {
      const int c1 = e / BW, c2 = e % BW;
      CX acc = czero<CX>();
      for (int u = 0; u < nown; ++u) cfmac(acc, Vs[(q + u * C) * BW + c1], Xs[u * BW + c2]);
      Wp[e] = acc;
    }
    cluster.sync();
    // ------------------------------------------------ (g) W = sum of partials; T^H W
    for (int e = tid; e < BW * BW; e += nt) {
      CX acc = czero<CX>();
      for (int k = 0; k < C; ++k) acc = cadd(acc, cluster.map_shared_rank(Wp, k)[e]);
      Wsum[e] = acc;
    }
    __syncthreads();
    for (int e = tid; e < BW * BW; e += nt) {
      const int c1 = e / BW, c2 = e % BW;
      CX acc = czero<CX>();
      for (int k = 0; k <= c1; ++k) cfmac(acc, Tp[k * BW + c1], Wsum[k * BW + c2]);  // (T^H)[c1][k] = conj(T[k][c1])
      Wt[e] = acc;
    }
    __syncthreads();
    // ------------------------------------------------ (h) Y = X - 1/2 V (T^H W), own rows -> Yx
    for (int e = tid; e < nown * BW; e += nt) {
      const int u = e / BW, c = e % BW;
      const int i = q + u * C;
      CX acc = czero<CX>();
#pragma unroll 4
      for (int k = 0; k < BW; ++k) cfma(acc, Vs[i * BW + k], Wt[k * BW + c]);
      const CX y = csub(Xs[e], cscale(acc, R(0.5)));
      S.Yx[(size_t)i * BW + c] = y;
    }
    cluster.sync();  // every row of Y visible
    for (int e = tid; e < m * BW; e += nt) Ws[e] = S.Yx[e];
    __syncthreads();
    // ------------------------------------------------ (j) A22 -= V Y^H + Y V^H, own rows
    for (int u = wid; u < nown; u += nw) {
      const int i = q + u * C;
      CX vi[BW], yi[BW];
#pragma unroll
      for (int c = 0; c < BW; ++c) {
        vi[c] = Vs[i * BW + c];
        yi[c] = Ws[i * BW + c];
      }
      CX* arow = H + (int64_t)(r0 + i) * ld + r0;
      for (int j = lane; j < m; j += 32) {
        CX a = arow[j];
#pragma unroll
        for (int c = 0; c < BW; ++c) {
          a = csub(a, cmul(vi[c], cconj(Ws[j * BW + c])));
          a = csub(a, cmul(yi[c], cconj(Vs[j * BW + c])));
        }
        arow[j] = a;
      }
    }
    cluster.sync();  // trailing matrix updated before the next panel
  }
}

// =========================================================================== stage 2
// Band storage in shared memory: B(i, j), 0 <= i - j < 2 BW, at BD[j * LD + (i - j)].
template <typename CX, int BW>
struct Band {
  static constexpr int LD = 2 * BW + 1;
  CX* BD;
  AGB_DEV CX& at(int i, int j) const { return BD[j * LD + (i - j)]; }
};

template <typename CX, int BW>
__global__ void __launch_bounds__(NWARP2 * 32, 1) band_to_tridiag_kernel(HeevdProb* __restrict__ probs) {
  typedef typename cx_traits<CX>::R R;
  HeevdProb& Pref = probs[blockIdx.x];
  const HeevdProb P = Pref;
  const int n = P.n;
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Band<CX, BW> B;
  B.BD = (CX*)smem_raw;
  CX* vbuf = B.BD + (size_t)n * Band<CX, BW>::LD;  // [NWARP2][BW]
  CX* wbuf = vbuf + NWARP2 * BW;                   // [NWARP2][BW]
  __shared__ volatile int progress[NWARP2];
  __shared__ volatile int fail;
  const CX* H = (const CX*)P.H;
  const int64_t ld = P.ldh;
  const TwoStage<CX> S = two_stage_layout<CX>(P.band, n, BW);
  const int KM = S.kmax;
  for (int e = tid; e < n * Band<CX, BW>::LD; e += blockDim.x) {
    const int j = e / Band<CX, BW>::LD, dd = e % Band<CX, BW>::LD;
    B.BD[e] = (dd <= BW && j + dd < n) ? H[(int64_t)(j + dd) * ld + j] : czero<CX>();
  }
  if (tid < NWARP2) progress[tid] = 0;
  if (tid == 0) fail = 0;
  __syncthreads();
  CX* v = vbuf + w * BW;
  CX* wv = wbuf + w * BW;
  for (int s = w; s <= n - 2 && !fail; s += NWARP2) {
    const int K = (n - 1 - s + BW - 1) / BW;
    const int Kp = (s > 0) ? (n - s + BW - 1) / BW : 0;  // tasks of sweep s - 1
    for (int k = 0; k < K; ++k) {
      if (s > 0) {
        const int need = (s - 1) * (KM + 1) + min(k + 3, Kp);
        volatile int* pr = &progress[(s - 1) % NWARP2];
        unsigned it = 0;
        while (*pr < need && it < SPIN_LIMIT && !fail) {
          __nanosleep(20);
          ++it;
        }
        if (it >= SPIN_LIMIT) fail = 1;
        if (fail) break;
        __threadfence_block();
      }
      const int r0 = s + 1 + k * BW;
      const int len = min(BW, n - r0);
      const int cb = (k == 0) ? s : (s + 1 + (k - 1) * BW);
      // ---- reflector from column cb, rows r0 .. r0+len-1
      const CX x = (lane < len) ? B.at(r0 + lane, cb) : czero<CX>();
      R xn2 = (lane >= 1 && lane < len) ? cabs2(x) : R(0);
      xn2 = warp_sum(xn2);
      const CX alpha = mk<CX>(__shfl_sync(0xffffffffu, x.x, 0), __shfl_sync(0xffffffffu, x.y, 0));
      R beta;
      CX tau, sc;
      householder(alpha, xn2, beta, tau, sc);
      const bool act = (tau.x != R(0) || tau.y != R(0));
      if (lane < BW) {
        const CX vi = (lane == 0) ? mk<CX>(1, 0) : (lane < len ? cmul(x, sc) : czero<CX>());
        v[lane] = vi;
        S.RV[((size_t)s * KM + k) * BW + lane] = vi;
      }
      if (lane == 0) S.RT[(size_t)s * KM + k] = tau;
      if (lane < len) B.at(r0 + lane, cb) = (lane == 0) ? mk<CX>(act ? beta : alpha.x, act ? R(0) : alpha.y)
                                                         : (act ? czero<CX>() : x);
      __syncwarp();
      if (act) {
        // ---- lanes 0..BW-1: p = tau D v (D = B(r0.., r0..), Hermitian);
        //      lanes BW..2BW-1: t = E v for E = B(r0+BW.., r0..)
        const int len2 = min(BW, n - r0 - BW);
        CX acc = czero<CX>();
        if (lane < len) {
          const int i = lane;
          for (int j = 0; j < len; ++j) {
            const CX d = (i >= j) ? B.at(r0 + i, r0 + j) : cconj(B.at(r0 + j, r0 + i));
            cfma(acc, d, v[j]);
          }
          acc = cmul(tau, acc);
        } else if (lane >= BW && lane - BW < len2) {
          const int i2 = lane - BW;
          for (int j = 0; j < len; ++j) cfma(acc, B.at(r0 + BW + i2, r0 + j), v[j]);
        }
        // coef = 1/2 conj(tau) (v^H p)
        CX vp = (lane < len) ? mk<CX>(v[lane].x * acc.x + v[lane].y * acc.y, v[lane].x * acc.y - v[lane].y * acc.x)
                             : czero<CX>();
        vp = warp_csum(vp);
        const CX coef = cscale(cmul(cconj(tau), vp), R(0.5));
        if (lane < len) {
          wv[lane] = csub(acc, cmul(coef, v[lane]));
        } else if (lane >= BW && lane - BW < len2) {
          // E <- E H = E - tau (E v) v^H
          const int i2 = lane - BW;
          const CX f = cmul(tau, acc);
          for (int j = 0; j < len; ++j) {
            CX& e = B.at(r0 + BW + i2, r0 + j);
            e = csub(e, cmul(f, cconj(v[j])));
          }
        }
        __syncwarp();
        if (lane < len) {
          // D <- D - v w^H - w v^H on the lower triangle, lane j owns column j
          const int j = lane;
          const CX vj = v[j], wj = wv[j];
          for (int i = j; i < len; ++i) {
            CX& d = B.at(r0 + i, r0 + j);
            d = csub(d, cadd(cmul(v[i], cconj(wj)), cmul(wv[i], cconj(vj))));
          }
        } else if (k >= 1 && lane >= BW && lane - BW < BW - 1) {
          // left application to the rest of the bulge: column c = cb + 1 + (lane - BW)
          const int c = cb + 1 + (lane - BW);
          CX dot = czero<CX>();
          for (int i = 0; i < len; ++i) cfmac(dot, v[i], B.at(r0 + i, c));
          const CX f = cmul(cconj(tau), dot);
          for (int i = 0; i < len; ++i) {
            CX& z = B.at(r0 + i, c);
            z = csub(z, cmul(v[i], f));
          }
        }
      }
      __syncwarp();
      __threadfence_block();
      if (lane == 0) progress[w] = s * (KM + 1) + k + 1;
    }
  }
  __syncthreads();
  if (fail) {
    if (tid == 0) Pref.fail = 1;
    return;
  }
  R* d = (R*)P.d;
  R* e = (R*)P.e;
  for (int i = tid; i < n; i += blockDim.x) {
    d[i] = B.at(i, i).x;
    e[i] = (i + 1 < n) ? B.at(i + 1, i).x : R(0);
  }
}

// =========================================================================== back-transformation
template <typename CX, int BW, int NC>
__global__ void __launch_bounds__(512, 1) bt_two_stage_kernel(const HeevdProb* __restrict__ probs) {
  typedef typename cx_traits<CX>::R R;
  const HeevdProb P = probs[blockIdx.y];
  const int n = P.n, ell = P.ell, nv = P.nvec;
  const int col0 = blockIdx.x * NC;
  if (col0 >= nv || P.skip_vectors) return;
  const int ncol = min(NC, nv - col0);
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5, nw = blockDim.x >> 5;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  CX* Z = (CX*)smem_raw;                // [n][NC]
  CX* Vp = Z + (size_t)n * NC;          // [n][BW] stage-1 panel V
  CX* Wb = Vp + (size_t)n * BW;         // [BW][NC]
  CX* Tb = Wb + BW * NC;                // [BW][BW]
  const TwoStage<CX> S = two_stage_layout<CX>(P.band, n, BW);
  const int KM = S.kmax;
  const R* Y = (const R*)P.Y;
  for (int e = tid; e < n * NC; e += blockDim.x) {
    const int i = e / NC, c = e % NC;
    Z[e] = (c < ncol) ? mk<CX>(Y[(int64_t)i * ell + col0 + c], 0) : czero<CX>();
  }
  __syncthreads();
  // ---- Q2: sweeps in reverse order; the tasks of a sweep (disjoint rows) in parallel,
  //      one warp per task, lanes over the columns
  for (int s = n - 2; s >= 0; --s) {
    const int K = (n - 1 - s + BW - 1) / BW;
    for (int k = wid; k < K; k += nw) {
      const CX t = S.RT[(size_t)s * KM + k];
      if (t.x == R(0) && t.y == R(0)) continue;
      const int r0 = s + 1 + k * BW;
      const int len = min(BW, n - r0);
      const CX* vv = S.RV + ((size_t)s * KM + k) * BW;
      if (lane < NC) {
        CX dot = czero<CX>();
        for (int i = 0; i < len; ++i) cfmac(dot, vv[i], Z[(r0 + i) * NC + lane]);
        const CX f = cmul(t, dot);
        for (int i = 0; i < len; ++i) {
          CX& z = Z[(r0 + i) * NC + lane];
          z = csub(z, cmul(vv[i], f));
        }
      }
    }
    __syncthreads();
  }
  // ---- Q1: panels in reverse order, Z[r0:, :] -= V (T (V^H Z[r0:, :]))
  const int npan = (n - 2) / BW > 0 ? (n - 2 + BW - 1) / BW : 0;
  for (int p = npan; p >= 0; --p) {
    const int c0 = p * BW, r0 = c0 + BW, m = n - r0;
    if (m < 2) continue;
    const CX* H = (const CX*)P.H;
    for (int e = tid; e < m * BW; e += blockDim.x) {
      const int i = e / BW, c = e % BW;
      Vp[e] = (i > c) ? H[(int64_t)(r0 + i) * P.ldh + c0 + c] : (i == c ? mk<CX>(1, 0) : czero<CX>());
    }
    for (int e = tid; e < BW * BW; e += blockDim.x) Tb[e] = S.T1[(size_t)p * BW * BW + e];
    __syncthreads();
    // W[c1][cz] = sum_i conj(V[i][c1]) Z[r0+i][cz]: warp per c1, lanes over the columns
    for (int c1 = wid; c1 < BW; c1 += nw) {
      if (lane < NC) {
        CX acc = czero<CX>();
        for (int i = c1; i < m; ++i) cfmac(acc, Vp[i * BW + c1], Z[(r0 + i) * NC + lane]);
        Wb[c1 * NC + lane] = acc;
      }
    }
    __syncthreads();
    // W <- T W (T upper triangular), in place by rows top-down per column
    if (tid < NC) {
      CX col[BW];
#pragma unroll
      for (int c1 = 0; c1 < BW; ++c1) col[c1] = Wb[c1 * NC + tid];
#pragma unroll
      for (int c1 = 0; c1 < BW; ++c1) {
        CX acc = czero<CX>();
#pragma unroll
        for (int k = 0; k < BW; ++k)
          if (k >= c1) cfma(acc, Tb[c1 * BW + k], col[k]);
        Wb[c1 * NC + tid] = acc;
      }
    }
    __syncthreads();
    for (int e = tid; e < m * NC; e += blockDim.x) {
      const int i = e / NC, cz = e % NC;
      CX acc = czero<CX>();
#pragma unroll
      for (int c1 = 0; c1 < BW; ++c1) cfma(acc, Vp[i * BW + c1], Wb[c1 * NC + cz]);
      Z[(r0 + i) * NC + cz] = csub(Z[(r0 + i) * NC + cz], acc);
    }
    __syncthreads();
  }
  CX* V = (CX*)P.V;
  for (int e = tid; e < n * NC; e += blockDim.x) {
    const int i = e / NC, c = e % NC;
    if (c < ncol) V[(int64_t)i * P.ldv + col0 + c] = Z[e];
  }
}

template <typename CX, int BW>
size_t stage1_smem(int n, int C) {
  const int rows_max = (n + C - 1) / C;
  return (size_t)(5 * BW * BW + BW) * sizeof(CX) + 32 * sizeof(typename cx_traits<CX>::R) +
         (size_t)(2 * n + rows_max) * BW * sizeof(CX);
}

template <typename CX, int BW>
size_t stage2_smem(int n) {
  return ((size_t)n * Band<CX, BW>::LD + 2 * NWARP2 * BW) * sizeof(CX);
}

template <typename CX, int BW>
int launch_two_stage_bw(HeevdProb* probs, int count, int maxn, cudaStream_t s) {
  const int C = 8;
  const size_t sm1 = stage1_smem<CX, BW>(maxn, C);
  auto k1 = band_reduce_kernel<CX, BW>;
  cudaError_t err = cudaFuncSetAttribute(k1, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm1);
  if (err != cudaSuccess) {
    agb_note_error(__FILE__, __LINE__, err);
    return AGB_ERR_CUDA;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(count * C, 1, 1);
  cfg.blockDim = dim3(512, 1, 1);
  cfg.dynamicSmemBytes = sm1;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = C;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  err = cudaLaunchKernelEx(&cfg, k1, (const HeevdProb*)probs, C);
  agb_note_launch();
  if (err != cudaSuccess) {
    agb_note_error(__FILE__, __LINE__, err);
    return AGB_ERR_CUDA;
  }
  const size_t sm2 = stage2_smem<CX, BW>(maxn);
  const cudaError_t oe = agb_smem_optin(band_to_tridiag_kernel<CX, BW>, sm2);
  if (oe != cudaSuccess) {
    agb_note_error(__FILE__, __LINE__, oe);
    return AGB_ERR_CUDA;
  }
  band_to_tridiag_kernel<CX, BW><<<count, NWARP2 * 32, sm2, s>>>(probs);
  AGB_CHECK_LAUNCH();
  return AGB_OK;
}

constexpr size_t kSmem2 = 220 * 1024;

template <typename CX, int BW>
size_t bt_smem(int n, int nc) {
  return ((size_t)n * (nc + BW) + BW * nc + BW * BW) * sizeof(CX);
}

template <typename CX, int BW, int NC>
int launch_bt_nc(const HeevdProb* probs, int count, int maxn, int maxell, cudaStream_t s) {
  const size_t sm = bt_smem<CX, BW>(maxn, NC);
  const cudaError_t oe = agb_smem_optin(bt_two_stage_kernel<CX, BW, NC>, sm);
  if (oe != cudaSuccess) {
    agb_note_error(__FILE__, __LINE__, oe);
    return AGB_ERR_CUDA;
  }
  dim3 grid((maxell + NC - 1) / NC, count);
  bt_two_stage_kernel<CX, BW, NC><<<grid, 512, sm, s>>>(probs);
  AGB_CHECK_LAUNCH();
  return AGB_OK;
}

// 32 eigenvector columns per CTA where they fit in shared memory, else 16 or 8
template <typename CX, int BW>
int launch_bt_two_stage_bw(const HeevdProb* probs, int count, int maxn, int maxell, cudaStream_t s) {
  if (bt_smem<CX, BW>(maxn, 32) <= kSmem2) return launch_bt_nc<CX, BW, 32>(probs, count, maxn, maxell, s);
  if (bt_smem<CX, BW>(maxn, 16) <= kSmem2) return launch_bt_nc<CX, BW, 16>(probs, count, maxn, maxell, s);
  return launch_bt_nc<CX, BW, 8>(probs, count, maxn, maxell, s);
}

}  // namespace

// Band width of the two-stage path for a batch whose largest matrix is maxn
// (0: the one-stage kernel).  The stage-1 panel and exchange buffers
// (2 n BW elements) and the stage-2 band (n (2 BW + 1) elements) must fit in
// shared memory.
int two_stage_bw(int esz, int maxn) {
  if (maxn < 64) return 0;
  for (int bw = 16; bw >= 8; bw /= 2) {
    const size_t s1 = (size_t)(2 * maxn + (maxn + 7) / 8) * bw * esz + (5 * bw * bw + bw) * (size_t)esz + 256;
    const size_t s2 = ((size_t)maxn * (2 * bw + 1) + 2 * NWARP2 * bw) * esz;
    const size_t s3 = ((size_t)maxn * (8 + bw) + bw * 8 + bw * bw) * esz;
    if (s1 <= kSmem2 && s2 <= kSmem2 && s3 <= kSmem2) return bw;
  }
  return 0;
}

template <typename CX>
int launch_two_stage(HeevdProb* probs, int count, int maxn, cudaStream_t s) {
  const int bw = two_stage_bw(sizeof(CX), maxn);
  if (bw == 16) return launch_two_stage_bw<CX, 16>(probs, count, maxn, s);
  if (bw == 8) return launch_two_stage_bw<CX, 8>(probs, count, maxn, s);
  return AGB_ERR_UNSUPPORTED;
}

template <typename CX>
int launch_bt_two_stage(const HeevdProb* probs, int count, int maxn, int maxell, cudaStream_t s) {
  const int bw = two_stage_bw(sizeof(CX), maxn);
  if (bw == 16) return launch_bt_two_stage_bw<CX, 16>(probs, count, maxn, maxell, s);
  if (bw == 8) return launch_bt_two_stage_bw<CX, 8>(probs, count, maxn, maxell, s);
  return AGB_ERR_UNSUPPORTED;
}

template int launch_two_stage<float2>(HeevdProb*, int, int, cudaStream_t);
template int launch_two_stage<double2>(HeevdProb*, int, int, cudaStream_t);
template int launch_bt_two_stage<float2>(const HeevdProb*, int, int, int, cudaStream_t);
template int launch_bt_two_stage<double2>(const HeevdProb*, int, int, int, cudaStream_t);
