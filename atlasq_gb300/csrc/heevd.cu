// Batched Hermitian eigensolver kernels (see heevd.cuh for the stage list).
#include <float.h>

#include "heevd.cuh"
#include "prof.cuh"

template <typename R> struct rlim;

// Reciprocal of an LU pivot, the pivot first floored at piv in magnitude (a
// zero pivot takes +piv).  The factors store reciprocals so that the back
// substitution's dependent chain is multiply-adds only.
template <typename R>
__device__ __forceinline__ R inv_pivot(R u, R piv) {
  if (fabs(u) < piv) u = copysign(piv, u == R(0) ? R(1) : u);
  return R(1) / u;
}
template <> struct rlim<float> {
  static AGB_HD float eps() { return FLT_EPSILON; }
  static AGB_HD float pivmin() { return 1e-30f; }
  static AGB_HD float huge() { return FLT_MAX; }
};
template <> struct rlim<double> {
  static AGB_HD double eps() { return DBL_EPSILON; }
  static AGB_HD double pivmin() { return 1e-290; }
  static AGB_HD double huge() { return DBL_MAX; }
};

void heevd_assign_scratch(HeevdProb& p, char* base, int esz) { heevd_assign_scratch_dev(p, base, esz); }

static int g_stages_mode = 1;
int tridiag_stages_mode() { return g_stages_mode; }
extern "C" int agb_set_tridiag_stages(int mode) {
  if (mode != 0 && mode != 1) return AGB_ERR_ARG;
  g_stages_mode = mode;
  return AGB_OK;
}

namespace {

// ------------------------------------------------------------------ stage 1
// Householder reflector for step j (zlarfg semantics): x = column j below the
// diagonal = conj(row j, cols > j).  Writes v into smem (v[j+1] = 1) and into
// row j of H (cols >= j+2); returns tau, beta via smem broadcast.
template <typename CX>
AGB_DEV void make_reflector(CX* H, int64_t ld, int n, int j, CX* v, typename cx_traits<CX>::R* red,
                            CX* bc, typename cx_traits<CX>::R* d, typename cx_traits<CX>::R* e,
                            CX* tau) {
  typedef typename cx_traits<CX>::R R;
  const int tid = threadIdx.x, nt = blockDim.x;
  CX* row = H + (int64_t)j * ld;
  R part = 0;
  for (int c = j + 2 + tid; c < n; c += nt) part += cabs2(row[c]);
  const R xnorm2 = block_sum(part, red);
  if (tid == 0) {
    const CX alpha = cconj(row[j + 1]);
    CX t = czero<CX>(), sc = czero<CX>();
    R beta;
    if (xnorm2 == R(0) && alpha.y == R(0)) {
      beta = alpha.x;
    } else {
      beta = -copysign(sqrt(alpha.x * alpha.x + alpha.y * alpha.y + xnorm2), alpha.x);
      t = mk<CX>((beta - alpha.x) / beta, -alpha.y / beta);
      sc = cinv(csub(alpha, mk<CX>(beta, 0)));
    }
    bc[0] = t;
    bc[1] = sc;
    e[j] = beta;
    tau[j] = t;
    d[j] = row[j].x;
  }
  __syncthreads();
  const CX sc = bc[1];
  for (int c = j + 2 + tid; c < n; c += nt) {
    const CX vc = cmul(cconj(row[c]), sc);
    v[c] = vc;
    row[c] = vc;
  }
  if (tid == 0) v[j + 1] = mk<CX>(1, 0);
  __syncthreads();
}

template <typename CX>
__global__ void __launch_bounds__(1024) tridiag_kernel(const HeevdProb* __restrict__ probs) {
  typedef typename cx_traits<CX>::R R;
  const HeevdProb P = probs[blockIdx.x];
  const int n = P.n;
  if (n <= 0) return;
  CX* H = (CX*)P.H;
  const int64_t ld = P.ldh;
  R* d = (R*)P.d;
  R* e = (R*)P.e;
  CX* tau = (CX*)P.tau;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  CX* va = (CX*)smem_raw;
  CX* vb = va + n;
  CX* w = vb + n;
  CX* pv = w + n;
  __shared__ R red[32];
  __shared__ CX bc[4];
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, wid = tid >> 5, nw = nt >> 5;

  // scale by the largest diagonal magnitude (Gram matrices: largest column norm)
  R mx = 0;
  for (int i = tid; i < n; i += nt) mx = fmax(mx, fabs(H[(int64_t)i * ld + i].x));
  {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if (lane == 0) red[wid] = mx;
    __syncthreads();
    if (tid == 0) {
      R m = 0;
      for (int i = 0; i < nw; ++i) m = fmax(m, red[i]);
      red[0] = m;
    }
    __syncthreads();
    mx = red[0];
    __syncthreads();
  }
  if (mx == R(0)) mx = R(1);
  if (tid == 0) *((R*)P.scale) = mx;
  const R inv = R(1) / mx;
  for (int64_t idx = tid; idx < (int64_t)n * n; idx += nt) {
    const int r = (int)(idx / n), c = (int)(idx % n);
    CX* a = H + (int64_t)r * ld + c;
    *a = cscale(*a, inv);
  }
  __syncthreads();
  if (n == 1) {
    if (tid == 0) {
      d[0] = H[0].x;
      e[0] = 0;
      tau[0] = czero<CX>();
    }
    return;
  }
  CX* v = va;
  CX* vn = vb;
  // reflector 0 and its matvec p = tau * H[1:,1:] v
  make_reflector(H, ld, n, 0, v, red, bc, d, e, tau);
  {
    const CX t0 = tau[0];
    for (int r = 1 + wid; r < n; r += nw) {
      const CX* row = H + (int64_t)r * ld;
      CX acc = czero<CX>();
      for (int c = 1 + lane; c < n; c += 32) cfma(acc, row[c], v[c]);
      acc = warp_csum(acc);
      if (lane == 0) pv[r] = cmul(t0, acc);
    }
  }
  __syncthreads();
  for (int j = 0; j <= n - 2; ++j) {
    const CX t = tau[j];
    const bool active = (t.x != R(0) || t.y != R(0));
    if (active) {
      // K = -1/2 tau (p^H v); w = p + K v   over r >= j+1
      CX part = czero<CX>();
      for (int r = j + 1 + tid; r < n; r += nt) cfmac(part, pv[r], v[r]);
      const R sr = block_sum(part.x, red);
      const R si = block_sum(part.y, red);
      const CX K = cscale(cmul(t, mk<CX>(sr, si)), R(-0.5));
      for (int r = j + 1 + tid; r < n; r += nt) w[r] = cadd(pv[r], cmul(K, v[r]));
      __syncthreads();
      // row j+1, cols >= j+1:  H -= v w^H + w v^H   (v[j+1] = 1)
      CX* row = H + (int64_t)(j + 1) * ld;
      const CX wr = w[j + 1];
      for (int c = j + 1 + tid; c < n; c += nt) {
        CX a = row[c];
        a = csub(a, cconj(w[c]));          // v[j+1] * conj(w[c])
        a = csub(a, cmul(wr, cconj(v[c])));
        row[c] = a;
      }
      __syncthreads();
    }
    CX tn = czero<CX>();
    if (j + 1 <= n - 2) {
      make_reflector(H, ld, n, j + 1, vn, red, bc, d, e, tau);
      tn = tau[j + 1];
    } else {
      if (tid == 0) {
        d[n - 1] = H[(int64_t)(n - 1) * ld + (n - 1)].x;
        e[n - 1] = 0;
      }
    }
    const bool next_active = (tn.x != R(0) || tn.y != R(0));
    // fused pass over rows r >= j+2: apply step-j update, accumulate next matvec
    if (active || next_active) {
      for (int r = j + 2 + wid; r < n; r += nw) {
        CX* row = H + (int64_t)r * ld;
        const CX vr = v[r], wr = w[r];
        CX acc = czero<CX>();
        for (int c = j + 2 + lane; c < n; c += 32) {
          CX a = row[c];
          if (active) {
            a = csub(a, cmul(vr, cconj(w[c])));
            a = csub(a, cmul(wr, cconj(v[c])));
            row[c] = a;
          }
          if (next_active) cfma(acc, a, vn[c]);
        }
        if (next_active) {
          acc = warp_csum(acc);
          if (lane == 0) pv[r] = cmul(tn, acc);
        }
      }
    }
    __syncthreads();
    CX* tmp = v;
    v = vn;
    vn = tmp;
  }
}

// ------------------------------------------------------------------ stage 2
// Number of eigenvalues of T below x (Sturm sequence of the LDL^T pivots).
// A pivot smaller than pm in magnitude is replaced by -pm BEFORE it is
// counted, so the count and the recurrence see the same sign (LAPACK dlaebz's
// order).  Replacing it only at the next step, after counting it as
// non-negative, loses one eigenvalue whenever a pivot cancels to exactly 0:
// in float32 that happened at x midway between two leading eigenvalues 1.6e-5
// apart, bisection then returned a value between them and inverse iteration
// produced two overlapping eigenvectors.
template <typename R>
AGB_DEV int sturm_count(const R* d, const R* e2, int n, R x) {
  const R pm = rlim<R>::pivmin();
  R q = d[0] - x;
  if (fabs(q) < pm) q = -pm;
  int cnt = q < R(0);
  for (int i = 1; i < n; ++i) {
    q = d[i] - x - e2[i - 1] / q;
    if (fabs(q) < pm) q = -pm;
    cnt += q < R(0);
  }
  return cnt;
}

template <typename R>
__global__ void __launch_bounds__(256) bisect_kernel(const HeevdProb* __restrict__ probs) {
  const HeevdProb P = probs[blockIdx.y];
  const int n = P.n, ell = P.ell;
  if (blockIdx.x * 8 >= ell) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  R* d = (R*)smem_raw;
  R* e2 = d + n;
  __shared__ R glim[2];
  const R* dg = (const R*)P.d;
  const R* eg = (const R*)P.e;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    d[i] = dg[i];
    e2[i] = (i < n - 1) ? eg[i] * eg[i] : R(0);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    R gl = d[0], gu = d[0];
    for (int i = 0; i < n; ++i) {
      const R r = (i > 0 ? fabs(eg[i - 1]) : R(0)) + (i < n - 1 ? fabs(eg[i]) : R(0));
      gl = fmin(gl, d[i] - r);
      gu = fmax(gu, d[i] + r);
    }
    const R span = fmax(fabs(gl), fabs(gu));
    glim[0] = gl - R(4) * rlim<R>::eps() * span - rlim<R>::pivmin();
    glim[1] = gu + R(4) * rlim<R>::eps() * span + rlim<R>::pivmin();
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int t = blockIdx.x * 8 + wid;
  if (t >= ell) return;
  const int idx = n - 1 - t;  // ascending index of the t-th largest eigenvalue
  R lo = glim[0], hi = glim[1];
  const R tol = R(2) * rlim<R>::eps() * fmax(fabs(lo), fabs(hi));
  for (int it = 0; it < 64 && hi - lo > tol; ++it) {
    const R x = lo + (hi - lo) * R(lane + 1) / R(33);
    const int c = sturm_count(d, e2, n, x);
    const unsigned m = __ballot_sync(0xffffffffu, c > idx);
    const int f = m ? __ffs(m) - 1 : 32;
    const R nhi = (f < 32) ? __shfl_sync(0xffffffffu, x, f) : hi;
    const R nlo = (f > 0) ? __shfl_sync(0xffffffffu, x, (f > 0 ? f - 1 : 0)) : lo;
    if (nhi == hi && nlo == lo) break;
    lo = nlo;
    hi = nhi;
  }
  if (lane == 0) ((R*)P.lam)[t] = R(0.5) * (lo + hi);
}

// ------------------------------------------------------------------ stage 3
template <typename R> AGB_DEV R cluster_tol(const R* lam, int ell, double tolrel);
template <typename R> AGB_DEV bool in_cluster(const R* lam, int ell, int t, R tol);

template <typename R>
__global__ void __launch_bounds__(128) invit_kernel(const HeevdProb* __restrict__ probs) {
  const HeevdProb P = probs[blockIdx.y];
  const int n = P.n, ell = P.ell, nv = P.nvec;
  if (blockIdx.x * 128 >= nv) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  R* d = (R*)smem_raw;
  R* e = d + n;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    d[i] = ((const R*)P.d)[i];
    e[i] = (i < n - 1) ? ((const R*)P.e)[i] : R(0);
  }
  __syncthreads();
  const int t = blockIdx.x * 128 + threadIdx.x;
  if (t >= nv || P.skip_vectors) return;
  if (in_cluster((const R*)P.lam, nv, t, cluster_tol((const R*)P.lam, ell, P.ctol))) return;
  const R lam = ((const R*)P.lam)[t];
  R tnorm = 0;
  for (int i = 0; i < n; ++i) tnorm = fmax(tnorm, fabs(d[i]) + fabs(e[i]) + (i ? fabs(e[i - 1]) : R(0)));
  const R piv = rlim<R>::eps() * fmax(tnorm, rlim<R>::pivmin());
  R* lu = (R*)P.lu;
  const int64_t L = ell;
  R* U0 = lu;
  R* U1 = lu + (int64_t)n * L;
  R* U2 = lu + 2 * (int64_t)n * L;
  R* Lm = lu + 3 * (int64_t)n * L;
  R* Pv = lu + 4 * (int64_t)n * L;
  // LU with partial pivoting of T - lam I (rows carry up to two superdiagonals)
  R u0 = d[0] - lam, u1 = (n > 1) ? e[0] : R(0), u2 = 0;
  for (int i = 0; i < n - 1; ++i) {
    const R sub = e[i], nd = d[i + 1] - lam, ns = (i + 1 < n - 1) ? e[i + 1] : R(0);
    R a0, a1, a2, m, pv;
    if (fabs(u0) >= fabs(sub)) {
      if (u0 == R(0)) u0 = piv;
      m = sub / u0;
      a0 = u0; a1 = u1; a2 = u2;
      u0 = nd - m * u1;
      u1 = ns - m * u2;
      pv = 0;
    } else {
      m = u0 / sub;
      a0 = sub; a1 = nd; a2 = ns;
      const R nu0 = u1 - m * nd, nu1 = u2 - m * ns;
      u0 = nu0;
      u1 = nu1;
      pv = 1;
    }
    u2 = 0;
    U0[i * L + t] = inv_pivot(a0, piv);
    U1[i * L + t] = a1;
    U2[i * L + t] = a2;
    Lm[i * L + t] = m;
    Pv[i * L + t] = pv;
  }
  U0[(int64_t)(n - 1) * L + t] = inv_pivot(u0, piv);
  U1[(int64_t)(n - 1) * L + t] = 0;
  U2[(int64_t)(n - 1) * L + t] = 0;
  R* Y = (R*)P.Y;
  // random start
  R nrm = 0;
  for (int i = 0; i < n; ++i) {
    const R b = (R)philox_normal(P.seed, (uint64_t)t * (uint64_t)n + i, 0x11u);
    Y[i * L + t] = b;
    nrm += b * b;
  }
  // three inverse-iteration solves from a random start: the shift is the
  // bisection eigenvalue (error ~eps*||T||), so each solve amplifies the wanted
  // component by ~gap/(eps*||T||) over its neighbours; with two, a start that
  // happens to be nearly orthogonal to the wanted vector leaves it
  // unconverged (measured: a 4e-4 fidelity loss after 150 gates of the 40-qubit
  // brickwork for one seed sequence, before any truncation)
  for (int it = 0; it < 3; ++it) {
    const R s = R(1) / sqrt(fmax(nrm, rlim<R>::pivmin()));
    // Forward (apply P and L) and backward substitution.  The factor and
    // iterate loads do not depend on the recurrence, so each chunk of IB steps
    // loads its operands into registers first and then runs the serial chain:
    // IB loads in flight instead of one dependent load per step.  Within a
    // chunk every load of Y precedes the store to the same element.
    constexpr int IB = 16;
    R bi = Y[t] * s;
    for (int i0 = 0; i0 < n - 1; i0 += IB) {
      R yb[IB], pv[IB], lm[IB];
#pragma unroll
      for (int k = 0; k < IB; ++k) {
        const int i = i0 + k;
        if (i < n - 1) {
          yb[k] = Y[(int64_t)(i + 1) * L + t];
          pv[k] = Pv[(int64_t)i * L + t];
          lm[k] = Lm[(int64_t)i * L + t];
        }
      }
#pragma unroll
      for (int k = 0; k < IB; ++k) {
        const int i = i0 + k;
        if (i < n - 1) {
          R bn = yb[k] * s;
          if (pv[k] != R(0)) {
            const R tmp = bi;
            bi = bn;
            bn = tmp;
          }
          Y[(int64_t)i * L + t] = bi;
          bi = bn - lm[k] * bi;
        }
      }
    }
    Y[(int64_t)(n - 1) * L + t] = bi;
    R x1 = 0, x2 = 0;
    nrm = 0;
    for (int i0 = n - 1; i0 >= 0; i0 -= IB) {
      R u0[IB], u1[IB], u2[IB], yb[IB];
#pragma unroll
      for (int k = 0; k < IB; ++k) {
        const int i = i0 - k;
        if (i >= 0) {
          u0[k] = U0[(int64_t)i * L + t];
          u1[k] = U1[(int64_t)i * L + t];
          u2[k] = U2[(int64_t)i * L + t];
          yb[k] = Y[(int64_t)i * L + t];
        }
      }
#pragma unroll
      for (int k = 0; k < IB; ++k) {
        const int i = i0 - k;
        if (i >= 0) {
          const R x = (yb[k] - u1[k] * x1 - u2[k] * x2) * u0[k];  // u0: reciprocal pivot
          Y[(int64_t)i * L + t] = x;
          nrm += x * x;
          x2 = x1;
          x1 = x;
        }
      }
    }
    if (!(nrm < R(1e300)) || !(nrm > R(0))) {  // overflow / breakdown: restart from a unit vector
      for (int i = 0; i < n; ++i) Y[(int64_t)i * L + t] = (i == (t % n)) ? R(1) : R(0);
      nrm = 1;
    }
  }
  const R s = R(1) / sqrt(fmax(nrm, rlim<R>::pivmin()));
  for (int i = 0; i < n; ++i) Y[i * L + t] *= s;
}

// ------------------------------------------------------------------ stage 4
// Eigenvalue clusters (consecutive eigenvalues closer than tolrel * max|lambda|)
// are solved with LAPACK stein's ingredients, its members in parallel: each
// member shifted by its own eigenvalue (member_shift), one LU per member, and
// two rounds of [one inverse-iteration solve
// of every member from its own random start; Gram-Schmidt (classical, twice)
// over the cluster in member order].  This keeps the iterates from collapsing
// onto one direction when T splits (exactly degenerate eigenvalues) or when
// the cluster sits at the noise floor of the Gram matrix.  One CTA per cluster.
template <typename R>
AGB_DEV R cluster_tol(const R* lam, int ell, double tolrel) {
  const R scale = fmax(fabs(lam[0]), fabs(lam[ell - 1]));
  return (R)tolrel * fmax(scale, rlim<R>::pivmin());
}

template <typename R>
AGB_DEV bool in_cluster(const R* lam, int ell, int t, R tol) {
  const bool left = (t > 0) && (lam[t - 1] - lam[t]) <= tol;
  const bool right = (t + 1 < ell) && (lam[t] - lam[t + 1]) <= tol;
  return left || right;
}

// Shift of cluster member j: its own eigenvalue.  LAPACK's stein walks the
// shifts of near-equal members apart by 10 eps |lambda| each, which is
// harmless in double precision but in float32 moves the last members of a
// cluster by ~1e-6 |lambda| per member, toward the first eigenvalue below
// the cluster.  Measured on 64-qubit HEA gates (chi 512): eight members within
// 6.6e-6 lambda_0 of each other and the next eigenvalue 1.2e-5 below; the
// walked shift of the eighth member amplified that outside eigenvector about
// a sixth as much as its own, and after the Gram-Schmidt pass had removed the
// directions of the first seven members, what remained was 92% the outside
// eigenvector.  With unwalked shifts the outside component is suppressed by
// (bisection error / gap) per solve; members with equal shifts still get
// independent iterates from their own random starts, which Gram-Schmidt
// separates.  The shift is also kept above the midpoint to the eigenvalue
// below the cluster.
template <typename R>
AGB_DEV R member_shift(const R* lam, int ell, int j, int t1) {
  const R sh = lam[j];
  if (t1 >= ell) return sh;
  return fmax(sh, R(0.5) * (lam[t1 - 1] + lam[t1]));
}

// LU with partial pivoting of T - lam I into the interleaved factor arrays
// (column t of each), as in invit_kernel.
template <typename R>
AGB_DEV void tri_lu(const R* d, const R* e, int n, R lam, R piv, R* U0, R* U1, R* U2, R* Lm, R* Pv,
                    int64_t L, int t) {
  R u0 = d[0] - lam, u1 = (n > 1) ? e[0] : R(0), u2 = 0;
  for (int i = 0; i < n - 1; ++i) {
    const R sub = e[i], nd = d[i + 1] - lam, ns = (i + 1 < n - 1) ? e[i + 1] : R(0);
    R a0, a1, a2, m, pv;
    if (fabs(u0) >= fabs(sub)) {
      if (u0 == R(0)) u0 = piv;
      m = sub / u0;
      a0 = u0; a1 = u1; a2 = u2;
      u0 = nd - m * u1;
      u1 = ns - m * u2;
      pv = 0;
    } else {
      m = u0 / sub;
      a0 = sub; a1 = nd; a2 = ns;
      const R nu0 = u1 - m * nd, nu1 = u2 - m * ns;
      u0 = nu0;
      u1 = nu1;
      pv = 1;
    }
    u2 = 0;
    U0[i * L + t] = inv_pivot(a0, piv);
    U1[i * L + t] = a1;
    U2[i * L + t] = a2;
    Lm[i * L + t] = m;
    Pv[i * L + t] = pv;
  }
  U0[(int64_t)(n - 1) * L + t] = inv_pivot(u0, piv);
  U1[(int64_t)(n - 1) * L + t] = 0;
  U2[(int64_t)(n - 1) * L + t] = 0;
}

// y <- (T - lam I)^{-1} (s * y) for column t of Y (stride L) with the stored
// factors of column t; returns ||y||^2.  Factor and iterate loads do not depend
// on the recurrence, so each chunk of IB steps loads them into registers first
// (IB loads in flight instead of one dependent load per step).
template <typename R>
AGB_DEV R tri_solve_pf(R* Y, int n, const R* U0, const R* U1, const R* U2, const R* Lm, const R* Pv, int64_t L,
                       int t, R piv, R s) {
  constexpr int IB = 16;
  R bi = Y[t] * s;
  for (int i0 = 0; i0 < n - 1; i0 += IB) {
    R yb[IB], pv[IB], lm[IB];
#pragma unroll
    for (int k = 0; k < IB; ++k) {
      const int i = i0 + k;
      if (i < n - 1) {
        yb[k] = Y[(int64_t)(i + 1) * L + t];
        pv[k] = Pv[(int64_t)i * L + t];
        lm[k] = Lm[(int64_t)i * L + t];
      }
    }
#pragma unroll
    for (int k = 0; k < IB; ++k) {
      const int i = i0 + k;
      if (i < n - 1) {
        R bn = yb[k] * s;
        if (pv[k] != R(0)) {
          const R tmp = bi;
          bi = bn;
          bn = tmp;
        }
        Y[(int64_t)i * L + t] = bi;
        bi = bn - lm[k] * bi;
      }
    }
  }
  Y[(int64_t)(n - 1) * L + t] = bi;
  R x1 = 0, x2 = 0, nrm = 0;
  for (int i0 = n - 1; i0 >= 0; i0 -= IB) {
    R u0[IB], u1[IB], u2[IB], yb[IB];
#pragma unroll
    for (int k = 0; k < IB; ++k) {
      const int i = i0 - k;
      if (i >= 0) {
        u0[k] = U0[(int64_t)i * L + t];
        u1[k] = U1[(int64_t)i * L + t];
        u2[k] = U2[(int64_t)i * L + t];
        yb[k] = Y[(int64_t)i * L + t];
      }
    }
#pragma unroll
    for (int k = 0; k < IB; ++k) {
      const int i = i0 - k;
      if (i >= 0) {
        const R x = (yb[k] - u1[k] * x1 - u2[k] * x2) * u0[k];  // u0: reciprocal pivot
        Y[(int64_t)i * L + t] = x;
        nrm += x * x;
        x2 = x1;
        x1 = x;
      }
    }
  }
  return nrm;
}

// Inverse iteration, complex64 path (float tridiagonal), for n <= 1024: the
// same LU, start vectors and three solves as invit_kernel, with the iterate of
// each thread's eigenvector kept in shared memory and the LU factors streamed
// from L2 through a per-thread ring of cp.async copies issued AHEAD chunks of
// CH steps before use.  The solves' recurrences are chains of multiply-adds
// (reciprocal pivots), so with the operands already in shared memory a step
// costs a few cycles instead of an L2 round trip every IB steps.  Each thread
// reads only its own ring entries and its own iterate column: no block-level
// synchronisation after the tridiagonal is staged.  TB threads per CTA.
__device__ __forceinline__ void cp_async4(float* dst, const float* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"((uint32_t)__cvta_generic_to_shared(dst)), "l"(src)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

constexpr int kInvCH = 16, kInvNCH = 6;  // steps per chunk, chunks in the ring (5 in flight)

size_t invit_async_smem(int n, int tb) {
  return ((size_t)2 * n + (size_t)n * tb + (size_t)3 * kInvNCH * kInvCH * tb) * sizeof(float);
}

template <int TB>
__global__ void __launch_bounds__(TB) invit_async_kernel(const HeevdProb* __restrict__ probs) {
  constexpr int CH = kInvCH, NCH = kInvNCH, RS = NCH * CH;  // ring steps per array
  typedef float R;
  const HeevdProb P = probs[blockIdx.y];
  const int n = P.n, ell = P.ell, nv = P.nvec;
  if (blockIdx.x * TB >= nv || P.skip_vectors) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  R* d = (R*)smem_raw;            // [n]
  R* e = d + n;                   // [n]
  R* ys = e + n;                  // [n][TB] iterate column of each thread
  R* ring = ys + (size_t)n * TB;  // [3][RS][TB] streamed factors
  for (int i = threadIdx.x; i < n; i += TB) {
    d[i] = ((const R*)P.d)[i];
    e[i] = (i < n - 1) ? ((const R*)P.e)[i] : R(0);
  }
  __syncthreads();  // the last block-level barrier: threads may leave from here on
  const int tid = threadIdx.x, t = blockIdx.x * TB + tid;
  if (t >= nv) return;
  if (in_cluster((const R*)P.lam, nv, t, cluster_tol((const R*)P.lam, ell, P.ctol))) return;
  const R lam = ((const R*)P.lam)[t];
  R tnorm = 0;
  for (int i = 0; i < n; ++i) tnorm = fmax(tnorm, fabs(d[i]) + fabs(e[i]) + (i ? fabs(e[i - 1]) : R(0)));
  const R piv = rlim<R>::eps() * fmax(tnorm, rlim<R>::pivmin());
  R* lu = (R*)P.lu;
  const int64_t L = ell;
  R* U0 = lu;
  R* U1 = lu + (int64_t)n * L;
  R* U2 = lu + 2 * (int64_t)n * L;
  R* Lm = lu + 3 * (int64_t)n * L;
  R* Pv = lu + 4 * (int64_t)n * L;
  tri_lu(d, e, n, lam, piv, U0, U1, U2, Lm, Pv, L, t);
  __threadfence_block();  // the factor stores precede the copies that read them back
  // start vector: uniform in [-1, 1), four entries per Philox call (a Gaussian
  // start costs a Philox call plus Box-Muller per entry, half of this kernel's
  // instructions; inverse iteration only needs a start with a component along
  // the wanted vector)
  R nrm = 0;
  const uint64_t per = (uint64_t)((n + 3) / 4);
  for (int i0 = 0; i0 < n; i0 += 4) {
    const uint64_t idx = (uint64_t)t * per + (uint64_t)(i0 >> 2);
    const philox_out o = philox4x32_10((uint32_t)idx, (uint32_t)(idx >> 32), 0x11u, 0x5EEDu, (uint32_t)P.seed,
                                       (uint32_t)(P.seed >> 32));
    const uint32_t w[4] = {o.x, o.y, o.z, o.w};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int i = i0 + k;
      if (i < n) {
        const R b = (R)(int32_t)w[k] * R(4.656612873077393e-10);  // 2^-31
        ys[i * TB + tid] = b;
        nrm += b * b;
      }
    }
  }
  auto rg = [&](int a, int step) -> R* { return ring + ((size_t)a * RS + step % RS) * TB + tid; };
  const int nf = n - 1;  // forward steps i = 0 .. n-2 (operands Pv[i], Lm[i])
  auto issue_f = [&](int c) {
    for (int k = 0; k < CH; ++k) {
      const int i = c * CH + k;
      if (i < nf) {
        cp_async4(rg(0, i), Pv + (int64_t)i * L + t);
        cp_async4(rg(1, i), Lm + (int64_t)i * L + t);
      }
    }
    cp_async_commit();
  };
  // backward steps j = 0 .. n-1 handle row i = n-1-j (operands U0, U1, U2 of row i)
  auto issue_b = [&](int c) {
    for (int k = 0; k < CH; ++k) {
      const int j = c * CH + k;
      if (j < n) {
        const int i = n - 1 - j;
        cp_async4(rg(0, j), U0 + (int64_t)i * L + t);
        cp_async4(rg(1, j), U1 + (int64_t)i * L + t);
        cp_async4(rg(2, j), U2 + (int64_t)i * L + t);
      }
    }
    cp_async_commit();
  };
  const int cf = (nf + CH - 1) / CH, cb = (n + CH - 1) / CH;
  for (int it = 0; it < 3; ++it) {
    const R s = R(1) / sqrt(fmax(nrm, rlim<R>::pivmin()));
    // forward: apply P and L
    for (int c = 0; c < NCH - 1; ++c) issue_f(c);
    R bi = ys[tid] * s;
    for (int c = 0; c < cf; ++c) {
      issue_f(c + NCH - 1);  // an empty group past the end keeps the count uniform
      cp_async_wait<NCH - 1>();  // chunk c has landed
#pragma unroll 4
      for (int k = 0; k < CH; ++k) {
        const int i = c * CH + k;
        if (i < nf) {
          R bn = ys[(i + 1) * TB + tid] * s;
          if (*rg(0, i) != R(0)) {
            const R tmp = bi;
            bi = bn;
            bn = tmp;
          }
          ys[i * TB + tid] = bi;
          bi = bn - *rg(1, i) * bi;
        }
      }
    }
    ys[(n - 1) * TB + tid] = bi;
    cp_async_wait<0>();  // no copy in flight into the ring before it is reused
    // backward substitution with the reciprocal pivots
    for (int c = 0; c < NCH - 1; ++c) issue_b(c);
    R x1 = 0, x2 = 0;
    nrm = 0;
    for (int c = 0; c < cb; ++c) {
      issue_b(c + NCH - 1);
      cp_async_wait<NCH - 1>();
#pragma unroll 4
      for (int k = 0; k < CH; ++k) {
        const int j = c * CH + k;
        if (j < n) {
          const int i = n - 1 - j;
          const R x = (ys[i * TB + tid] - *rg(1, j) * x1 - *rg(2, j) * x2) * *rg(0, j);
          ys[i * TB + tid] = x;
          nrm += x * x;
          x2 = x1;
          x1 = x;
        }
      }
    }
    cp_async_wait<0>();
    if (!(nrm < R(1e300)) || !(nrm > R(0))) {  // overflow / breakdown: restart from a unit vector
      for (int i = 0; i < n; ++i) ys[i * TB + tid] = (i == (t % n)) ? R(1) : R(0);
      nrm = 1;
    }
  }
  const R sc = R(1) / sqrt(fmax(nrm, rlim<R>::pivmin()));
  R* Y = (R*)P.Y;
  for (int i = 0; i < n; ++i) Y[(int64_t)i * L + t] = ys[i * TB + tid] * sc;
}

// CGS2 of column jj of the staged cluster block Z (n x c, row-major in shared
// memory) against its columns [0, jj), then normalisation (block-wide).
template <typename R>
AGB_DEV void cgs2_block_smem(R* Z, int n, int c, int jj, R* coef, R* red, R* part) {
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, wid = tid >> 5, nw = nt >> 5;
  for (int pass = 0; pass < 2 && jj > 0; ++pass) {
    for (int c0 = 0; c0 < jj; c0 += 32) {
      const int i = c0 + lane;
      R a = 0;
      if (i < jj)
        for (int r = wid; r < n; r += nw) a += Z[(int64_t)r * c + i] * Z[(int64_t)r * c + jj];
      part[wid * 32 + lane] = a;
      __syncthreads();
      if (wid == 0 && i < jj) {
        R sum = 0;
        for (int w = 0; w < nw; ++w) sum += part[w * 32 + lane];
        coef[i] = sum;
      }
      __syncthreads();
    }
    for (int r = wid; r < n; r += nw) {
      R* row = Z + (int64_t)r * c;
      R acc = 0;
      for (int i = lane; i < jj; i += 32) acc += coef[i] * row[i];
      acc = warp_sum(acc);
      if (lane == 0) row[jj] -= acc;
    }
    __syncthreads();
  }
  R psum = 0;
  for (int r = tid; r < n; r += nt) psum += Z[(int64_t)r * c + jj] * Z[(int64_t)r * c + jj];
  const R nrm = block_sum(psum, red);
  const R sc = R(1) / sqrt(fmax(nrm, rlim<R>::pivmin()));
  for (int r = tid; r < n; r += nt) Z[(int64_t)r * c + jj] *= sc;
  __syncthreads();
}

// CGS2 of the working column y (shared memory) against columns [t0, j) of Y
// and normalisation (block-wide).  Dot products: tiles of 32 columns, lanes
// over the columns (coalesced rows of Y), warps over row groups, partial sums
// combined in shared memory; update: one warp per row, lanes over the columns.
template <typename R>
AGB_DEV void cgs2_normalize(R* y, const R* Y, int n, int64_t L, int t0, int j, R* coef, R* red, R* part) {
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, wid = tid >> 5, nw = nt >> 5;
  const int cols = j - t0;
  for (int pass = 0; pass < 2 && cols > 0; ++pass) {
    for (int c0 = 0; c0 < cols; c0 += 32) {
      const int c = c0 + lane;
      R a0 = 0, a1 = 0;
      if (c < cols) {
        const R* col = Y + t0 + c;
        int r = wid;
        for (; r + nw < n; r += 2 * nw) {
          a0 += col[(int64_t)r * L] * y[r];
          a1 += col[(int64_t)(r + nw) * L] * y[r + nw];
        }
        if (r < n) a0 += col[(int64_t)r * L] * y[r];
      }
      part[wid * 32 + lane] = a0 + a1;
      __syncthreads();
      if (wid == 0 && c < cols) {
        R sum = 0;
        for (int w = 0; w < nw; ++w) sum += part[w * 32 + lane];
        coef[c] = sum;
      }
      __syncthreads();
    }
    for (int r = wid; r < n; r += nw) {
      const R* row = Y + (int64_t)r * L + t0;
      R acc = 0;
      for (int c = lane; c < cols; c += 32) acc += coef[c] * row[c];
      acc = warp_sum(acc);
      if (lane == 0) y[r] -= acc;
    }
    __syncthreads();
  }
  R psum = 0;
  for (int r = tid; r < n; r += nt) psum += y[r] * y[r];
  const R nrm = block_sum(psum, red);
  const R sc = R(1) / sqrt(fmax(nrm, rlim<R>::pivmin()));
  for (int r = tid; r < n; r += nt) y[r] *= sc;
  __syncthreads();
}

// Clusters of the leading nvec eigenvalues (consecutive gaps <= tol), once per
// problem: P.M (the polish scratch, free until the polish) receives the count
// and the (t0, t1) pairs.
template <typename R>
__global__ void cluster_list_kernel(const HeevdProb* __restrict__ probs, int count) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= count) return;
  const HeevdProb P = probs[b];
  int* clist = (int*)P.M;
  const int ell = P.ell, nv = P.nvec;
  if (nv < 2 || P.skip_vectors) {
    clist[0] = 0;
    return;
  }
  const R* lam = (const R*)P.lam;
  const R tol = cluster_tol(lam, ell, P.ctol);
  int found = 0, s = 0;
  for (int t = 1; t <= nv; ++t) {
    if (t == nv || (lam[t - 1] - lam[t]) > tol) {
      if (t - s > 1) {
        clist[1 + 2 * found] = s;
        clist[2 + 2 * found] = t;
        ++found;
      }
      s = t;
    }
  }
  clist[0] = found;
}

template <typename R>
__global__ void __launch_bounds__(256) cluster_invit_kernel(const HeevdProb* __restrict__ probs, int zcap) {
  const HeevdProb P = probs[blockIdx.y];
  const int n = P.n, ell = P.ell, nv = P.nvec;
  if (nv < 2 || P.skip_vectors) return;
  // this CTA's cluster from the list cluster_list_kernel left in P.M
  // (count, then (t0, t1) pairs): CTAs beyond the count exit at once
  const int* clist = (const int*)P.M;
  if ((int)blockIdx.x >= clist[0]) return;
  const int t0 = clist[1 + 2 * blockIdx.x], t1 = clist[2 + 2 * blockIdx.x];
  extern __shared__ __align__(16) unsigned char smem_raw[];
  R* d = (R*)smem_raw;   // [n]
  R* e = d + n;          // [n]
  R* coef = e + n;       // [ell]
  R* f = coef + ell;     // [5n] LU factors of the current member (U0,U1,U2,L,P)
  R* ycol = f + 5 * n;   // [n]  working column of the current member
  R* Zs = ycol + n;      // [n * zcap] staged cluster block (parallel path)
  __shared__ R red[32];
  __shared__ R part[256];
  __shared__ R ctile[32 * 32];  // blocked Gram-Schmidt coefficients (32 earlier members x block)
  __shared__ R s_shift, s_nrm;
  const R* lamg = (const R*)P.lam;
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int i = tid; i < n; i += nt) {
    d[i] = ((const R*)P.d)[i];
    e[i] = (i < n - 1) ? ((const R*)P.e)[i] : R(0);
  }
  __syncthreads();
  R tnorm = 0;
  for (int i = tid; i < n; i += nt) tnorm = fmax(tnorm, fabs(d[i]) + fabs(e[i]) + (i ? fabs(e[i - 1]) : R(0)));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) tnorm = fmax(tnorm, __shfl_xor_sync(0xffffffffu, tnorm, o));
  if ((tid & 31) == 0) red[tid >> 5] = tnorm;
  __syncthreads();
  tnorm = 0;
  for (int w = 0; w < (nt >> 5); ++w) tnorm = fmax(tnorm, red[w]);
  __syncthreads();
  const R piv = rlim<R>::eps() * fmax(tnorm, rlim<R>::pivmin());
  const int64_t L = ell;
  R* Y = (R*)P.Y;
  const int c = t1 - t0;
  if (c >= 2) {
    // Members in parallel (LAPACK stein's iteration with the solves of all
    // members at once): each member's own eigenvalue as its shift; one LU per
    // member (global, column j); two rounds of [solve every member;
    // Gram-Schmidt in member order].
    R* shs = f;  // [c] shifts (c <= ell <= 5n)
    if (tid == 0) {
      for (int j = t0; j < t1; ++j) shs[j - t0] = member_shift(lamg, ell, j, t1);
    }
    __syncthreads();
    R* lu = (R*)P.lu;
    R* U0 = lu;
    R* U1 = lu + (int64_t)n * L;
    R* U2 = lu + 2 * (int64_t)n * L;
    R* Lm = lu + 3 * (int64_t)n * L;
    R* Pv = lu + 4 * (int64_t)n * L;
    for (int j = t0 + tid; j < t1; j += nt) tri_lu(d, e, n, shs[j - t0], piv, U0, U1, U2, Lm, Pv, L, j);
    for (int64_t idx = tid; idx < (int64_t)n * c; idx += nt) {
      const int r = (int)(idx / c), j = t0 + (int)(idx % c);
      Y[(int64_t)r * L + j] = (R)philox_normal(P.seed, (uint64_t)j * (uint64_t)n + r, 0x11u);
    }
    __syncthreads();
    const bool staged = c <= zcap;
    for (int it = 0; it < 2; ++it) {
      for (int j = t0 + tid; j < t1; j += nt) {
        const R nrm = tri_solve_pf(Y, n, U0, U1, U2, Lm, Pv, L, j, piv, R(1));
        if (!(nrm < R(1e300)) || !(nrm > R(0)))  // overflow / breakdown: restart from a new random vector
          for (int r = 0; r < n; ++r)
            Y[(int64_t)r * L + j] = (R)philox_normal(P.seed ^ 0xABCDEFull, (uint64_t)(j + it + 1) * (uint64_t)n + r, 0x13u);
        else {
          const R sc = R(1) / sqrt(nrm);  // keep magnitudes O(1) for the float Gram-Schmidt
          for (int r = 0; r < n; ++r) Y[(int64_t)r * L + j] *= sc;
        }
      }
      __syncthreads();
      if (staged) {
        for (int64_t idx = tid; idx < (int64_t)n * c; idx += nt) {
          const int r = (int)(idx / c), jj = (int)(idx % c);
          Zs[idx] = Y[(int64_t)r * L + t0 + jj];
        }
        __syncthreads();
        for (int jj = 0; jj < c; ++jj) cgs2_block_smem(Zs, n, c, jj, coef, red, part);
        for (int64_t idx = tid; idx < (int64_t)n * c; idx += nt) {
          const int r = (int)(idx / c), jj = (int)(idx % c);
          Y[(int64_t)r * L + t0 + jj] = Zs[idx];
        }
        __syncthreads();
      } else {
        // Blocked Gram-Schmidt for clusters wider than the staging area: blocks of
        // B members are staged in shared memory, projected off every earlier member
        // (tiles of 32 columns read from Y, twice), then orthonormalised inside the block.
        const int B = zcap < 32 ? zcap : 32;  // ctile holds 32 x 32 coefficients
        const int lane = tid & 31, wid = tid >> 5, nw = nt >> 5;
        for (int b0 = t0; b0 < t1; b0 += B) {
          const int bw = min(B, t1 - b0);
          for (int64_t idx = tid; idx < (int64_t)n * bw; idx += nt) {
            const int r = (int)(idx / bw), jj = (int)(idx % bw);
            Zs[idx] = Y[(int64_t)r * L + b0 + jj];
          }
          __syncthreads();
          for (int pass = 0; pass < 2 && b0 > t0; ++pass) {
            for (int c0 = t0; c0 < b0; c0 += 32) {
              const int tw = min(32, b0 - c0);
              // coefficients ctile[i][jj] = Y[:, c0+i] . Z[:, jj]   (lanes over i: coalesced rows of Y)
              for (int jj0 = 0; jj0 < bw; jj0 += 4 * nw) {
                R acc[4] = {0, 0, 0, 0};
                if (lane < tw) {
                  for (int r = 0; r < n; ++r) {
                    const R yv = Y[(int64_t)r * L + c0 + lane];
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                      const int jj = jj0 + wid + u * nw;
                      if (jj < bw) acc[u] += yv * Zs[(int64_t)r * bw + jj];
                    }
                  }
                }
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                  const int jj = jj0 + wid + u * nw;
                  if (jj < bw && lane < tw) ctile[lane * 32 + jj] = acc[u];
                }
              }
              __syncthreads();
              // Z[r][jj] -= sum_i Y[r, c0+i] ctile[i][jj]   (thread per row)
              for (int r = tid; r < n; r += nt) {
                R yr[32];
#pragma unroll
                for (int i = 0; i < 32; ++i) yr[i] = (i < tw) ? Y[(int64_t)r * L + c0 + i] : R(0);
                for (int jj = 0; jj < bw; ++jj) {
                  R a = 0;
#pragma unroll
                  for (int i = 0; i < 32; ++i)
                    if (i < tw) a += yr[i] * ctile[i * 32 + jj];  // rows >= tw were not written
                  Zs[(int64_t)r * bw + jj] -= a;
                }
              }
              __syncthreads();
            }
          }
          for (int jj = 0; jj < bw; ++jj) cgs2_block_smem(Zs, n, bw, jj, coef, red, part);
          for (int64_t idx = tid; idx < (int64_t)n * bw; idx += nt) {
            const int r = (int)(idx / bw), jj = (int)(idx % bw);
            Y[(int64_t)r * L + b0 + jj] = Zs[idx];
          }
          __syncthreads();
        }
      }
    }
    return;
  }
}

// ------------------------------------------------------------------ stage 5 (backtransform2_kernel below)
// ------------------------------------------------------------------ stage 6
// GEMM problems for one Newton-Schulz step: M = Vs^H Vs; Vd = 1.5 Vs - 0.5 Vs M
__global__ void polish_setup_kernel(HeevdProb* __restrict__ probs, GemmProb* gp, int count,
                                    int step) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const HeevdProb P = probs[i];
  const bool fwd = (step & 1) == 0;  // even steps V -> V2, odd steps V2 -> V
  if (step == 0 && !P.skip_vectors) {
    probs[i].orth_max2 = 0u;
    probs[i].orth_w2 = 0u;
  }
  // steps 2 and 3 only for the problems whose first product showed an overlap
  // above kOrthPolish (two steps take an overlap d to ~0.42 d^4)
  const bool idle = P.skip_vectors || (step >= 2 && !orth_above(P.orth_max2, kOrthPolish));
  const void* Vs = fwd ? P.V : P.V2;
  void* Vd = fwd ? P.V2 : P.V;
  const int64_t lds = fwd ? P.ldv : P.ell;
  const int64_t ldd = fwd ? P.ell : P.ldv;
  GemmProb g;
  g.A = Vs; g.B = Vs; g.D = P.M; g.Csrc = P.M;
  g.lda = lds; g.ldb = lds; g.ldd = P.ell; g.ldc = P.ell;
  g.M = P.nvec; g.N = P.nvec; g.K = P.n;
  g.opA = 2; g.opB = 0;
  g.alpha_re = 1; g.alpha_im = 0; g.beta_re = 0; g.beta_im = 0;
  if (idle) g.M = 0;
  gp[i] = g;
  GemmProb h;
  h.A = Vs; h.B = P.M; h.D = Vd; h.Csrc = Vs;
  h.lda = lds; h.ldb = P.ell; h.ldd = ldd; h.ldc = lds;
  h.M = P.n; h.N = P.nvec; h.K = P.nvec;
  h.opA = 0; h.opB = 0;
  h.alpha_re = -0.5; h.alpha_im = 0; h.beta_re = 1.5; h.beta_im = 0;
  if (idle) h.M = 0;
  gp[count + i] = h;
}

// Orthogonality guard on the first polish product M = V^H V (row stride ell).
// Only eigenvectors whose eigenvalue lies above the float rounding level of
// the Gram matrix (64 ulp of lambda_0, the level below which the rank rule
// cannot see a value) are checked: vectors of numerically-zero eigenvalues
// may mix among themselves and with the others at no cost to X V_k V_k^H,
// since X maps them to ~0.  The largest |M_ij|^2 over those pairs (i > j)
// is folded into P.orth_max2 (float bits; atomicMax on non-negative floats
// orders like the values); a non-finite entry stores +inf.  The same pairs
// weighted by lambda_i / lambda_0 of the smaller eigenvalue go to P.orth_w2
// (reported only).  Above kOrthPolish the polish takes two more steps, above
// kOrthGuard the two-site repair pass re-runs the vector phase (heevd.cuh).
// Grid: (problems, row groups).
template <typename CX>
__global__ void __launch_bounds__(256) orth_guard_kernel(HeevdProb* __restrict__ probs) {
  typedef typename cx_traits<CX>::R R;
  HeevdProb& P = probs[blockIdx.x];
  if (P.skip_vectors) return;
  const int nv = P.nvec, ell = P.ell;
  const R* lam = (const R*)P.lam;
  const R l0 = lam[0];
  if (!(l0 > R(0))) return;
  const R floor_ = l0 * R(64) * (sizeof(R) == 4 ? R(5.96e-8) : R(1.11e-16));
  int kl = 0;
  while (kl < nv && lam[kl] > floor_) ++kl;  // descending: the checked columns are [0, kl)
  const CX* M = (const CX*)P.M;
  float worst = 0.f, wworst = 0.f;
  for (int i = 1 + blockIdx.y; i < kl; i += gridDim.y) {
    const float wi = (float)(lam[i] / l0);  // the smaller eigenvalue of the pair, relative
    for (int j = threadIdx.x; j < i; j += blockDim.x) {
      const CX z = M[(int64_t)i * ell + j];
      const float a2 = (float)cabs2(z);
      const bool fin = isfinite(z.x) && isfinite(z.y);
      worst = fin ? fmaxf(worst, a2) : __int_as_float(0x7f800000);
      wworst = fin ? fmaxf(wworst, a2 * wi) : __int_as_float(0x7f800000);
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    worst = fmaxf(worst, __shfl_xor_sync(0xffffffffu, worst, o));
    wworst = fmaxf(wworst, __shfl_xor_sync(0xffffffffu, wworst, o));
  }
  if ((threadIdx.x & 31) == 0 && worst > 0.f) atomicMax(&P.orth_max2, __float_as_uint(worst));
  if ((threadIdx.x & 31) == 0 && wworst > 0.f) atomicMax(&P.orth_w2, __float_as_uint(wworst));
}

// c_p = v_{j-1}^H v_j for the reflector pairs (j, j-1), j = n-2-2p, that the
// back-transformation applies together (v_j[j+1] = 1, v_j[r] = H[j][r] for
// r > j+1; v_{j-1}[j] = 1, v_{j-1}[r] = H[j-1][r] for r > j).  One warp per
// pair; the result goes to P.lu, which the vector phase no longer needs.
template <typename CX>
__global__ void __launch_bounds__(256) bt_pair_coef_kernel(const HeevdProb* __restrict__ probs) {
  const HeevdProb P = probs[blockIdx.y];
  if (P.skip_vectors) return;
  const int n = P.n, lane = threadIdx.x & 31;
  const int pi = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int j = n - 2 - 2 * pi;
  if (j < 1) return;
  const CX* H = (const CX*)P.H;
  const CX* row = H + (int64_t)j * P.ldh;
  const CX* row2 = H + (int64_t)(j - 1) * P.ldh;
  CX c = czero<CX>();
  for (int r = j + 1 + lane; r < n; r += 32) {
    const CX v1 = (r == j + 1) ? mk<CX>(1, 0) : row[r];
    cfmac(c, row2[r], v1);
  }
  c = warp_csum(c);
  if (lane == 0) ((CX*)P.lu)[pi] = c;
}

// V = Q Y, reflectors applied in pairs (j, j-1), each pair staged once per CTA
// in shared memory (double-buffered, one barrier per pair); each warp owns two
// columns of Y held in registers.  WARPS warps per CTA -> 2*WARPS columns.
//   H_{j-1} H_j z = z - v_j s1 - v_{j-1} s2 with
//   s1 = tau_j (v_j^H z),  s2 = tau_{j-1} (v_{j-1}^H z - (v_{j-1}^H v_j) s1):
// one pass forms the three dot products (the last one does not depend on z),
// one pass applies both reflectors.
template <typename CX, int NK, int WARPS>
__global__ void __launch_bounds__(WARPS * 32) backtransform2_kernel(const HeevdProb* __restrict__ probs) {
  typedef typename cx_traits<CX>::R R;
  const HeevdProb P = probs[blockIdx.y];
  const int n = P.n, ell = P.ell, nv = P.nvec;
  const int col0 = blockIdx.x * 2 * WARPS;
  if (col0 >= nv || n > NK * 32 || P.skip_vectors) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  CX* vbuf = (CX*)smem_raw;  // [2 buffers][2 reflectors][NK * 32]
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int t0 = col0 + 2 * wid, t1 = t0 + 1;
  const bool h0 = t0 < nv, h1 = t1 < nv;
  const R* Y = (const R*)P.Y;
  CX z0[NK], z1[NK];
#pragma unroll
  for (int k = 0; k < NK; ++k) {
    const int r = lane + 32 * k;
    z0[k] = (r < n && h0) ? mk<CX>(Y[(int64_t)r * ell + t0], 0) : czero<CX>();
    z1[k] = (r < n && h1) ? mk<CX>(Y[(int64_t)r * ell + t1], 0) : czero<CX>();
  }
  const CX* H = (const CX*)P.H;
  const CX* tau = (const CX*)P.tau;
  const CX* pair_coef = (const CX*)P.lu;  // free after inverse iteration
  // the rows of the next pair are read from global memory one pair ahead
  // (registers), so the L2 round trip overlaps the current pair's work;
  // thread tid stages rows tid + WARPS * 32 * u
  constexpr int PF = (NK * 32 + WARPS * 32 - 1) / (WARPS * 32);
  CX pa[PF], pb[PF];
  CX ta = czero<CX>(), tb = czero<CX>();
  auto fetch = [&](int j) {  // reflectors j and j-1 (if j >= 1)
    const CX* row = H + (int64_t)j * P.ldh;
    const CX* row2 = H + (int64_t)(j - 1) * P.ldh;
#pragma unroll
    for (int u = 0; u < PF; ++u) {
      const int r = tid + WARPS * 32 * u;
      pa[u] = (r < n && r > j + 1) ? row[r] : czero<CX>();
      pb[u] = (j >= 1 && r < n && r > j) ? row2[r] : czero<CX>();
    }
    ta = tau[j];
    tb = (j >= 1) ? tau[j - 1] : czero<CX>();
  };
  if (n >= 2) fetch(n - 2);
  for (int j = n - 2; j >= 0; j -= 2) {
    CX* b1 = vbuf + (size_t)((j >> 1) & 1) * 2 * (NK * 32);  // v_j
    CX* b2 = b1 + NK * 32;                                    // v_{j-1} (zero when j == 0)
#pragma unroll
    for (int u = 0; u < PF; ++u) {
      const int r = tid + WARPS * 32 * u;
      if (r < n) {
        b1[r] = (r == j + 1) ? mk<CX>(1, 0) : pa[u];
        b2[r] = (j >= 1 && r == j) ? mk<CX>(1, 0) : pb[u];
      }
    }
    const CX t1 = ta, t2 = tb;
    if (j >= 2) fetch(j - 2);
    __syncthreads();
    const bool a1 = (t1.x != R(0) || t1.y != R(0)), a2 = (t2.x != R(0) || t2.y != R(0));
    if (!a1 && !a2) continue;
    // v_{j-1}^H v_j, the same for every column: from bt_pair_coef_kernel
    const CX c = (j >= 1) ? pair_coef[(n - 2 - j) >> 1] : czero<CX>();
    CX d10 = czero<CX>(), d11 = czero<CX>(), d20 = czero<CX>(), d21 = czero<CX>();
    // v_j and v_{j-1} are zero in rows < j: chunks of 32 rows below that are
    // skipped (a warp-uniform test, so the register arrays keep static indices)
#pragma unroll
    for (int k = 0; k < NK; ++k) {
      const int r = lane + 32 * k;
      if (32 * k + 31 >= j && r < n) {
        const CX v1 = b1[r], v2 = b2[r];
        cfmac(d10, v1, z0[k]);
        cfmac(d11, v1, z1[k]);
        cfmac(d20, v2, z0[k]);
        cfmac(d21, v2, z1[k]);
      }
    }
    d10 = warp_csum(d10);
    d11 = warp_csum(d11);
    d20 = warp_csum(d20);
    d21 = warp_csum(d21);
    const CX s10 = cmul(t1, d10), s11 = cmul(t1, d11);
    const CX s20 = cmul(t2, csub(d20, cmul(c, s10))), s21 = cmul(t2, csub(d21, cmul(c, s11)));
#pragma unroll
    for (int k = 0; k < NK; ++k) {
      const int r = lane + 32 * k;
      if (32 * k + 31 >= j && r < n) {
        const CX v1 = b1[r], v2 = b2[r];
        z0[k] = csub(z0[k], cadd(cmul(v1, s10), cmul(v2, s20)));
        z1[k] = csub(z1[k], cadd(cmul(v1, s11), cmul(v2, s21)));
      }
    }
  }
  CX* V = (CX*)P.V;
#pragma unroll
  for (int k = 0; k < NK; ++k) {
    const int r = lane + 32 * k;
    if (r < n) {
      if (h0) V[(int64_t)r * P.ldv + t0] = z0[k];
      if (h1) V[(int64_t)r * P.ldv + t1] = z1[k];
    }
  }
}

template <typename CX, int NK>
int launch_bt(const HeevdProb* probs, int count, int maxell, cudaStream_t s) {
  // 4 warps (8 columns) per CTA: a saturated headline layer then has 32 CTAs
  // per large problem instead of 8, so the large problems' work spreads over
  // every SM rather than the ~96 their CTAs covered while the small problems'
  // SMs idled (each CTA stages every reflector pair once; the extra reads hit L2).
  constexpr int WARPS = 4;
  constexpr size_t smem = (size_t)4 * NK * 32 * sizeof(CX);
  const cudaError_t oe = agb_smem_optin(backtransform2_kernel<CX, NK, WARPS>, smem);
  if (oe != cudaSuccess) {
    agb_note_error(__FILE__, __LINE__, oe);
    return AGB_ERR_CUDA;
  }
  const int npairs = NK * 32 / 2;  // pairs for the largest n this instance handles
  bt_pair_coef_kernel<CX><<<dim3((npairs + 7) / 8, count), 256, 0, s>>>(probs);
  AGB_CHECK_LAUNCH();
  dim3 grid((maxell + 2 * WARPS - 1) / (2 * WARPS), count);
  backtransform2_kernel<CX, NK, WARPS><<<grid, WARPS * 32, smem, s>>>(probs);
  AGB_CHECK_LAUNCH();
  return AGB_OK;
}

}  // namespace

template <typename CX>
int launch_heevd_values(HeevdProb* probs, int count, int maxn, int maxell, cudaStream_t s) {
  typedef typename cx_traits<CX>::R R;
  if (count <= 0 || maxn <= 0) return AGB_OK;
  if (maxn > 1024) return AGB_ERR_UNSUPPORTED;
  const int esz = sizeof(CX);
  const size_t sm_tri = 4 * (size_t)maxn * esz;
  static bool attr_set[2] = {false, false};
  if (!attr_set[esz == 16]) {
    cudaFuncSetAttribute(tridiag_kernel<CX>, cudaFuncAttributeMaxDynamicSharedMemorySize, 65536);
    attr_set[esz == 16] = true;
  }
  prof_mark(AGB_ST_TRIDIAG, s);
  // two-stage reduction (band on a cluster, then bulge chasing) where the band
  // fits; else the one-stage cluster kernel (rows in distributed shared memory,
  // overflow rows in L2); the single-CTA kernel only if the device refuses the
  // cluster launch
  if (tridiag_stages_mode() == 0 && two_stage_bw(esz, maxn) > 0) {
    const int rc2 = launch_two_stage<CX>(probs, count, maxn, s);
    if (rc2 != AGB_OK) return rc2;
  } else {
  const int rc0 = tridiag_cluster_size(esz, maxn) > 0 ? launch_tridiag_cluster<CX>(probs, count, maxn, s)
                                                      : AGB_ERR_UNSUPPORTED;
  if (rc0 != AGB_OK) {
    cudaGetLastError();
    tridiag_kernel<CX><<<count, 1024, sm_tri, s>>>(probs);
    AGB_CHECK_LAUNCH();
  }
  }
  if (maxell <= 0) return AGB_OK;
  const size_t sm_r = 2 * (size_t)maxn * sizeof(R);
  prof_mark(AGB_ST_BISECT, s);
  bisect_kernel<R><<<dim3((maxell + 7) / 8, count), 256, sm_r, s>>>(probs);
  AGB_CHECK_LAUNCH();
  return AGB_OK;
}

template <typename CX>
int launch_heevd_vectors(HeevdProb* probs, GemmProb* gp, int count, int maxn, int maxell, cudaStream_t s,
                         const GemmCtx* ctx) {
  typedef typename cx_traits<CX>::R R;
  if (count <= 0 || maxn <= 0 || maxell <= 0) return AGB_OK;
  const size_t sm_r = 2 * (size_t)maxn * sizeof(R);
  prof_mark(AGB_ST_INVIT, s);
  if (sizeof(R) == 4 && maxn <= 1024) {
    // complex64: iterate in shared memory, factors streamed by cp.async
    const int tb = maxn <= 512 ? 64 : 32;
    const size_t sm = invit_async_smem(maxn, tb);
    const cudaError_t oe = tb == 64 ? agb_smem_optin(invit_async_kernel<64>, sm)
                                    : agb_smem_optin(invit_async_kernel<32>, sm);
    if (oe != cudaSuccess) {
      agb_note_error(__FILE__, __LINE__, oe);
      return AGB_ERR_CUDA;
    }
    if (tb == 64)
      invit_async_kernel<64><<<dim3((maxell + 63) / 64, count), 64, sm, s>>>(probs);
    else
      invit_async_kernel<32><<<dim3((maxell + 31) / 32, count), 32, sm, s>>>(probs);
  } else {
    invit_kernel<R><<<dim3((maxell + 127) / 128, count), 128, sm_r, s>>>(probs);
  }
  AGB_CHECK_LAUNCH();
  prof_mark(AGB_ST_CLUSTER, s);
  {
    // base: d, e, coef, 5n LU factors, a working column; then a staging area
    // for the parallel path's cluster block (as many columns of n as fit)
    const size_t base = (8 * (size_t)maxn + (size_t)maxell) * sizeof(R);
    const size_t budget = 160 * 1024;
    int zcap = base < budget ? (int)((budget - base) / ((size_t)maxn * sizeof(R))) : 0;
    if (zcap > maxell) zcap = maxell;
    const size_t sm = base + (size_t)zcap * maxn * sizeof(R);
    const cudaError_t oe = agb_smem_optin(cluster_invit_kernel<R>, sm);
    if (oe != cudaSuccess) {
      agb_note_error(__FILE__, __LINE__, oe);
      return AGB_ERR_CUDA;
    }
    const int maxcl = maxell / 2 > 0 ? maxell / 2 : 1;
    cluster_list_kernel<R><<<(count + 127) / 128, 128, 0, s>>>(probs, count);
    AGB_CHECK_LAUNCH();
    cluster_invit_kernel<R><<<dim3(maxcl, count), 256, sm, s>>>(probs, zcap);
    AGB_CHECK_LAUNCH();
  }
  int rc;
  prof_mark(AGB_ST_BACKTRANS, s);
  if (tridiag_stages_mode() == 0 && two_stage_bw(sizeof(CX), maxn) > 0)
    rc = launch_bt_two_stage<CX>(probs, count, maxn, maxell, s);
  else if (maxn <= 128) rc = launch_bt<CX, 4>(probs, count, maxell, s);
  else if (maxn <= 256) rc = launch_bt<CX, 8>(probs, count, maxell, s);
  else if (maxn <= 512) rc = launch_bt<CX, 16>(probs, count, maxell, s);
  else rc = launch_bt<CX, 32>(probs, count, maxell, s);
  if (rc) return rc;
  prof_mark(AGB_ST_POLISH, s);
  // Newton-Schulz V <- V (3I - V^H V) / 2: quadratic convergence.  The vectors
  // arrive within ~eps*||T||/gap of orthonormal (gaps below the cluster
  // tolerance are handled by the cluster kernel), normally below 1e-2 in
  // float32, so two steps reach the float32 floor; problems whose first
  // product shows more take two more (an even count leaves the result in V).
  // The extra steps run on the SIMT GEMM: they are rare, and a launch whose
  // problems are all idle then costs one short wave of small CTAs instead of
  // several waves of tensor-core CTAs that reserve ~200 KB of shared memory each.
  for (int step = 0; step < 4; ++step) {
    const GemmCtx* c = step < 2 ? ctx : nullptr;
    polish_setup_kernel<<<(count + 127) / 128, 128, 0, s>>>(probs, gp, count, step);
    AGB_CHECK_LAUNCH();
    if ((rc = launch_gemm_probs<CX>(gp, count, maxell, maxell, s, c, maxn))) return rc;
    if (step == 0) {
      orth_guard_kernel<CX><<<dim3(count, 8), 256, 0, s>>>(probs);
      AGB_CHECK_LAUNCH();
    }
    if ((rc = launch_gemm_probs<CX>(gp + count, count, maxn, maxell, s, c, maxell))) return rc;
  }
  return AGB_OK;
}

template <typename CX>
int launch_heevd(HeevdProb* probs, GemmProb* gp, int count, int maxn, int maxell, cudaStream_t s) {
  int rc = launch_heevd_values<CX>(probs, count, maxn, maxell, s);
  if (rc) return rc;
  return launch_heevd_vectors<CX>(probs, gp, count, maxn, maxell, s);
}

template int launch_heevd<float2>(HeevdProb*, GemmProb*, int, int, int, cudaStream_t);
template int launch_heevd<double2>(HeevdProb*, GemmProb*, int, int, int, cudaStream_t);
template int launch_heevd_values<float2>(HeevdProb*, int, int, int, cudaStream_t);
template int launch_heevd_values<double2>(HeevdProb*, int, int, int, cudaStream_t);
template int launch_heevd_vectors<float2>(HeevdProb*, GemmProb*, int, int, int, cudaStream_t, const GemmCtx*);
template int launch_heevd_vectors<double2>(HeevdProb*, GemmProb*, int, int, int, cudaStream_t, const GemmCtx*);

// ------------------------------------------------------------------ standalone entry
namespace {
__global__ void heevd_setup_kernel(HeevdProb* probs, void* H, void* evecs, char* scratch,
                                   size_t scratch_stride, int batch, int n, int ell, int esz,
                                   uint64_t seed) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= batch) return;
  HeevdProb p;
  p.H = (char*)H + (size_t)b * n * n * esz;
  p.ldh = n;
  p.n = n;
  p.ell = ell;
  p.V = (char*)evecs + (size_t)b * n * ell * esz;
  p.ldv = ell;
  p.seed = seed + 0x9E3779B97F4A7C15ull * (uint64_t)b;
  p.skip_vectors = 0;
  p.nvec = ell;
  p.redo = 0;
  p.orth_max2 = 0u;
  p.orth_w2 = 0u;
  p.ctol = kClusterTol;
  p.fail = 0;
  heevd_assign_scratch_dev(p, scratch + (size_t)b * scratch_stride, esz);
  probs[b] = p;
}

template <typename R>
__global__ void heevd_evals_kernel(const HeevdProb* probs, R* evals, int batch, int ell) {
  const int b = blockIdx.y;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= batch || t >= ell) return;
  const HeevdProb p = probs[b];
  evals[(size_t)b * ell + t] = ((const R*)p.lam)[t] * *((const R*)p.scale);
}
}  // namespace

extern "C" size_t agb_heevd_workspace(int dtype, int n, int ell) {
  const int esz = dtype == AGB_C64 ? 8 : 16;
  return agb_align(heevd_scratch_bytes(esz, n, ell)) + agb_align(sizeof(HeevdProb)) +
         agb_align(2 * sizeof(GemmProb));
}

extern "C" int agb_heevd(int dtype, int batch, int n, int ell, void* H, void* evals, void* evecs,
                         void* ws, size_t ws_bytes, uint64_t seed, void* stream) {
  if (dtype != AGB_C64 && dtype != AGB_C128) return AGB_ERR_ARG;
  if (batch < 0 || n < 0 || ell < 0 || ell > n) return AGB_ERR_ARG;
  if (n > 1024) return AGB_ERR_UNSUPPORTED;
  if (batch == 0 || n == 0) return AGB_OK;
  const int esz = dtype == AGB_C64 ? 8 : 16;
  const size_t stride = agb_align(heevd_scratch_bytes(esz, n, ell));
  const size_t need = (size_t)batch * (stride + agb_align(sizeof(HeevdProb)) + agb_align(2 * sizeof(GemmProb)));
  if (ws_bytes < need) return AGB_ERR_WORKSPACE;
  char* base = (char*)ws;
  HeevdProb* probs = (HeevdProb*)base;
  GemmProb* gp = (GemmProb*)(base + agb_align((size_t)batch * sizeof(HeevdProb)));
  char* scratch = base + agb_align((size_t)batch * sizeof(HeevdProb)) + agb_align((size_t)batch * 2 * sizeof(GemmProb));
  cudaStream_t s = (cudaStream_t)stream;
  heevd_setup_kernel<<<(batch + 127) / 128, 128, 0, s>>>(probs, H, evecs, scratch, stride, batch, n, ell, esz, seed);
  AGB_CHECK_LAUNCH();
  int rc = (dtype == AGB_C64) ? launch_heevd<float2>(probs, gp, batch, n, ell, s)
                              : launch_heevd<double2>(probs, gp, batch, n, ell, s);
  if (rc) return rc;
  if (ell > 0) {
    dim3 g((ell + 127) / 128, batch);
    if (dtype == AGB_C64) heevd_evals_kernel<float><<<g, 128, 0, s>>>(probs, (float*)evals, batch, ell);
    else heevd_evals_kernel<double><<<g, 128, 0, s>>>(probs, (double*)evals, batch, ell);
    AGB_CHECK_LAUNCH();
  }
  return AGB_OK;
}
