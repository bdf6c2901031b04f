// Two-site MPS update for a batch of gates on disjoint bonds (sm_103a).
//
// Per gate g (bond i, A = site i [chiL,2,chiM], B = site i+1 [chiM,2,chiR]):
//   X  = fused contraction + gate          [m = 2chiL, n = 2chiR]
//   G  = X^H X                             (n x n Hermitian Gram matrix)
//   V  = top-ell eigenvectors of G         (heevd.cu)
//   AV = X V ;  sigma_t^2 = ||AV[:, t]||^2 (Rayleigh quotients, sorted)
//   k  = reference rank rule on sigma (truncation.py:21-83)
//   A_new = AV[:, :k]  (= U_k S_k: singular values absorbed LEFT, adaptive_mps.py:281-285)
//   B_new = V[:, :k]^H (= Vh_k)
// The Gram formulation never divides by a singular value: A_new B_new = X V_k V_k^H
// is the projection of X onto the kept right singular subspace.
#include <math.h>

#include "gemm_tc.cuh"
#include "heevd.cuh"
#include "prof.cuh"

namespace {

struct Slab {
  size_t X, G, heevd, V, AV, sig2, perm, total;
};

AGB_HD Slab slab_layout(int m, int n, int ell, int esz) {
  Slab s;
  size_t o = 0;
  s.X = o;     o += agb_align((size_t)m * n * esz);
  s.G = o;     o += agb_align((size_t)n * n * esz);
  s.heevd = o; o += agb_align(heevd_scratch_bytes(esz, n, ell));
  s.V = o;     o += agb_align((size_t)n * ell * esz);
  s.AV = o;    o += agb_align((size_t)m * ell * esz);
  s.sig2 = o;  o += agb_align((size_t)ell * sizeof(double));
  s.perm = o;  o += agb_align((size_t)ell * sizeof(int));
  s.total = o;
  return s;
}

AGB_HD double dbits(int64_t v) {
  union {
    int64_t i;
    double d;
  } u;
  u.i = v;
  return u.d;
}
AGB_HD int64_t bitsd(double v) {
  union {
    int64_t i;
    double d;
  } u;
  u.d = v;
  return u.i;
}

// header of the batch workspace: [HeevdProb x G][GemmProb x 4G][ContractProb x G]
struct ContractProb {
  const void* A;
  const void* B;
  const void* U;
  void* X;
  int chiL, chiM, chiR;
  int64_t ldx;
};

AGB_HD size_t header_bytes(int ng) {
  return agb_align((size_t)ng * sizeof(HeevdProb)) + agb_align((size_t)ng * 4 * sizeof(GemmProb)) +
         agb_align((size_t)ng * sizeof(ContractProb)) + 256;  // + tensor-core status word
}
AGB_HD int* status_word(char* ws, int ng) { return (int*)(ws + header_bytes(ng) - 256); }

// Scratch of the tensor-core GEMMs of a batch (complex64 only), the largest
// over Gram (n x n, K = m), X V (m x ell, K = n) and the polish products
// (ell x ell, K = n; n x ell, K = ell); it occupies the last bytes of the
// workspace (a token: the split operands live in shared memory).
size_t tc_tail_bytes(int dtype, int ng, int maxm, int maxn, int maxell) {
  if (dtype != AGB_C64 || ng <= 0) return 0;
  size_t b = tc_gemm_scratch_bytes(ng, maxn, maxn, maxm);
  size_t t = tc_gemm_scratch_bytes(ng, maxm, maxell, maxn);
  if (t > b) b = t;
  t = tc_gemm_scratch_bytes(ng, maxell, maxell, maxn);
  if (t > b) b = t;
  t = tc_gemm_scratch_bytes(ng, maxn, maxell, maxell);
  if (t > b) b = t;
  return agb_align(b);
}

// ------------------------------------------------------------------ setup
__global__ void setup_kernel(int64_t* __restrict__ desc, int ng, char* ws, int esz) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= ng) return;
  int64_t* D = desc + (int64_t)g * AGB_D_NFIELDS;
  D[AGB_D_STATUS] = AGB_OK;
  D[AGB_D_REPAIR] = 0;
  if (D[AGB_D_DIMS]) {
    // device-resident MPS: the shapes are whatever earlier launches left in the
    // bond-dimension array, bounded by the capacities the batch was planned
    // with (CAPL/CAPM/CAPR, ELLPLAN stay untouched, so a captured launch
    // sequence can be replayed)
    const int* dims = (const int*)D[AGB_D_DIMS];
    const int b = (int)D[AGB_D_BOND];
    const int cL = dims[b], cM = dims[b + 1], cR = dims[b + 2];
    const bool ok = cL >= 1 && cM >= 1 && cR >= 1 && cL <= (int)D[AGB_D_CAPL] && cM <= (int)D[AGB_D_CAPM] &&
                    cR <= (int)D[AGB_D_CAPR];
    D[AGB_D_CHIL] = ok ? cL : 1;  // 1 x 1 x 1: a shape every kernel handles
    D[AGB_D_CHIM] = ok ? cM : 1;
    D[AGB_D_CHIR] = ok ? cR : 1;
    if (!ok) D[AGB_D_STATUS] = AGB_ERR_ARG;
    const int mm = 2 * (int)D[AGB_D_CHIL], nn = 2 * (int)D[AGB_D_CHIR], cap = (int)D[AGB_D_CAP];
    int full = mm < nn ? mm : nn;
    if (cap < full) full = cap;
    const int ep = (int)D[AGB_D_ELLPLAN];
    D[AGB_D_ELL] = ep < full ? ep : full;
  }
  const int chiL = (int)D[AGB_D_CHIL], chiM = (int)D[AGB_D_CHIM], chiR = (int)D[AGB_D_CHIR];
  const int m = 2 * chiL, n = 2 * chiR, ell = (int)D[AGB_D_ELL];
  char* slab = ws + D[AGB_D_WS];
  const Slab L = slab_layout(m, n, ell, esz);
  HeevdProb* hp = (HeevdProb*)ws;
  GemmProb* gp = (GemmProb*)(ws + agb_align((size_t)ng * sizeof(HeevdProb)));
  ContractProb* cp = (ContractProb*)(ws + agb_align((size_t)ng * sizeof(HeevdProb)) +
                                     agb_align((size_t)ng * 4 * sizeof(GemmProb)));
  HeevdProb p;
  p.H = slab + L.G;
  p.ldh = n;
  p.n = n;
  p.ell = ell;
  p.V = slab + L.V;
  p.ldv = ell;
  p.seed = (uint64_t)D[AGB_D_SEED];
  p.skip_vectors = 0;
  p.nvec = ell;
  p.redo = 0;
  p.orth_max2 = 0u;
  p.orth_w2 = 0u;
  p.fail = 0;
  p.ctol = D[AGB_D_CTOL] ? dbits(D[AGB_D_CTOL]) : kClusterTol;
  heevd_assign_scratch_dev(p, slab + L.heevd, esz);
  hp[g] = p;
  // gp[0..2ng) reserved for the eigensolver polish; [2ng, 3ng) Gram; [3ng, 4ng) AV
  GemmProb gr;
  gr.A = slab + L.X; gr.B = slab + L.X; gr.D = slab + L.G; gr.Csrc = slab + L.G;
  gr.lda = n; gr.ldb = n; gr.ldd = n; gr.ldc = n;
  gr.M = n; gr.N = n; gr.K = m;
  gr.opA = 2; gr.opB = 0;
  gr.alpha_re = 1; gr.alpha_im = 0; gr.beta_re = 0; gr.beta_im = 0;
  gp[2 * ng + g] = gr;
  GemmProb av;
  av.A = slab + L.X; av.B = slab + L.V; av.D = slab + L.AV; av.Csrc = slab + L.AV;
  av.lda = n; av.ldb = ell; av.ldd = ell; av.ldc = ell;
  av.M = m; av.N = ell; av.K = n;
  av.opA = 0; av.opB = 0;
  av.alpha_re = 1; av.alpha_im = 0; av.beta_re = 0; av.beta_im = 0;
  gp[3 * ng + g] = av;
  ContractProb c;
  c.A = (const void*)D[AGB_D_A];
  c.B = (const void*)D[AGB_D_B];
  c.U = (const void*)D[AGB_D_U];
  c.X = slab + L.X;
  c.chiL = chiL;
  c.chiM = chiM;
  c.chiR = chiR;
  c.ldx = n;
  cp[g] = c;
}

// ------------------------------------------------------------------ contraction
// Tile: 16 left indices l x 16 right indices j, all four (p', q'), K-chunks of 16.
template <typename CX>
__global__ void __launch_bounds__(256) contract_gate_kernel(const ContractProb* __restrict__ probs,
                                                            ContractProb single) {
  const ContractProb P = probs ? probs[blockIdx.z] : single;
  const int l0 = blockIdx.y * 16, j0 = blockIdx.x * 16;
  if (l0 >= P.chiL || j0 >= P.chiR) return;
  __shared__ CX As[16][2][17];
  __shared__ CX Bs[16][2][17];
  __shared__ CX Us[16];
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const CX* A = (const CX*)P.A;
  const CX* B = (const CX*)P.B;
  if (tid < 16) Us[tid] = ((const CX*)P.U)[tid];
  CX th[2][2];
  th[0][0] = th[0][1] = th[1][0] = th[1][1] = czero<CX>();
  const int chiM = P.chiM, chiR = P.chiR, chiL = P.chiL;
  for (int r0 = 0; r0 < chiM; r0 += 16) {
#pragma unroll
    for (int e = 0; e < 2; ++e) {
      const int idx = tid + 256 * e;  // 0..511
      // A[l][p][r]: l = idx / 32, p = (idx / 16) % 2, r = idx % 16
      {
        const int l = idx >> 5, pp = (idx >> 4) & 1, r = idx & 15;
        const int gl = l0 + l, gr = r0 + r;
        As[l][pp][r] = (gl < chiL && gr < chiM) ? A[((int64_t)gl * 2 + pp) * chiM + gr] : czero<CX>();
      }
      // B[r][q][j]: r = idx / 32, q = (idx / 16) % 2, j = idx % 16
      {
        const int r = idx >> 5, q = (idx >> 4) & 1, j = idx & 15;
        const int gr = r0 + r, gj = j0 + j;
        Bs[r][q][j] = (gr < chiM && gj < chiR) ? B[((int64_t)gr * 2 + q) * chiR + gj] : czero<CX>();
      }
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < 16; ++r) {
      const CX a0 = As[ty][0][r], a1 = As[ty][1][r];
      const CX b0 = Bs[r][0][tx], b1 = Bs[r][1][tx];
      cfma(th[0][0], a0, b0);
      cfma(th[0][1], a0, b1);
      cfma(th[1][0], a1, b0);
      cfma(th[1][1], a1, b1);
    }
    __syncthreads();
  }
  const int l = l0 + ty, j = j0 + tx;
  if (l >= chiL || j >= chiR) return;
  CX* X = (CX*)P.X;
#pragma unroll
  for (int p = 0; p < 2; ++p)
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const int row = 2 * p + q;
      CX acc = czero<CX>();
      cfma(acc, Us[row * 4 + 0], th[0][0]);
      cfma(acc, Us[row * 4 + 1], th[0][1]);
      cfma(acc, Us[row * 4 + 2], th[1][0]);
      cfma(acc, Us[row * 4 + 3], th[1][1]);
      X[((int64_t)l * 2 + p) * P.ldx + (int64_t)q * chiR + j] = acc;
    }
}

// The reference rank rule (truncation.py:21-83) for one gate, on sigma^2 values
// sorted descending, with torch-CPU float32 semantics when f32 (double-
// accumulated cumsum rounded to float32 per element; threshold
// f32(f32(1 - eps^2) * total)).  total is E[-1] of the reference: the cumsum's
// end when every potentially non-zero value is present (ell >= kmax), else
// ||X||_F^2 (total_d).  All threads of the block call it: the cumsum is a
// parallel double prefix sum, the first index reaching the threshold a block
// minimum, the entropy terms a block sum (skipped when !stats).  On GB300 a
// serial double-precision loop over the values costs ~0.6 ms per gate.
AGB_DEV void rank_rule_block(const double* s_sorted, double* E, int ell, int kmax, int cap, double eps, bool f32,
                             double total_d, int& k, double& eps_local, double& entropy, double& condS,
                             int& status, int& needed, bool stats = true) {
  __shared__ double sh_d[64];
  __shared__ int sh_i[4];
  __shared__ double sh_tot[2];
  const int tid = threadIdx.x, nt = blockDim.x;
  eps_local = 0;
  entropy = 0;
  condS = INFINITY;
  status = AGB_OK;
  needed = ell;
  if (ell == 0) {
    k = 0;
    return;
  }
  for (int t = tid; t < ell; t += nt) {
    if (f32) {
      const float sv = sqrtf((float)s_sorted[t]);
      E[t] = (double)(sv * sv);
    } else {
      const double sv = sqrt(s_sorted[t]);
      E[t] = sv * sv;
    }
  }
  __syncthreads();
  // inclusive Hillis-Steele scan (ell <= 1024 <= 2 * blockDim)
  for (int off = 1; off < ell; off <<= 1) {
    double v0 = 0, v1 = 0;
    const int t0 = tid, t1 = tid + nt;
    if (t0 < ell && t0 >= off) v0 = E[t0 - off];
    if (t1 < ell && t1 >= off) v1 = E[t1 - off];
    __syncthreads();
    if (t0 < ell) E[t0] += v0;
    if (t1 < ell) E[t1] += v1;
    __syncthreads();
  }
  for (int t = tid; t < ell; t += nt) E[t] = f32 ? (double)(float)E[t] : E[t];
  __syncthreads();
  if (tid == 0) {
    const double total = (ell >= kmax) ? E[ell - 1] : (f32 ? (double)(float)total_d : total_d);
    sh_tot[0] = total;
    sh_tot[1] = f32 ? (double)(float)((float)(1.0 - eps * eps) * (float)total) : (1.0 - eps * eps) * total;
    sh_i[0] = 0x7fffffff;
  }
  __syncthreads();
  const double total = sh_tot[0], thresh = sh_tot[1];
  if (total < 1e-30) {
    k = 1;
    return;
  }
  for (int t = tid; t < ell; t += nt)
    if (E[t] >= thresh) atomicMin(&sh_i[0], t);
  __syncthreads();
  int ktol = (sh_i[0] == 0x7fffffff) ? -1 : sh_i[0] + 1;
  const int full = min(kmax, cap);
  if (ktol < 0 && ell < full) {
    // Only the leading ell values are present.  If what is missing from the
    // total is below the resolution of the rule (eps^2, or the float32 /
    // float64 rounding of the total, whichever is larger), the cumulative sum
    // has reached its final value inside the present values: k is where it
    // stops changing, as in the full rule (where total is the cumsum's end).
    const double res = fmax(eps * eps, f32 ? 1.2e-7 : 2.3e-16);
    if (total_d - E[ell - 1] <= res * total_d) {
      if (tid == 0) sh_i[1] = 0x7fffffff;
      __syncthreads();
      for (int t = tid; t < ell; t += nt)
        if (E[t] >= E[ell - 1]) atomicMin(&sh_i[1], t);
      __syncthreads();
      ktol = sh_i[1] + 1;
    } else {
      status = AGB_ERR_RANK;
      needed = full;
      ktol = ell;
    }
  } else if (ktol < 0) {
    ktol = kmax;
  }
  ktol = min(ktol, kmax);
  k = min(min(ktol, cap), ell);
  const double rem = total - E[k - 1];
  eps_local = f32 ? (double)sqrtf((float)fmax(rem, 0.0)) : sqrt(fmax(rem, 0.0));
  if (!stats) return;
  double ssum = 0;
  for (int t = tid; t < k; t += nt) ssum += s_sorted[t];
  ssum = block_sum(ssum, sh_d);
  // entropy terms in the working precision (float32 logs for complex64: the
  // double-precision log is tens of FP64 operations per value)
  double ent = 0;
  if (f32) {
    const float inv = 1.0f / (float)ssum;
    for (int t = tid; t < k; t += nt) {
      const float pr = (float)s_sorted[t] * inv;
      ent -= (double)(pr * logf(fmaxf(pr, 1e-30f)));
    }
  } else {
    for (int t = tid; t < k; t += nt) {
      const double pr = s_sorted[t] / ssum;
      ent -= pr * log(fmax(pr, 1e-30));
    }
  }
  entropy = block_sum(ent, sh_d);
  if (k > 1) {
    if (f32) {
      const float s0 = sqrtf((float)s_sorted[0]), sk = sqrtf((float)s_sorted[k - 1]);
      condS = sk > 0.f ? (double)(s0 / sk) : INFINITY;
    } else {
      const double s0 = sqrt(s_sorted[0]), sk = sqrt(s_sorted[k - 1]);
      condS = sk > 0 ? s0 / sk : INFINITY;
    }
  }
}

// Between the eigenvalue and eigenvector phases, with the eigenvalues of G:
// * when the rank rule keeps every column (k == n <= m), any orthonormal basis
//   factorises X exactly (X = (X V)(V^H)), so the gate takes V = I: A_new = X,
//   B_new = I.  This is a unitary gauge change on the bond relative to the SVD
//   factors, so the state and every later gate's spectrum are unchanged.  Flat
//   spectra (maximally mixed small subsystems at the chain ends) would
//   otherwise need one large eigenvalue cluster orthogonalised.
// * otherwise only the eigenvectors the rank rule can keep are computed: the
//   rule applied to the eigenvalues gives k_lam; the vector phase computes
//   nvec = k_lam + pad (never splitting an eigenvalue cluster), and the rank
//   kernel applies the rule again to the Rayleigh quotients of those vectors.
//   If the threshold is not reached within nvec, the gate reports
//   AGB_ERR_RANK and the caller re-runs it with every vector (NVEC = -1).
//   Rank-deficient X (a zero eigenvalue of multiplicity n - rank) then costs
//   nothing in the vector phase.
template <typename CX>
__global__ void __launch_bounds__(512) prerank_kernel(int64_t* __restrict__ desc, int ng, char* ws) {
  typedef typename cx_traits<CX>::R R;
  const int g = blockIdx.x, tid = threadIdx.x, nt = blockDim.x;
  int64_t* D = desc + (int64_t)g * AGB_D_NFIELDS;
  const int chiL = (int)D[AGB_D_CHIL], chiR = (int)D[AGB_D_CHIR];
  const int m = 2 * chiL, n = 2 * chiR, ell = (int)D[AGB_D_ELL], cap = (int)D[AGB_D_CAP];
  HeevdProb* hp = (HeevdProb*)ws;
  GemmProb* gp = (GemmProb*)(ws + agb_align((size_t)ng * sizeof(HeevdProb)));
  if (tid == 0) {
    D[AGB_D_MODE] = 0;
    hp[g].skip_vectors = 0;
    hp[g].nvec = ell;
    gp[3 * ng + g].N = ell;
  }
  if (n > 1024 || ell <= 0) return;
  const HeevdProb P = hp[g];
  const R* lam = (const R*)P.lam;
  const R scale = *((const R*)P.scale);
  __shared__ double s2[1024], E[1024];
  __shared__ double red[32];
  for (int t = tid; t < ell; t += nt) {
    const R v = lam[t] * scale;
    const double a = v > R(0) ? (double)v : 0.0;
    s2[t] = (sizeof(R) == 4) ? (double)(float)a : a;
  }
  // trace(G) = sum of the tridiagonal's diagonal (times the scale)
  SumAcc<R> ta;
  for (int i = tid; i < n; i += nt) ta.add(((const R*)P.d)[i]);
  const double tr = block_sum(ta.value(), red) * (double)scale;  // (ends with a barrier: s2 is complete)
  const int kmax = min(m, n);
  int k, status, needed;
  double el, en, cs;
  rank_rule_block(s2, E, ell, kmax, cap, dbits(D[AGB_D_EPS]), sizeof(R) == 4, tr, k, el, en, cs, status, needed,
                  false);
  if (tid != 0) return;
  if (m >= n && ell == n && status == AGB_OK && k == n) {
    D[AGB_D_MODE] = 1;
    hp[g].skip_vectors = 1;
    gp[3 * ng + g].M = 0;  // no X*V product
    return;
  }
  if (D[AGB_D_NVEC] < 0 || status != AGB_OK) return;  // every vector
  // k from the eigenvalues, then every eigenvalue above the float rounding
  // level of G (values the rule on the Rayleigh quotients could still count),
  // plus a pad for the difference between eigenvalues and Rayleigh quotients
  int kl = k;
  const double floor_ = s2[0] * (sizeof(R) == 4 ? 64.0 * 5.96e-8 : 64.0 * 1.11e-16);
  while (kl < ell && s2[kl] > floor_) ++kl;
  int nv = kl + max(8, kl / 8);
  if (nv >= ell) return;
  // do not split a cluster (the tolerance of the cluster kernel)
  const R scl = fmax(fabs(lam[0]), fabs(lam[ell - 1]));
  const R tol = (R)P.ctol * fmax(scl, (R)(sizeof(R) == 4 ? 1e-30 : 1e-290));
  while (nv < ell && (lam[nv - 1] - lam[nv]) <= tol) ++nv;
  hp[g].nvec = nv;
  gp[3 * ng + g].N = nv;
}

// ------------------------------------------------------------------ rank selection
// One block per gate.  sigma_t^2 = ||AV[:, t]||^2, sorted descending; then the
// reference rank rule with torch-CPU float32 semantics for complex64:
//   E = cumsum(S*S) accumulated in double, each partial rounded to float32;
//   thresh = f32(f32(1 - eps^2) * total); k_tol = searchsorted_left(E, thresh) + 1.
template <typename CX>
// pass: 0 first pass (a repair pass follows), 1 repair pass (only repaired
// gates), 2 first pass with no repair pass.  In passes 1 and 2 a gate whose
// eigenvectors failed the orthogonality guard reports AGB_ERR_NOCONV unless
// `guard` is 0 (the guard is then only reported).
__global__ void __launch_bounds__(1024) rank_kernel(int64_t* __restrict__ desc, int ng, char* ws, int pass,
                                                    int guard) {
  typedef typename cx_traits<CX>::R R;
  const bool f32 = sizeof(R) == 4;
  const int g = blockIdx.x;
  if (pass == 1 && !((const HeevdProb*)ws)[g].redo) return;
  int64_t* D = desc + (int64_t)g * AGB_D_NFIELDS;
  const int chiL = (int)D[AGB_D_CHIL], chiR = (int)D[AGB_D_CHIR];
  const int m = 2 * chiL, n = 2 * chiR, ell = (int)D[AGB_D_ELL], cap = (int)D[AGB_D_CAP];
  const double eps = dbits(D[AGB_D_EPS]);
  char* slab = ws + D[AGB_D_WS];
  const Slab Ls = slab_layout(m, n, ell, sizeof(CX));
  const CX* X = (const CX*)(slab + Ls.X);
  const CX* AV = (const CX*)(slab + Ls.AV);
  double* sig2 = (double*)(slab + Ls.sig2);
  int* perm = (int*)(slab + Ls.perm);
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double* s_raw = (double*)smem_raw;  // [ell]
  double* s_sorted = s_raw + ell;     // [ell]
  __shared__ double red[32];
  R* s_key = (R*)(s_sorted + 2 * (size_t)ell);  // [ell] sort keys (values are exact in R)
  __shared__ double part[1024];
  const int tid = threadIdx.x, nt = blockDim.x;
  // total = ||X||_F^2 to double accuracy
  SumAcc<R> xa;
  for (int64_t i = tid; i < (int64_t)m * n; i += nt) xa.add(cabs2(X[i]));
  const double total_d = block_sum(xa.value(), red);
  __shared__ int nonfinite;
  if (tid == 0) nonfinite = !isfinite(total_d);
  __syncthreads();
  const int mode0 = (int)D[AGB_D_MODE];
  const HeevdProb* hp = (const HeevdProb*)ws;
  // values present: the nvec leading eigenvectors (all ell in the identity mode);
  // AV and V keep the row stride ell
  const int nv = (mode0 == 1) ? ell : min(hp[g].nvec, ell);
  // column norms of AV: a pass covers cw consecutive columns (one per thread,
  // coalesced along the row); G = nt / cw groups of threads split the rows and
  // group 0 adds the groups' partials in a fixed order
  if (mode0 != 1) {
    const int cw = min(max(32, ((nv + 31) / 32) * 32), nt), G = nt / cw;
    const int lt = tid % cw, grp = tid / cw;
    for (int c0 = 0; c0 < nv; c0 += cw) {
      const int t = c0 + lt;
      SumAcc<R> ca;
      if (grp < G && t < nv)
        for (int r = grp; r < m; r += G) ca.add(cabs2(AV[(int64_t)r * ell + t]));
      part[tid] = ca.value();
      __syncthreads();
      if (grp == 0 && t < nv) {
        double acc = 0;
        for (int q = 0; q < G; ++q) acc += part[q * cw + lt];
        s_raw[t] = acc;
      }
      __syncthreads();
    }
  }
  for (int t = tid; t < nv; t += nt) {
    double acc = s_raw[t];
    if (mode0 == 1) {
      // identity basis: the eigenvalues (descending) are the sigma^2
      const R v = ((const R*)hp[g].lam)[t] * *((const R*)hp[g].scale);
      acc = v > R(0) ? (double)v : 0.0;
    }
    if (!isfinite(acc)) {
      nonfinite = 1;
      acc = -1.0;  // sorts last; the gate is reported as failed below
    }
    s_raw[t] = f32 ? (double)(float)acc : acc;
    s_key[t] = (R)s_raw[t];
  }
  __syncthreads();
  // rank of each value (descending, ties by index): always a permutation of 0..nv-1.
  // The keys compare in R (exact: the values are rounded to R above), so the
  // nv^2 comparisons stay off the FP64 pipe for complex64.
  // The identity-basis mode keeps the eigenvalue order (already descending), so
  // the rank rule sees exactly the values the pre-rank decision used.
  for (int t = tid; t < nv; t += nt) {
    const double v = s_raw[t];
    int rk = t;
    if (mode0 != 1) {
      const R vk = s_key[t];
      rk = 0;
      for (int u = 0; u < nv; ++u) {
        const R w = s_key[u];
        rk += (w > vk) || (w == vk && u < t);
      }
    }
    s_sorted[rk] = v;
    perm[rk] = t;
  }
  __syncthreads();
  for (int t = tid; t < nv; t += nt) sig2[t] = s_sorted[t];
  const int kmax = min(m, n);
  int k, status, needed;
  double eps_local, entropy, condS;
  rank_rule_block(s_sorted, s_sorted + ell, nv, kmax, cap, eps, f32, total_d, k, eps_local, entropy, condS, status,
                  needed);
  if (tid != 0) return;
  if (nonfinite) {
    status = AGB_ERR_NOCONV;
    k = 0;
  }
  if (guard && pass != 0 && orth_exceeds(hp[g].orth_max2) && mode0 != 1) {  // not orthonormal, no repair left
    status = AGB_ERR_NOCONV;
    k = 0;
  }
  if (hp[g].fail) {  // a bounded wait of the band stage expired
    status = AGB_ERR_TIMEOUT;
    k = 0;
  }
  if (*status_word(ws, ng) != 0) {  // a bounded wait in a tensor-core GEMM expired
    status = *status_word(ws, ng);
    k = 0;
  }
  if (D[AGB_D_STATUS] != AGB_OK) {  // shapes rejected in setup
    status = (int)D[AGB_D_STATUS];
    k = 0;
  }
  D[AGB_D_K] = k;
  D[AGB_D_EPSLOC] = bitsd(eps_local);
  D[AGB_D_ENTROPY] = bitsd(entropy);
  D[AGB_D_CONDS] = bitsd(condS);
  D[AGB_D_STATUS] = status;
  D[AGB_D_TOTAL] = bitsd(total_d);
  D[AGB_D_NEEDED] = needed;
  D[AGB_D_ORTH] = bitsd(mode0 == 1 ? 0.0 : (double)__uint_as_float(hp[g].orth_max2));
  D[AGB_D_ORTHW] = bitsd(mode0 == 1 ? 0.0 : (double)__uint_as_float(hp[g].orth_w2));
}

// ------------------------------------------------------------------ scatter
template <typename CX>
__global__ void scatter_kernel(const int64_t* __restrict__ desc, char* ws) {
  const int g = blockIdx.y;
  const int64_t* D = desc + (int64_t)g * AGB_D_NFIELDS;
  const int chiL = (int)D[AGB_D_CHIL], chiR = (int)D[AGB_D_CHIR];
  const int m = 2 * chiL, n = 2 * chiR, ell = (int)D[AGB_D_ELL], k = (int)D[AGB_D_K];
  char* slab = ws + D[AGB_D_WS];
  const Slab Ls = slab_layout(m, n, ell, sizeof(CX));
  const CX* AV = (const CX*)(slab + Ls.AV);
  const CX* V = (const CX*)(slab + Ls.V);
  const CX* X = (const CX*)(slab + Ls.X);
  const int* perm = (const int*)(slab + Ls.perm);
  const int mode = (int)D[AGB_D_MODE];
  CX* An = (CX*)D[AGB_D_ANEW];
  CX* Bn = (CX*)D[AGB_D_BNEW];
  const int nv = (mode == 1) ? ell : min(((const HeevdProb*)ws)[g].nvec, ell);
  if (!An || !Bn || k <= 0 || k > nv) return;
  if (mode == 1 && k != n) return;
  if (D[AGB_D_STATUS] != AGB_OK) return;
  if (D[AGB_D_DIMS] && blockIdx.x == 0 && threadIdx.x == 0)
    ((int*)D[AGB_D_DIMS])[(int)D[AGB_D_BOND] + 1] = k;  // read by the next batch's setup
  const int64_t na = (int64_t)m * k, nb = (int64_t)k * n;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < na + nb;
       i += (int64_t)gridDim.x * blockDim.x) {
    if (mode == 1) {
      if (i < na) {
        An[i] = X[i];  // k == n: A_new = X
      } else {
        const int64_t ii = i - na;
        Bn[ii] = ((ii / n) == (ii % n)) ? mk<CX>(1, 0) : czero<CX>();
      }
      continue;
    }
    if (i < na) {
      const int r = (int)(i / k), j = (int)(i % k);
      const int pj = perm[j];
      An[i] = (pj >= 0 && pj < nv) ? AV[(int64_t)r * ell + pj] : czero<CX>();
    } else {
      const int64_t ii = i - na;
      const int j = (int)(ii / n), c = (int)(ii % n);
      const int pj = perm[j];
      Bn[ii] = (pj >= 0 && pj < nv) ? cconj(V[(int64_t)c * ell + pj]) : czero<CX>();
    }
  }
}

// Singular values of each gate of the last run, descending: out[g][t] =
// sqrt(sigma^2_t) for the values the run computed (t < nvec, every ell in the
// identity mode), zero beyond them, `count` entries per gate.  A gate that
// failed (status other than OK / RANK) reports zeros.
__global__ void spectra_kernel(const int64_t* __restrict__ desc, const char* ws, int esz, int count,
                               double* __restrict__ out) {
  const int g = blockIdx.y;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= count) return;
  const int64_t* D = desc + (int64_t)g * AGB_D_NFIELDS;
  const int chiL = (int)D[AGB_D_CHIL], chiR = (int)D[AGB_D_CHIR], ell = (int)D[AGB_D_ELL];
  const int st = (int)D[AGB_D_STATUS];
  const HeevdProb* hp = (const HeevdProb*)ws;
  const int nv = (D[AGB_D_MODE] == 1) ? ell : min(hp[g].nvec, ell);
  double v = 0.0;
  if ((st == AGB_OK || st == AGB_ERR_RANK) && t < nv) {
    const Slab Ls = slab_layout(2 * chiL, 2 * chiR, ell, esz);
    const double s2 = ((const double*)(ws + D[AGB_D_WS] + Ls.sig2))[t];
    v = s2 > 0.0 ? sqrt(s2) : 0.0;
  }
  out[(int64_t)g * count + t] = v;
}

// Repair pass (on the device, no host round trip): a gate whose eigenvector
// phase was cut short by the eigenvalue-guided count (AGB_ERR_RANK with
// nvec < ell), or whose eigenvectors failed the orthogonality guard (then with
// the wide cluster tolerance), runs its vector phase, X*V and rank selection
// again with every vector; every other gate is skipped by those launches.
__global__ void repair_setup_kernel(int64_t* __restrict__ desc, int ng, char* ws, int guard) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= ng) return;
  int64_t* D = desc + (int64_t)g * AGB_D_NFIELDS;
  HeevdProb* hp = (HeevdProb*)ws;
  GemmProb* gp = (GemmProb*)(ws + agb_align((size_t)ng * sizeof(HeevdProb)));
  const int ell = (int)D[AGB_D_ELL];
  const int st = (int)D[AGB_D_STATUS];
  const bool short_count = st == AGB_ERR_RANK && hp[g].nvec < ell && D[AGB_D_MODE] == 0;
  const bool overlap =
      guard && orth_exceeds(hp[g].orth_max2) && D[AGB_D_MODE] == 0 && (st == AGB_OK || st == AGB_ERR_RANK);
  if (short_count || overlap) {
    hp[g].redo = 1;
    hp[g].nvec = ell;
    hp[g].skip_vectors = 0;
    if (overlap) hp[g].ctol = kClusterTolWide;
    gp[3 * ng + g].N = ell;
    gp[3 * ng + g].M = 2 * (int)D[AGB_D_CHIL];
    D[AGB_D_STATUS] = AGB_OK;
    D[AGB_D_REPAIR] = (short_count ? 1 : 0) | (overlap ? 2 : 0);
  } else {
    hp[g].redo = 0;
    hp[g].skip_vectors = 1;
    gp[3 * ng + g].M = 0;
  }
}

template <typename CX>
int run_impl(int ng, int64_t* desc, int maxL, int maxM, int maxR, int maxell, char* ws, size_t ws_bytes,
             size_t tc_bytes, cudaStream_t s, int flags) {
  const int esz = sizeof(CX);
  if (cudaMemsetAsync(status_word(ws, ng), 0, sizeof(int), s) != cudaSuccess) return AGB_ERR_CUDA;
  prof_mark(AGB_ST_SETUP, s);
  setup_kernel<<<(ng + 127) / 128, 128, 0, s>>>(desc, ng, ws, esz);
  AGB_CHECK_LAUNCH();
  HeevdProb* hp = (HeevdProb*)ws;
  GemmProb* gp = (GemmProb*)(ws + agb_align((size_t)ng * sizeof(HeevdProb)));
  ContractProb* cp = (ContractProb*)(ws + agb_align((size_t)ng * sizeof(HeevdProb)) +
                                     agb_align((size_t)ng * 4 * sizeof(GemmProb)));
  ContractProb none = {};
  prof_mark(AGB_ST_CONTRACT, s);
  contract_gate_kernel<CX><<<dim3((maxR + 15) / 16, (maxL + 15) / 16, ng), 256, 0, s>>>(cp, none);
  AGB_CHECK_LAUNCH();
  const int maxm = 2 * maxL, maxn = 2 * maxR;
  GemmCtx ctx;
  ctx.tc_bytes = tc_bytes;
  ctx.tc_scratch = tc_bytes ? ws + ws_bytes - tc_bytes : nullptr;
  ctx.status = status_word(ws, ng);
  prof_mark(AGB_ST_GRAM, s);
  int rc = launch_gemm_probs<CX>(gp + 2 * ng, ng, maxn, maxn, s, &ctx, maxm);
  if (rc) return rc;
  rc = launch_heevd_values<CX>(hp, ng, maxn, maxell, s);
  if (rc) return rc;
  prerank_kernel<CX><<<ng, 512, 0, s>>>(desc, ng, ws);
  AGB_CHECK_LAUNCH();
  rc = launch_heevd_vectors<CX>(hp, gp, ng, maxn, maxell, s, &ctx);
  if (rc) return rc;
  prof_mark(AGB_ST_AV, s);
  rc = launch_gemm_probs<CX>(gp + 3 * ng, ng, maxm, maxell, s, &ctx, maxn);
  if (rc) return rc;
  prof_mark(AGB_ST_RANK, s);
  const int guard = (flags & AGB_RUN_NO_GUARD) ? 0 : 1;
  rank_kernel<CX><<<ng, 1024, 4 * (size_t)maxell * sizeof(double), s>>>(desc, ng, ws,
                                                                          (flags & AGB_RUN_REPAIR) ? 0 : 2, guard);
  AGB_CHECK_LAUNCH();
  if (!(flags & AGB_RUN_REPAIR)) {
    prof_mark(AGB_ST_GAP, s);
    return AGB_OK;
  }
  // repair pass for gates whose guided eigenvector count was too small
  repair_setup_kernel<<<(ng + 127) / 128, 128, 0, s>>>(desc, ng, ws, guard);
  AGB_CHECK_LAUNCH();
  rc = launch_heevd_vectors<CX>(hp, gp, ng, maxn, maxell, s, &ctx);
  if (rc) return rc;
  prof_mark(AGB_ST_AV, s);
  rc = launch_gemm_probs<CX>(gp + 3 * ng, ng, maxm, maxell, s, &ctx, maxn);
  if (rc) return rc;
  prof_mark(AGB_ST_RANK, s);
  rank_kernel<CX><<<ng, 1024, 4 * (size_t)maxell * sizeof(double), s>>>(desc, ng, ws, 1, guard);
  AGB_CHECK_LAUNCH();
  prof_mark(AGB_ST_GAP, s);
  return AGB_OK;
}

}  // namespace

extern "C" int agb_version(void) { return 100; }

extern "C" int agb_contract_gate(int dtype, const void* A, const void* B, const void* U, void* X,
                                 int chiL, int chiM, int chiR, void* stream) {
  if (dtype != AGB_C64 && dtype != AGB_C128) return AGB_ERR_ARG;
  if (chiL <= 0 || chiM <= 0 || chiR <= 0 || !A || !B || !U || !X) return AGB_ERR_ARG;
  ContractProb p;
  p.A = A;
  p.B = B;
  p.U = U;
  p.X = X;
  p.chiL = chiL;
  p.chiM = chiM;
  p.chiR = chiR;
  p.ldx = 2 * (int64_t)chiR;
  cudaStream_t s = (cudaStream_t)stream;
  dim3 grid((chiR + 15) / 16, (chiL + 15) / 16, 1);
  if (dtype == AGB_C64) contract_gate_kernel<float2><<<grid, 256, 0, s>>>(nullptr, p);
  else contract_gate_kernel<double2><<<grid, 256, 0, s>>>(nullptr, p);
  AGB_CHECK_LAUNCH();
  return AGB_OK;
}

extern "C" int agb_two_site_plan(int dtype, int ng, int64_t* desc, size_t* ws_bytes) {
  if (dtype != AGB_C64 && dtype != AGB_C128) return AGB_ERR_ARG;
  if (ng < 0 || (ng > 0 && !desc) || !ws_bytes) return AGB_ERR_ARG;
  const int esz = dtype == AGB_C64 ? 8 : 16;
  size_t off = header_bytes(ng);
  for (int g = 0; g < ng; ++g) {
    int64_t* D = desc + (int64_t)g * AGB_D_NFIELDS;
    const int chiL = (int)D[AGB_D_CHIL], chiM = (int)D[AGB_D_CHIM], chiR = (int)D[AGB_D_CHIR];
    const int cap = (int)D[AGB_D_CAP];
    if (chiL <= 0 || chiM <= 0 || chiR <= 0 || cap <= 0) return AGB_ERR_ARG;
    const int m = 2 * chiL, n = 2 * chiR;
    if (n > 1024) return AGB_ERR_UNSUPPORTED;
    const int full = m < n ? (m < cap ? m : cap) : (n < cap ? n : cap);
    int ell = (int)D[AGB_D_ELL];
    if (ell <= 0 || ell > full) ell = full;
    D[AGB_D_ELL] = ell;
    if (D[AGB_D_DIMS]) {  // device-resident: the given shapes are capacities
      D[AGB_D_CAPL] = chiL;
      D[AGB_D_CAPM] = chiM;
      D[AGB_D_CAPR] = chiR;
      D[AGB_D_ELLPLAN] = ell;
    }
    D[AGB_D_WS] = (int64_t)off;
    off += agb_align(slab_layout(m, n, ell, esz).total);
  }
  int mL = 1, mR = 1, mE = 1;
  for (int g = 0; g < ng; ++g) {
    const int64_t* D = desc + (int64_t)g * AGB_D_NFIELDS;
    mL = (int)D[AGB_D_CHIL] > mL ? (int)D[AGB_D_CHIL] : mL;
    mR = (int)D[AGB_D_CHIR] > mR ? (int)D[AGB_D_CHIR] : mR;
    mE = (int)D[AGB_D_ELL] > mE ? (int)D[AGB_D_ELL] : mE;
  }
  *ws_bytes = off + tc_tail_bytes(dtype, ng, 2 * mL, 2 * mR, mE);
  return AGB_OK;
}

extern "C" int agb_two_site_run(int dtype, int ng, const int64_t* desc_dev, int64_t* desc_out,
                                int max_chiL, int max_chiM, int max_chiR, int max_ell, void* ws,
                                size_t ws_bytes, void* stream, int flags) {
  (void)max_chiM;
  (void)desc_dev;
  if (dtype != AGB_C64 && dtype != AGB_C128) return AGB_ERR_ARG;
  if (ng <= 0) return AGB_OK;
  if (!desc_out || !ws || max_chiL <= 0 || max_chiR <= 0 || max_ell <= 0) return AGB_ERR_ARG;
  if (2 * max_chiR > 1024 || max_ell > 1024) return AGB_ERR_UNSUPPORTED;
  if (ws_bytes < header_bytes(ng)) return AGB_ERR_WORKSPACE;
  const size_t tc = tc_tail_bytes(dtype, ng, 2 * max_chiL, 2 * max_chiR, max_ell);
  cudaStream_t s = (cudaStream_t)stream;
  if (dtype == AGB_C64)
    return run_impl<float2>(ng, desc_out, max_chiL, max_chiM, max_chiR, max_ell, (char*)ws, ws_bytes, tc, s, flags);
  return run_impl<double2>(ng, desc_out, max_chiL, max_chiM, max_chiR, max_ell, (char*)ws, ws_bytes, tc, s,
                           flags);
}

extern "C" int agb_two_site_finalize(int dtype, int ng, const int64_t* desc_dev, int max_chiL,
                                     int max_chiR, int max_k, void* ws, void* stream) {
  if (dtype != AGB_C64 && dtype != AGB_C128) return AGB_ERR_ARG;
  if (ng <= 0) return AGB_OK;
  if (!desc_dev || !ws) return AGB_ERR_ARG;
  const int64_t tot = (int64_t)2 * max_chiL * max_k + (int64_t)max_k * 2 * max_chiR;
  int blocks = (int)((tot + 255) / 256);
  if (blocks < 1) blocks = 1;
  if (blocks > 4096) blocks = 4096;
  cudaStream_t s = (cudaStream_t)stream;
  prof_mark(AGB_ST_SCATTER, s);
  if (dtype == AGB_C64) scatter_kernel<float2><<<dim3(blocks, ng), 256, 0, s>>>(desc_dev, (char*)ws);
  else scatter_kernel<double2><<<dim3(blocks, ng), 256, 0, s>>>(desc_dev, (char*)ws);
  AGB_CHECK_LAUNCH();
  prof_mark(AGB_ST_GAP, s);
  return AGB_OK;
}

extern "C" int agb_two_site_spectra(int dtype, int ng, const int64_t* desc_dev, const void* ws, int count,
                                    double* out, void* stream) {
  if (dtype != AGB_C64 && dtype != AGB_C128) return AGB_ERR_ARG;
  if (ng < 0 || count < 0) return AGB_ERR_ARG;
  if (ng == 0 || count == 0) return AGB_OK;
  if (!desc_dev || !ws || !out || ng > 65535) return AGB_ERR_ARG;
  const int esz = dtype == AGB_C64 ? 8 : 16;
  spectra_kernel<<<dim3((count + 127) / 128, ng), 128, 0, (cudaStream_t)stream>>>(desc_dev, (const char*)ws, esz,
                                                                                 count, out);
  AGB_CHECK_LAUNCH();
  return AGB_OK;
}
