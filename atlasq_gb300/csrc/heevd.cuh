// Batched Hermitian eigensolver (top-`ell` eigenpairs, descending) for sm_103a.
//
// Stages (one problem per batch entry):
//   1. tridiag:   Householder reduction H = Q T Q^H (LAPACK zhetd2 formulation:
//                 real symmetric tridiagonal T, complex tau, reflector vectors
//                 stored in the rows of H).  H is first scaled by 1/max|H_ii|.
//   2. bisect:    32-way multisection on Sturm counts for the top `ell`
//                 eigenvalues (one warp per eigenvalue).
//   3. invit:     inverse iteration on T - lambda I (tridiagonal LU with
//                 partial pivoting, Philox start vector, 3 solves); one thread
//                 per eigenvector.
//   4. cluster:   modified Gram-Schmidt (twice) inside tight eigenvalue clusters.
//   5. backtrans: V = Q Y by applying the reflectors in reverse order.
//   6. polish:    two Newton-Schulz steps V <- V (3I - V^H V) / 2 (GEMMs) so V
//                 is orthonormal to working precision.
#pragma once
#include "gemm.cuh"

// Eigenvalues closer than kClusterTol * max|lambda| are solved as a cluster
// (re-orthogonalised inverse iteration, LAPACK stein's scheme); wider gaps
// leave inverse-iteration vectors within ~(bisection error / gap)^3 of
// orthogonal, which the Newton-Schulz polish removes.  The first polish
// product V^H V is checked over the eigenvectors above the Gram's float32
// floor (the orthogonality guard):
//  * an overlap above kOrthPolish gets two more polish steps (two steps take
//    an overlap d to ~0.42 d^4, so four reach float32 orthonormality from
//    below kOrthGuard).  Measured: on flat spectra (64-qubit HEA, chi 512)
//    2% of gates show overlaps between 1e-2 and 0.29, and the polished
//    factors reproduce X to the optimal truncation error;
//  * an overlap above kOrthGuard marks vectors that converged onto the same
//    eigenvector (measured: 0.48-0.56 when a zero pivot of the Sturm count was
//    mis-ordered): the polish cannot restore the missing direction, so the
//    problem's vector phase is re-run with the wider kClusterTolWide (the
//    repair pass of the two-site pipeline).  On the 64-qubit HEA (chi 512)
//    18% of gates exceeded it while cluster shifts were walked apart
//    (member_shift in heevd.cu has why); since, none of 3 024 in the first
//    pass.
// On dense spectra of large Gram matrices (n >= 512) a wide tolerance chains
// hundreds of eigenvalues into one cluster, so it is only a repair setting.
constexpr double kClusterTol = 1e-5;
constexpr double kClusterTolWide = 1e-2;
constexpr float kOrthPolish = 1e-2f;
constexpr float kOrthGuard = 0.3f;
AGB_HD bool orth_above(unsigned max2_bits, float limit) {
  union {
    unsigned u;
    float f;
  } c;
  c.u = max2_bits;
  return !(c.f <= limit * limit);  // NaN / inf included
}
AGB_HD bool orth_exceeds(unsigned max2_bits) { return orth_above(max2_bits, kOrthGuard); }

struct HeevdProb {
  void* H;       // CX[n x ldh], Hermitian input, overwritten by the reduction
  int64_t ldh;
  int n, ell;
  void* d;       // R[n]
  void* e;       // R[n]
  void* tau;     // CX[n]
  void* lam;     // R[ell]   eigenvalues of H / scale, descending
  void* Y;       // R[n*ell] tridiagonal eigenvectors, element (i, t) at i*ell + t
  void* lu;      // R[5*n*ell] inverse-iteration LU factors (interleaved)
  void* V;       // CX[n*ldv] eigenvectors of H, element (i, t) at i*ldv + t
  int64_t ldv;
  void* V2;      // CX[n*ell] polish scratch
  void* M;       // CX[ell*ell] polish scratch
  void* scale;   // R[1] scale applied to H (eigenvalues of H = lam * scale)
  uint64_t seed;
  int skip_vectors;  // set by the caller between the two phases: no eigenvectors needed
  int nvec;          // eigenvectors to compute (the leading nvec of the ell eigenvalues), <= ell;
                     // may be lowered between the two phases; strides stay ell
  int redo;          // set by the two-site repair pass: this problem's vector phase runs again
  unsigned orth_max2;  // orthogonality guard: largest |(V^H V)_ij|^2 over the checked pairs (float bits)
  unsigned orth_w2;    // largest |(V^H V)_ij|^2 * lambda_i / lambda_0 (i > j) over the same pairs (float bits)
  double ctol;       // cluster tolerance relative to max|lambda| (kClusterTol unless repaired)
  void* band;        // scratch of the two-stage tridiagonalisation (block-reflector factors,
                     // exchange rows, band-stage reflectors), tridiag_2stage.cu
  int fail;          // set when a bounded wait of the band stage expired
};

// Bytes of the two-stage scratch for an n x n problem (the larger of the band
// widths the launcher may choose).
AGB_HD size_t two_stage_scratch_bytes(int esz, int n) {
  size_t best = 0;
  for (int bw = 8; bw <= 16; bw *= 2) {
    const size_t np = (size_t)(n + bw - 1) / bw;
    const size_t km = (size_t)((n - 1 + bw - 1) / bw > 0 ? (n - 1 + bw - 1) / bw : 1);
    const size_t b = agb_align(np * bw * bw * esz) + agb_align((size_t)n * bw * esz) +
                     agb_align((size_t)n * km * bw * esz) + agb_align((size_t)n * km * esz);
    if (b > best) best = b;
  }
  return best;
}

// Bytes of per-problem scratch (d, e, tau, lam, Y, lu, V2, M, scale) for one
// problem of size n with ell eigenpairs; V and H are not included.
// Fill scratch pointers of `p` from a scratch base pointer.
void heevd_assign_scratch(HeevdProb& p, char* base, int esz);
AGB_HD void heevd_assign_scratch_dev(HeevdProb& p, char* base, int esz) {
  const int rsz = esz / 2;
  const size_t n = p.n, ell = p.ell;
  size_t o = 0;
  p.d = base + o;     o += agb_align(n * rsz);
  p.e = base + o;     o += agb_align(n * rsz);
  p.tau = base + o;   o += agb_align(n * esz);
  p.lam = base + o;   o += agb_align(ell * rsz);
  p.Y = base + o;     o += agb_align(n * ell * rsz);
  p.lu = base + o;    o += agb_align(5 * n * ell * rsz);
  p.V2 = base + o;    o += agb_align(n * ell * esz);
  p.M = base + o;     o += agb_align(ell * ell * esz);
  p.scale = base + o; o += agb_align(rsz);
  p.band = base + o;  o += agb_align(two_stage_scratch_bytes(esz, p.n));
}

AGB_HD size_t heevd_scratch_bytes(int esz, int n, int ell) {
  const int rsz = esz / 2;
  const size_t N = n, L = ell;
  return agb_align(N * rsz) * 2 + agb_align(N * esz) + agb_align(L * rsz) + agb_align(N * L * rsz) +
         agb_align(5 * N * L * rsz) + agb_align(N * L * esz) + agb_align(L * L * esz) + agb_align(rsz) +
         agb_align(two_stage_scratch_bytes(esz, n));
}



// Two-stage tridiagonalisation (tridiag_2stage.cu): band width for a batch
// (0 = not applicable), stage 1 + 2, and the matching back-transformation.
int two_stage_bw(int esz, int maxn);
template <typename CX>
int launch_two_stage(HeevdProb* probs, int count, int maxn, cudaStream_t s);
template <typename CX>
int launch_bt_two_stage(const HeevdProb* probs, int count, int maxn, int maxell, cudaStream_t s);
// 0: two-stage where it applies, 1 (default): always the one-stage kernels.
int tridiag_stages_mode();

// Cluster (distributed shared memory) tridiagonalisation, tridiag_cluster.cu.
size_t tridiag_cluster_smem(int esz, int n, int C);
int tridiag_cluster_size(int esz, int n);
template <typename CX>
int launch_tridiag_cluster(const HeevdProb* probs, int count, int maxn, cudaStream_t s);

// Launch all stages.  `probs` is a device array of `count` problems with
// n <= maxn and ell <= maxell; `gemm_scratch` holds 4*count GemmProb entries.
template <typename CX>
int launch_heevd(HeevdProb* probs, GemmProb* gemm_scratch, int count, int maxn, int maxell,
                 cudaStream_t s);
// The same work in two phases: eigenvalues (tridiag + bisect), then
// eigenvectors (inverse iteration, clusters, back-transform, polish) for the
// problems whose skip_vectors flag is 0.
template <typename CX>
int launch_heevd_values(HeevdProb* probs, int count, int maxn, int maxell, cudaStream_t s);
template <typename CX>
int launch_heevd_vectors(HeevdProb* probs, GemmProb* gemm_scratch, int count, int maxn, int maxell,
                         cudaStream_t s, const GemmCtx* ctx = nullptr);
