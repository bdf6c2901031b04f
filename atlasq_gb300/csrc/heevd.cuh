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

// Eigenvalues closer than cluster_tol_rel(n) * max|lambda| are solved as a
// cluster (re-orthogonalised inverse iteration); wider gaps leave
// inverse-iteration vectors close enough to orthogonal for the Newton-Schulz
// polish.  Measured on a Trotter-Ising two-site update (58 x 56, ten leading
// eigenvalues 1e-5..4e-5 apart): at 1e-5, two vectors collapsed onto one
// direction for 78% of random starts, dropping a leading singular vector
// (relative error 0.26); at 1e-4, 3 of 400 starts; at 1e-3 (LAPACK stein's
// ortol) none.  On the dense spectra of large Gram matrices (n >= 512) gaps
// below 1e-4 chain into clusters of hundreds of members, which makes the
// cluster stage several times slower, so those keep 1e-5 (with the remaining
// risk described in the design notes).
AGB_HD double cluster_tol_rel(int n) { return n <= 256 ? 1e-3 : 1e-5; }

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
};

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
}

AGB_HD size_t heevd_scratch_bytes(int esz, int n, int ell) {
  const int rsz = esz / 2;
  const size_t N = n, L = ell;
  return agb_align(N * rsz) * 2 + agb_align(N * esz) + agb_align(L * rsz) + agb_align(N * L * rsz) +
         agb_align(5 * N * L * rsz) + agb_align(N * L * esz) + agb_align(L * L * esz) + agb_align(rsz);
}



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
