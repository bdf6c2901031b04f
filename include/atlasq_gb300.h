/*
 * atlasq_gb300 -- C ABI of the GB300 (sm_103a) MPS circuit-simulation hot path.
 *
 * Drop-in boundary for the matrix-product-state path of ATLAS-Q
 * (followthesapper/ATLAS-Q 0.7.0).  Every entry point takes plain device
 * pointers, sizes and a CUDA stream (as void*), never allocates or frees, and
 * returns an int status (AGB_OK == 0).  Complex numbers are interleaved
 * (re, im) pairs: complex64 = two floats, complex128 = two doubles -- the same
 * memory layout as torch.complex64 / torch.complex128 tensors.  Site tensors are
 * contiguous row-major [chiL, 2, chiR].
 *
 * Each entry point names the reference interface it replaces (file:line,
 * relative to the reference project root).
 */
#ifndef ATLASQ_GB300_H
#define ATLASQ_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ status */
#define AGB_OK 0
#define AGB_ERR_ARG 1          /* bad shape / argument (reference: assert / ValueError) */
#define AGB_ERR_WORKSPACE 2    /* workspace smaller than the planned size */
#define AGB_ERR_NOCONV 3       /* eigensolver residual check failed */
#define AGB_ERR_TIMEOUT 4      /* a bounded device-side wait expired */
#define AGB_ERR_CUDA 5         /* CUDA launch / runtime error */
#define AGB_ERR_UNSUPPORTED 6  /* size or mode not supported by this build */
#define AGB_ERR_RANK 7         /* eigenpairs computed < rank required (caller re-plans) */
#define AGB_ERR_TOO_LARGE 8    /* problem exceeds the fixed scratch of agb_qr_noalloc */

/* dtype codes */
#define AGB_C64 0
#define AGB_C128 1

/* ---------------------------------------------------- two-site descriptor
 * One row of int64 fields per two-site gate of a batch.  Pointers are device
 * addresses stored as int64; reals are stored as the bits of an IEEE double.
 * Fields marked (in) are filled by the caller, (plan) by agb_two_site_plan,
 * (out) by the device.
 */
enum agb_desc_field {
  AGB_D_A = 0,        /* (in)  const site tensor i   [chiL,2,chiM]            */
  AGB_D_B = 1,        /* (in)  const site tensor i+1 [chiM,2,chiR]            */
  AGB_D_U = 2,        /* (in)  const gate [4,4] row-major, same dtype          */
  AGB_D_CHIL = 3,     /* (in)                                                  */
  AGB_D_CHIM = 4,     /* (in)                                                  */
  AGB_D_CHIR = 5,     /* (in)                                                  */
  AGB_D_CAP = 6,      /* (in)  chi_max for this bond                           */
  AGB_D_EPS = 7,      /* (in)  eps_bond (double bits)                          */
  AGB_D_ANEW = 8,     /* (in, finalize) output site i   [chiL,2,k]             */
  AGB_D_BNEW = 9,     /* (in, finalize) output site i+1 [k,2,chiR]             */
  AGB_D_ELL = 10,     /* (in)  eigenpairs to compute; 0 = min(2chiR, cap)      */
  AGB_D_SEED = 11,    /* (in)  Philox seed for start vectors                   */
  AGB_D_WS = 12,      /* (plan) byte offset of this gate's workspace slab      */
  AGB_D_CTOL = 13,    /* (in)  eigenvalue cluster tolerance relative to the largest
                       *       eigenvalue (double bits); 0 = the default 1e-5     */
  AGB_D_ORTH = 14,    /* (out) largest |(V^H V)_ij|^2, i != j, before the polish, over
                       *       eigenvectors above the Gram's float floor (double bits) */
  AGB_D_ORTHW = 15,   /* (out) the same pairs weighted by lambda_i / lambda_0 of the
                       *       smaller eigenvalue (double bits)                    */
  AGB_D_K = 16,       /* (out) kept rank                                       */
  AGB_D_EPSLOC = 17,  /* (out) eps_local (double bits)                         */
  AGB_D_ENTROPY = 18, /* (out) entropy in nats (double bits)                   */
  AGB_D_CONDS = 19,   /* (out) sigma_0 / sigma_{k-1} (double bits)             */
  AGB_D_STATUS = 20,  /* (out) per-gate status                                 */
  AGB_D_TOTAL = 21,   /* (out) ||X||_F^2 (double bits)                         */
  AGB_D_NEEDED = 22,  /* (out) eigenpairs actually required (fallback sizing)   */
  AGB_D_MODE = 23,    /* (out) 1: nothing truncated and m >= n, so A_new = X, B_new = I */
  /* Device-resident MPS (optional).  With DIMS set, CHIL/CHIM/CHIR given to the
   * plan are CAPACITIES; at run time the device reads the shapes from the
   * instance's int32 bond-dimension array (site s is [dims[s], 2, dims[s+1]]),
   * rewrites CHIL/CHIM/CHIR/ELL with them, and finalize writes dims[BOND+1] = k.
   * A, B, ANEW, BNEW are then the capacity buffers of sites BOND, BOND+1
   * (updated in place).  No host synchronisation is needed between batches, and
   * a launch sequence over such descriptors can be captured and replayed. */
  AGB_D_DIMS = 24,    /* (in)  int32* bond-dimension array, or 0              */
  AGB_D_BOND = 25,    /* (in)  bond index i (with DIMS)                        */
  AGB_D_CAPL = 26,    /* (plan) capacities recorded by the plan (with DIMS)    */
  AGB_D_CAPM = 27,
  AGB_D_CAPR = 28,
  AGB_D_ELLPLAN = 29, /* (plan) planned eigenpair count (with DIMS)            */
  AGB_D_NVEC = 30,    /* (in)  0: eigenvectors only for the values the rank rule can
                       *       keep (from the eigenvalues, plus a pad); -1: all ell */
  AGB_D_REPAIR = 31,  /* (out) vector phase re-run on the device: bit 0 the guided
                       *       count fell short, bit 1 the eigenvectors failed the
                       *       orthogonality guard (re-run with tolerance 1e-2)   */
  AGB_D_NFIELDS = 32
};

/* Version / build information. */
int agb_version(void);

/* (a2) Fused contraction + two-qubit gate.
 * Replaces fused_two_qubit_gate_pytorch (src/triton_kernels/mps_complex.py:343-368)
 * and its Triton twin (mps_complex.py:221-336).
 * X[(l,p),(q,j)] = sum_{p'q'} U[2p+q, 2p'+q'] sum_r A[l,p',r] B[r,q',j];
 * X is row-major [2chiL, 2chiR]. */
int agb_contract_gate(int dtype, const void* A, const void* B, const void* U, void* X, int chiL,
                      int chiM, int chiR, void* stream);

/* (a1) Two-site update, batched over gates on disjoint bonds.
 * Replaces AdaptiveMPS.apply_two_site_gate (src/atlas_q/adaptive_mps.py:182-308)
 * together with robust_svd (src/atlas_q/linalg_robust.py:17-52) and
 * choose_rank_from_sigma (src/atlas_q/truncation.py:21-83).
 *
 * agb_two_site_plan   fills AGB_D_WS of every row of `desc_host` and returns the
 *                     workspace bytes needed (the caller allocates it).
 * agb_two_site_run    contraction -> Gram -> Hermitian eigensolver -> Rayleigh
 *                     singular values -> rank selection; writes the (out) fields
 *                     of `desc_dev` (device copy of the planned rows).
 * agb_two_site_finalize  writes A_new = X V_k (singular values absorbed left, as
 *                     adaptive_mps.py:281-285) and B_new = V_k^H into the
 *                     AGB_D_ANEW / AGB_D_BNEW buffers sized from AGB_D_K. */
int agb_two_site_plan(int dtype, int ngates, int64_t* desc_host, size_t* ws_bytes);
#define AGB_RUN_REPAIR 1 /* flags: re-run, on the device, the vector phase of gates whose
                          * eigenvalue-guided eigenvector count fell short (AGB_D_NVEC = 0)
                          * or whose eigenvectors overlap by more than 0.3 after the
                          * eigensolver (then with the cluster tolerance widened to 1e-2);
                          * without it such gates report AGB_ERR_RANK / AGB_ERR_NOCONV */
#define AGB_RUN_NO_GUARD 2 /* flags: measure the orthogonality guard (AGB_D_ORTH/ORTHW) but
                            * neither repair nor reject on it */
int agb_two_site_run(int dtype, int ngates, const int64_t* desc_dev, int64_t* desc_dev_out,
                     int max_chiL, int max_chiM, int max_chiR, int max_ell, void* ws, size_t ws_bytes,
                     void* stream, int flags);
int agb_two_site_finalize(int dtype, int ngates, const int64_t* desc_dev, int max_chiL, int max_chiR,
                          int max_k, void* ws, void* stream);

/* Singular values of every gate of the last agb_two_site_run on `ws` (read it
 * before the workspace is reused): out[g * count + t] = sigma_t (double,
 * descending) for the values the run computed, zero-padded to `count`.  The
 * spectrum behind robust_svd's S (src/atlas_q/linalg_robust.py:37) as the
 * reference's SVD-event records keep it (S_top128, src/atlas_q/tools_qih/tn_core.py:247-274). */
int agb_two_site_spectra(int dtype, int ngates, const int64_t* desc_dev, const void* ws, int count, double* out,
                         void* stream);

/* (a6) Single-qubit gate, applied as the reference does: T'[a,t,b] = sum_s U[s,t] T[a,s,b]
 * (U^T; src/atlas_q/adaptive_mps.py:159-180).  In place. */
int agb_single_qubit_gate(int dtype, void* T, const void* U, int chiL, int chiR, void* stream);

/* Queued single-qubit gates of many sites (and many MPS instances) in one launch,
 * same arithmetic per gate as agb_single_qubit_gate.  desc (device, int64):
 * [ngroups][5] = {T, chiL, chiR, first, count} followed by the gate pointers
 * (2x2 matrices of the tensor's type); group g applies gates first..first+count-1
 * to T in order.  Groups must name distinct tensors.  max_elems >= chiL*chiR of
 * every group.  ngroups <= 65535.  A device-resident tensor is given as
 * {T, -1, (int64)&dims[site], first, count}: its shape is read on the device. */
int agb_single_qubit_batch(int dtype, int ngroups, const int64_t* desc, int max_elems, void* stream);

/* Autotuning of the Householder tridiagonalisation (the eigensolver's first
 * stage): times every admissible thread-block-cluster size on `count`
 * synthetic Hermitian n x n problems and keeps the fastest for this size
 * (bucket of 32) and batch class (<= 8, <= 32, more problems per launch); later
 * launches of that shape use it.  Synchronises the stream.  Returns the chosen
 * size and its time per launch.  agb_tuned_tridiag_cluster reports the size
 * currently used for a shape. */
size_t agb_tune_tridiag_workspace(int dtype, int n, int count);
int agb_tune_tridiag(int dtype, int n, int count, void* ws, size_t ws_bytes, void* stream, int* best_C,
                     float* best_ms);
int agb_tuned_tridiag_cluster(int dtype, int n, int count);
/* Set the cluster size C (1..16) and threads per CTA (256 or 512) the
 * tridiagonalisation uses for this shape class, as agb_tune_tridiag would;
 * C = 0 restores the built-in choice.  AGB_ERR_UNSUPPORTED if the matrix does
 * not fit that cluster. */
int agb_set_tridiag_cluster(int dtype, int n, int count, int C, int threads);

/* Tridiagonalisation used by the eigensolver: 0 the two-stage reduction
 * (dense -> band of width 16 or 8 on a thread-block cluster, then bulge
 * chasing in shared memory) wherever its buffers fit, else the one-stage
 * kernel; 1 (default) the one-stage Householder kernel always.  Process-wide;
 * this build's own switch (no reference counterpart), for comparing the paths. */
int agb_set_tridiag_stages(int mode);

/* Hermitian eigensolver (batched), exposed for robust_svd / tests.
 * Replaces the torch.linalg.svd call inside robust_svd (linalg_robust.py:37) when
 * used as X -> Gram -> eigenpairs.  H: [batch, n, n] Hermitian (overwritten);
 * evals: [batch, ell] descending; evecs: [batch, n, ell] (column t = eigenvector t). */
size_t agb_heevd_workspace(int dtype, int n, int ell);
int agb_heevd(int dtype, int batch, int n, int ell, void* H, void* evals, void* evecs, void* ws,
              size_t ws_bytes, uint64_t seed, void* stream);

/* Householder QR of op(A) (M x N; transA = 1 reads a row-major N x M matrix
 * transposed).  Q: [M, min(M,N)], R: [min(M,N), N] upper triangular, or their
 * plain transposes when trans_out = 1.  Replaces robust_qr / torch.linalg.qr
 * (src/atlas_q/linalg_robust.py:55-76) in the canonical sweeps
 * (adaptive_mps.py:310-385, mps_pytorch.py:91-152). */
size_t agb_qr_workspace(int dtype, int M, int N);
int agb_qr(int dtype, const void* A, int M, int N, int transA, void* Q, void* R, int trans_out,
           void* ws, size_t ws_bytes, void* stream);

/* Allocation-free variant of agb_qr (no counterpart in the reference).
 * For callers that cannot allocate device memory -- e.g. a host runtime that
 * reaches this library only through the C ABI with device pointers handed to
 * it by the owner of the GPU memory.  Same arguments as agb_qr but no
 * workspace: it always runs the single-CTA Householder kernel, whose scratch
 * (the working copy of op(A), M*N elements; the reflector scalars,
 * min(M,N); the Q block, M*min(M,N); each rounded up to 256 bytes) lives in a
 * fixed device array of AGB_QR_NOALLOC_MAX_BYTES (8 MiB, held by every GPU
 * that loads the library) -- larger problems return AGB_ERR_TOO_LARGE.  For
 * M*N >= 4096, where agb_qr uses its blocked cluster kernels, the two agree
 * to rounding, not bit for bit.  The first call on a device looks up the
 * array's address (cudaGetSymbolAddress): make it before any stream capture.
 * All calls share the array, so calls that overlap on the GPU race;
 * serialise them.  Allocates nothing. */
#define AGB_QR_NOALLOC_MAX_BYTES (8u << 20)
int agb_qr_noalloc(int dtype, const void* A, int M, int N, int transA, void* Q, void* R, int trans_out,
                   void* stream);

/* (a9) One site of batched sequential-conditional sampling.
 * Replaces the per-site body of _batch_sweep_sample (src/atlas_q/mps_pytorch.py:282-352)
 * with torch.multinomial replaced by a Philox4x32-10 stream:
 * temp [shots, 2chiR] = L @ T.reshape(chiL, 2chiR) (computed by the caller);
 * outputs bits <<= 1 | outcome, L_new [shots, chiR] (may be NULL on the last site)
 * and optionally P(0) per shot (pz_out, double; may be NULL). */
int agb_sample_site(int dtype, const void* temp, int shots, int chiR, int site, uint64_t seed,
                    uint64_t shot_offset, int64_t* bits, void* Lnew, double* pz_out, void* stream);

/* (a10) MPO mixing step of the expectation sweep (src/atlas_q/mpo_ops.py:1132-1145):
 * N[R][a][t][B] = sum_{L,s} W[L][s][t][R] M[L][a][s][B]. */
int agb_mpo_mix(int dtype, const void* M, const void* W, void* N, int Lw, int Rw, int chiA, int chiB,
                void* stream);
/* (a10) The single-site form of the same mixing for a batch of `count` items, one
 * 2x2 operator each (W: count x 2 x 2, contiguous):
 * N[g][a][t][b] = sum_s W[g][s][t] M[g][a][s][b], M and N count x chiA x 2 x chiB.
 * The per-site einsum of expectation_value with a [1,2,2,1] MPO tensor
 * (src/atlas_q/mpo_ops.py:1145), batched over the observables of a sweep. */
int agb_site_mix(int dtype, const void* M, const void* W, void* N, int count, int chiA, int chiB, void* stream);
/* (f4) One site of apply_mpo_to_mps (src/atlas_q/mpo_ops.py:1034-1082, the
 * einsum "lstr, atb -> lasrb" at :1068): out[(l, a), s, (r, b)] =
 * sum_t W[l, s, t, r] A[a, t, b]; W [Dl, 2, 2, Dr] and A [chiA, 2, chiB] of the
 * same dtype, out [Dl * chiA, 2, Dr * chiB].  Also the site product of the
 * Pauli-exponential MPO (mpo_ops.py:1296-1358). */
int agb_mpo_apply_site(int dtype, const void* W, const void* A, void* out, int Dl, int Dr, int chiA, int chiB,
                       void* stream);
/* (f1) TDVP local step with the index pattern of tdvp_apply_local_H_optimized
 * (src/triton_kernels/tdvp_mpo_ops.py:89-106, einsum 'qli, lstn, isj, unj -> itj'):
 * H[i, t, j] = sum_{q,l,s,n,u} L[q, l, i] W[l, s, t, n] A[i, s, j] R[u, n, j]
 * with L [chiQ, Dl, chiI], W [Dl, 2, 2, Dn], A [chiI, 2, chiJ], R [chiU, Dn, chiJ],
 * H [chiI, 2, chiJ].  ws: agb_tdvp_local_h_workspace bytes. */
size_t agb_tdvp_local_h_workspace(int dtype, int Dl, int Dn, int chiI, int chiJ);
int agb_tdvp_local_h(int dtype, const void* L, const void* W, const void* A, const void* R, void* H, int chiQ,
                     int Dl, int chiI, int Dn, int chiU, int chiJ, void* ws, size_t ws_bytes, void* stream);
/* out2[0] + i out2[1] = sum_{r,c} E[r,c] Q[c,r]  (double accuracy; out2 is device memory). */
int agb_trace_prod(int dtype, const void* E, const void* Q, int n, double* out2, void* stream);

/* Where the most recent failed launch check of this library was, as
 * "file:line: cudaErrorName (description)"; empty if none (this build's own
 * diagnostics; the string is owned by the library). */
const char* agb_last_error(void);

/* Per-stage CUDA-event timer of the two-site pipeline (this build's own
 * instrumentation; no reference counterpart).  agb_prof_begin enables marks on
 * the launching stream (capacity = max marks); agb_prof_end disables them and
 * returns summed milliseconds and mark counts per stage id (16 entries):
 * 0 host gap, 1 setup, 2 contract, 3 gram, 4 tridiag, 5 bisect, 6 invit,
 * 7 cluster, 8 backtransform, 9 polish, 10 X*V, 11 rank, 12 scatter. */
int agb_prof_begin(int capacity);
/* Number of kernels this library has launched since it was loaded. */
long long agb_launch_count(void);
int agb_prof_end(double* ms_per_stage, int* marks_per_stage, int nstages);

/* (a14) Learned rank predictor: MLP 5 -> 64 -> 64 -> 64 -> 1 (ReLU hidden,
 * sigmoid output), FP32, parameters in one buffer of AGB_MLP_NPARAM floats
 * (W1[64][5] b1 W2[64][64] b2 W3[64][64] b3 W4[64] b4).  New in this build:
 * the reference's predictor (src/atlas_q/tools_qih/ai_rank_predictor.py:14-89)
 * reads singular values after the SVD; this one predicts the kept rank before
 * it from (chi_L, chi_R, entangling power, neighbouring-bond entropy, previous
 * rank).  X: [B][5] features, Y/T: [B] rank fraction in (0, 1).
 * agb_mlp_backward writes d mean((y-t)^2) / d params to `grads` and, if
 * loss_sum is not NULL, sum (y-t)^2 to *loss_sum; deterministic (fixed-order
 * reductions through ws, agb_mlp_backward_workspace(B) bytes).  agb_mlp_adam
 * is AdamW (step >= 1). */
#define AGB_MLP_NPARAM 8769
int agb_mlp_forward(const float* params, const float* X, int B, float* Y, void* stream);
size_t agb_mlp_backward_workspace(int B);
int agb_mlp_backward(const float* params, const float* X, const float* T, int B, float* grads, float* loss_sum,
                     void* ws, size_t ws_bytes, void* stream);
int agb_mlp_adam(float* params, const float* grads, float* m, float* v, int step, float lr, float beta1,
                 float beta2, float eps, float weight_decay, void* stream);

/* Batched complex64 GEMM on the tcgen05 tensor cores (3xTF32 split precision,
 * the split into TF32 planes done in shared memory inside the kernel), strided
 * batch: C[b] = alpha op(A[b]) op(B[b]) + beta C[b]; op is 'N', 'T', 'C' or 'R'
 * (conjugated, not transposed).
 * Replaces the torch/cuBLAS complex matmuls of the reference path
 * (mps_complex.py:359-366, mps_pytorch.py:300-352, mpo_ops.py:1145).
 * ws: agb_cgemm_tc_workspace(batch, M, N, K) bytes.  If status_host is not
 * NULL the call synchronises the stream and returns the device status
 * (AGB_ERR_TIMEOUT if a bounded wait expired). */
size_t agb_cgemm_tc_workspace(int batch, int M, int N, int K);
int agb_cgemm_tc(char opA, char opB, int batch, int M, int N, int K, const void* A, int64_t lda,
                 int64_t strideA, const void* B, int64_t ldb, int64_t strideB, void* C, int64_t ldc,
                 int64_t strideC, float alpha_re, float alpha_im, float beta_re, float beta_im, void* ws,
                 size_t ws_bytes, int* status_host, void* stream);
/* The same GEMM without any synchronisation: a bounded wait that expires sets
 * *status_dev (device memory) to AGB_ERR_TIMEOUT; the word is never cleared
 * by the library, so one read after a sequence of calls checks them all. */
int agb_cgemm_tc_async(char opA, char opB, int batch, int M, int N, int K, const void* A, int64_t lda,
                       int64_t strideA, const void* B, int64_t ldb, int64_t strideB, void* C, int64_t ldc,
                       int64_t strideC, float alpha_re, float alpha_im, float beta_re, float beta_im, void* ws,
                       size_t ws_bytes, int* status_dev, void* stream);

/* Poll limit of the tensor-core GEMM's pipeline waits (process-wide; a negative
 * value restores the default of 2^26 polls).  A test hook with no reference
 * counterpart: at 0 the waits expire at once, the kernel records
 * AGB_ERR_TIMEOUT, waits (full limit) for the MMAs it issued, frees its tensor
 * memory and returns; the context stays usable. */
int agb_set_gemm_wait_limit(long long polls);

/* Batched complex GEMM (SIMT reference-free kernel, used by the host layer):
 * C[b] = alpha * op(A[b]) op(B[b]) + beta * C[b]; op: 'N' (as stored), 'T' (transposed),
 * 'C' (conjugate-transposed), 'R' (conjugated, not transposed). */
int agb_cgemm_batched(int dtype, char opA, char opB, int batch, int M, int N, int K,
                      const void* A, int64_t lda, int64_t strideA, const void* B, int64_t ldb,
                      int64_t strideB, void* C, int64_t ldc, int64_t strideC, double alpha_re,
                      double alpha_im, double beta_re, double beta_im, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* ATLASQ_GB300_H */
