"""Randomized (sketch) truncation vs exact truncation on the 40-qubit Haar
brickwork (depth 20, chi_max 256, eps 1e-8), in complex128 on the CPU.

Design study, not test or product code: it measures what the sketch-based
factorisation (randomized range finder with oversampling p and q power
iterations, then an FP64 SVD of the projected l x n matrix) costs in accuracy
at the cap, given a PERFECT rank prediction (the sketch is sized from the
exact rule's k, the best a learned predictor can do).  Both states are
evolved side by side from |0...0>; printed per checkpoint gate:

* the discarded weight (fraction of each gate's sum of sigma^2 not kept),
  summed over the gates so far, of the sketch and of the exact truncation;
* the fidelity |<psi_sketch|psi_exact>|^2 of the two states.

    python oracle/sketch_study.py [p] [q] [seed]     (defaults 16 2 1234)
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

from oracle.mps_oracle import choose_rank_from_sigma, fused_two_qubit_gate, mps_fidelity  # noqa: E402

N, DEPTH, CHI, EPS = 40, 20, 256, 1e-8
CHECKPOINTS = (150, 250, 330, 390)


def _orth(Y):
    Q, _ = np.linalg.qr(Y)
    return Q


def sketch_factor(X, k, p, q, rng):
    """Rank-k factor (U_k S_k, Vh_k) of X from a Gaussian sketch of width
    k + p with q power iterations (re-orthonormalised each half step)."""
    m, n = X.shape
    ell = min(k + p, m, n)
    Om = (rng.standard_normal((n, ell)) + 1j * rng.standard_normal((n, ell))) / np.sqrt(2)
    Q = _orth(X @ Om)
    for _ in range(q):
        Q = _orth(X @ _orth(X.conj().T @ Q))
    Bm = Q.conj().T @ X                      # ell x n, the projected problem (FP64)
    Ub, S, Vh = np.linalg.svd(Bm, full_matrices=False)
    return (Q @ Ub[:, :k]) * S[:k], Vh[:k], S


def main():
    p = int(sys.argv[1]) if len(sys.argv) > 1 else 16
    q = int(sys.argv[2]) if len(sys.argv) > 2 else 2
    seed = int(sys.argv[3]) if len(sys.argv) > 3 else 1234
    sys.path.insert(0, os.path.dirname(HERE))
    from atlasq_gb300.circuits import haar_brickwork
    ops = haar_brickwork(N, DEPTH, seed=seed)
    rng = np.random.default_rng(seed + 7)

    def zero():
        ts = []
        for _ in range(N):
            t = np.zeros((1, 2, 1), dtype=np.complex128)
            t[0, 0, 0] = 1
            ts.append(t)
        return ts
    ex, sk = zero(), zero()
    disc_ex = disc_sk = 0.0
    for g, (_, i, U) in enumerate(ops, start=1):
        U = U.numpy().astype(np.complex128)
        # exact truncation
        A, B = ex[i], ex[i + 1]
        X = fused_two_qubit_gate(A, B, U)
        Uu, S, Vh = np.linalg.svd(X, full_matrices=False)
        k = choose_rank_from_sigma(S, EPS, CHI)[0]
        disc_ex += float(np.sum(S[k:] ** 2) / np.sum(S ** 2))
        ex[i] = (Uu[:, :k] * S[:k]).reshape(A.shape[0], 2, k)
        ex[i + 1] = Vh[:k].reshape(k, 2, B.shape[2])
        # sketch, sized from the exact rule's rank on the sketch state's own X
        A, B = sk[i], sk[i + 1]
        X = fused_two_qubit_gate(A, B, U)
        S_full = np.linalg.svd(X, compute_uv=False)
        k = choose_rank_from_sigma(S_full, EPS, CHI)[0]
        US, Vk, _ = sketch_factor(X, k, p, q, rng)
        kept = float(np.linalg.norm(US) ** 2)
        disc_sk += max(0.0, 1.0 - kept / float(np.sum(S_full ** 2)))
        sk[i] = US.reshape(A.shape[0], 2, k)
        sk[i + 1] = Vk.reshape(k, 2, B.shape[2])
        if g in CHECKPOINTS:
            f = mps_fidelity(sk, ex)
            print(f"p={p} q={q} gate {g}: discarded weight (sum over gates) sketch {disc_sk:.6g}, exact "
                  f"{disc_ex:.6g}, fidelity(sketch, exact) {f:.6f}", flush=True)


if __name__ == "__main__":
    main()
