"""Capture of tests/golden/collapse_case.npz (needs a GB300; not run by the tests).

The fixture is the input of one two-site update (site tensors A [29,2,26],
B [26,2,28] and the gate U, bond 8 of a 16-qubit chain, chi_max 128,
eps 1e-3) whose X = U (A B), 58 x 56, has ten leading eigenvalues of X^H X
only 1e-5..4e-5 apart (relative).  With the eigensolver's former 1e-5 cluster
tolerance, 78% of the inverse-iteration starting vectors lost one of those
leading directions (relative reconstruction error 0.26 instead of the 7e-4 of
the truncation).

It came up as the gate a rank-predictor run re-ran at full size: a predictor
trained as in tests/test_rank_predictor.py sizes the eigensolver for a
Trotter-Ising circuit (seed 11), and this script keeps the input of the first
gate that falls back.  The predictor's training uses float atomics, so not
every training leads to a fallback; the script retrains until one does.

    python tests/golden/capture_collapse_case.py
"""
import os
import sys

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import atlasq_gb300 as aq  # noqa: E402
import atlasq_gb300.adaptive_mps as amod  # noqa: E402
from atlasq_gb300.circuits import trotter_ising  # noqa: E402
from atlasq_gb300.rank_predictor import RankPredictor, collect_training_data  # noqa: E402


def main(attempts=6):
    n, chi, eps, steps, dtr = 16, 128, 1e-3, 20, (0.05, 0.25)
    circ = lambda sd: trotter_ising(n, steps, sd, dt_range=dtr)  # noqa: E731
    X, T = collect_training_data(circ, range(6), n, chi, eps)
    ops = circ(11)
    orig = amod._run_pipeline
    captured = []

    def spy(entries, dt, ells, all_vectors=False):
        if all_vectors and not captured:
            m, i, U = entries[0]
            captured.append((i, m._tensors[i].detach().cpu(), m._tensors[i + 1].detach().cpu(), U.detach().cpu()))
        return orig(entries, dt, ells, all_vectors)

    amod._run_pipeline = spy
    try:
        for _ in range(attempts):
            rp = RankPredictor(seed=0)
            rp.train(X, T, steps=600, batch=512, lr=3e-3)
            m = aq.AdaptiveMPS(n, bond_dim=1, eps_bond=eps, chi_max_per_bond=chi, device="cuda")
            m.rank_predictor = rp
            for kind, q, U in ops:
                (m.apply_two_site_gate if kind == "2q" else m.apply_single_qubit_gate)(q, U)
            m.flush()
            if captured:
                break
    finally:
        amod._run_pipeline = orig
    if not captured:
        raise SystemExit("no rank fallback in any attempt")
    i, A, B, U = captured[0]
    np.savez_compressed(os.path.join(HERE, "collapse_case.npz"), A=A.numpy(), B=B.numpy(), U=U.numpy(),
                        bond=np.int64(i), n_qubits=np.int64(n), chi_max=np.int64(chi), eps=np.float64(eps))
    print("saved bond", i, tuple(A.shape), tuple(B.shape))


if __name__ == "__main__":
    main()
