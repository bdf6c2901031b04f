"""The float32 model of the eigensolver stages (tests/f32_eigensolver_model.py)
on the captured near-degenerate case: the algorithm itself separates the ten
leading eigenvectors, whose gaps are 1e-5..4e-5 of lambda_0, for every start."""
import numpy as np

from conftest import load_golden
import f32_eigensolver_model as fm


def _gram():
    g = load_golden("collapse_case")
    A, B, U = (g[k].astype(np.complex128) for k in ("A", "B", "U"))
    th = np.einsum("apm,mqb->apqb", A, B)
    X = np.einsum("PQpq,apqb->aPQb", U.reshape(2, 2, 2, 2), th).reshape(2 * A.shape[0], 2 * B.shape[2])
    X32 = X.astype(np.complex64)
    return (X32.conj().T @ X32).astype(np.complex64)


def test_model_eigenvalues_and_separated_leading_group():
    G = _gram()
    d, e = fm.tridiagonalize(G)
    mx = np.abs(np.real(np.diag(G))).max()
    exact = np.linalg.eigvalsh(G.astype(np.complex128) / mx)[::-1]
    lam = np.array([fm.bisect(d, e, t) for t in range(10)])
    assert np.max(np.abs(lam - exact[:10])) < 1e-6 * exact[0]
    gaps = -np.diff(exact[:10]) / exact[0]
    assert gaps.max() < 2e-4 and gaps.min() < 2e-5  # the near-degenerate group
    for seed in range(5):
        rng = np.random.default_rng(seed)
        Y = np.stack([fm.inverse_iteration(d, e, lam[t], rng) for t in range(10)], axis=1).astype(np.float64)
        assert np.linalg.svd(Y, compute_uv=False).min() > 0.9
        assert np.max(np.abs(Y.T @ Y - np.eye(10))) < 0.1
