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


def _sturm_count_late_replacement(d, e, x):
    """The former kernel order: a pivot is counted first and replaced by
    -pivmin only when the next step divides by it."""
    x = np.float32(x)
    q = d[0] - x
    c = int(q < 0)
    for k in range(1, len(d)):
        if abs(q) < np.float32(1e-30):
            q = np.float32(-1e-30)
        q = d[k] - x - (e[k - 1] * e[k - 1]) / q
        c += int(q < 0)
    return c


def test_sturm_count_with_a_pivot_that_cancels_to_zero():
    """T - 2I has a leading 2 x 2 block that is exactly singular in float32
    (pivots 1, then 0.5625 - 0.5625 = 0).  Counting that zero pivot before
    replacing it by -pivmin (the kernel's order, LAPACK dlaebz's) gives the
    exact count of eigenvalues below 2; counting it as non-negative and
    replacing it only at the next division loses one.  That lost count made
    the bisection return a leading eigenvalue midway between two neighbours
    1.6e-5 apart, and inverse iteration then produced overlapping vectors."""
    d = np.array([3.0, 2.5625, 2.0], dtype=np.float32)
    e = np.array([0.75, 0.5, 0.0], dtype=np.float32)
    T = np.diag(d.astype(np.float64)) + np.diag(e[:2].astype(np.float64), 1) + np.diag(e[:2].astype(np.float64), -1)
    exact = int(np.sum(np.linalg.eigvalsh(T) < 2.0))
    assert exact == 1
    assert fm._sturm(d, e, 2.0) == exact
    assert _sturm_count_late_replacement(d, e, 2.0) == exact - 1
