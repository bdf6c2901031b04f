"""A NumPy float32 model of the library's Hermitian eigensolver stages, for
comparing the GPU kernels stage by stage (test infrastructure only).

It restates, with the kernels' own formulas and tolerances:
* the Householder reduction to real tridiagonal form of the scaled matrix
  (zhetd2-style, lower: beta = -sign(Re alpha) ||x||, tau, v = x / (alpha - beta),
  w = p + K v, rank-2 update), in complex64;
* the 32-way multisection on Sturm counts with the kernel's tolerance
  2 eps max(|lo|, |hi|) from the Gershgorin interval;
* inverse iteration: LU with partial pivoting of T - lambda I (rows with up to
  two superdiagonals, zero and tiny pivots floored at eps ||T||), three
  solves from a random start, renormalised before each.
"""
import numpy as np

EPS = np.float32(np.finfo(np.float32).eps)


def tridiagonalize(G):
    """Hermitian G (complex) -> (d, e) float32, T similar to G / max|Re diag|."""
    n = G.shape[0]
    mx = np.float32(np.abs(np.real(np.diag(G))).max()) or np.float32(1)
    A = (np.asarray(G, np.complex64) / mx).astype(np.complex64)
    A = (np.tril(A) + np.tril(A, -1).conj().T).astype(np.complex64)
    d = np.zeros(n, np.float32)
    e = np.zeros(n, np.float32)
    for j in range(n - 1):
        x = A[j + 1:, j].copy()
        alpha = x[0]
        xn2 = np.float32(np.sum(np.abs(x[1:]) ** 2))
        v = np.zeros_like(x)
        if xn2 == 0 and alpha.imag == 0:
            beta, tau = np.float32(alpha.real), np.complex64(0)
            v[0] = 1
        else:
            beta = np.float32(-np.copysign(np.sqrt(alpha.real ** 2 + alpha.imag ** 2 + xn2), alpha.real))
            tau = np.complex64(complex((beta - alpha.real) / beta, -alpha.imag / beta))
            v = (x * np.complex64(1 / (alpha - beta))).astype(np.complex64)
            v[0] = 1
        d[j], e[j] = np.float32(A[j, j].real), beta
        A22 = A[j + 1:, j + 1:]
        p = (tau * (A22 @ v)).astype(np.complex64)
        K = np.complex64(-0.5 * tau * np.vdot(p, v))
        w = (p + K * v).astype(np.complex64)
        A[j + 1:, j + 1:] = A22 - (np.outer(v, w.conj()) + np.outer(w, v.conj())).astype(np.complex64)
    d[n - 1] = np.float32(A[n - 1, n - 1].real)
    return d, e


def _sturm(d, e, x):
    x = np.float32(x)
    q, c = np.float32(1), 0
    for k in range(len(d)):
        q = d[k] - x - ((e[k - 1] * e[k - 1]) / q if k > 0 else np.float32(0))
        if abs(q) < np.float32(1e-30):
            q = np.float32(-1e-30)
        if q < 0:
            c += 1
    return c


def bisect(d, e, t):
    """The t-th largest eigenvalue of T by 32-way multisection."""
    n = len(d)
    r = [(abs(e[k - 1]) if k else 0) + (abs(e[k]) if k < n - 1 else 0) for k in range(n)]
    gl = min(d[k] - r[k] for k in range(n))
    gu = max(d[k] + r[k] for k in range(n))
    span = max(abs(gl), abs(gu))
    lo, hi = np.float32(gl - 4 * EPS * span), np.float32(gu + 4 * EPS * span)
    idx = n - 1 - t
    tol = 2 * EPS * max(abs(lo), abs(hi))
    for _ in range(64):
        if hi - lo <= tol:
            break
        xs = [np.float32(lo + (hi - lo) * np.float32(l + 1) / np.float32(33)) for l in range(32)]
        f = next((l for l in range(32) if _sturm(d, e, xs[l]) > idx), 32)
        nhi = xs[f] if f < 32 else hi
        nlo = xs[f - 1] if f > 0 else lo
        if nhi == hi and nlo == lo:
            break
        lo, hi = nlo, nhi
    return np.float32(0.5) * (lo + hi)


def inverse_iteration(d, e, lam, rng, solves=3):
    """Unit eigenvector of T for the shift lam, from a random start."""
    n = len(d)
    tnorm = max(abs(d[k]) + abs(e[k]) + (abs(e[k - 1]) if k else 0) for k in range(n))
    piv = EPS * max(tnorm, np.float32(1e-30))
    U0, U1, U2, Lm = (np.zeros(n, np.float32) for _ in range(4))
    Pv = np.zeros(n, np.int8)
    u0, u1, u2 = d[0] - lam, (e[0] if n > 1 else np.float32(0)), np.float32(0)
    for k in range(n - 1):
        sub, nd = e[k], d[k + 1] - lam
        ns = e[k + 1] if k + 1 < n - 1 else np.float32(0)
        if abs(u0) >= abs(sub):
            if u0 == 0:
                u0 = piv
            m = sub / u0
            a = (u0, u1, u2)
            u0, u1 = nd - m * u1, ns - m * u2
            pv = 0
        else:
            m = u0 / sub
            a = (sub, nd, ns)
            u0, u1 = u1 - m * nd, u2 - m * ns
            pv = 1
        u2 = np.float32(0)
        U0[k], U1[k], U2[k], Lm[k], Pv[k] = a[0], a[1], a[2], m, pv
    if abs(u0) < piv:
        u0 = np.float32(np.copysign(piv, u0 if u0 != 0 else 1))
    U0[n - 1] = u0
    y = rng.standard_normal(n).astype(np.float32)
    nrm = np.float32((y * y).sum())
    for _ in range(solves):
        b = y / np.sqrt(max(nrm, np.float32(1e-30)))
        bi = b[0]
        for k in range(n - 1):
            bn = b[k + 1]
            if Pv[k]:
                bi, bn = bn, bi
            y[k] = bi
            bi = bn - Lm[k] * bi
        y[n - 1] = bi
        x1 = x2 = np.float32(0)
        for k in range(n - 1, -1, -1):
            u = U0[k] if abs(U0[k]) >= piv else np.float32(np.copysign(piv, U0[k] if U0[k] != 0 else 1))
            val = (y[k] - U1[k] * x1 - U2[k] * x2) / u
            y[k], x2, x1 = val, x1, val
        nrm = np.float32((y * y).sum())
    return y / np.sqrt(nrm)
