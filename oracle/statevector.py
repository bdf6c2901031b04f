"""Exact dense statevector simulator with the reference's gate conventions
(test infrastructure only; n <= 24).

* qubit 0 is the most significant bit of the basis index
  (mps_pytorch.py:615 ``bits = [(basis_state >> (n-1-i)) & 1 ...]``);
* a two-qubit gate on (i, i+1) applies U with qubit i as the high bit of the
  4-index (mps_complex.py:343-368, the path AdaptiveMPS uses);
* a single-qubit gate applies U^T (adaptive_mps.py:177).
"""
import numpy as np


def zero_state(n, dtype=np.complex128):
    psi = np.zeros(2 ** n, dtype=dtype)
    psi[0] = 1.0
    return psi


def apply_two_qubit(psi, n, i, U):
    t = psi.reshape((2 ** i, 4, 2 ** (n - i - 2)))
    t = np.einsum("ab,xby->xay", np.asarray(U).reshape(4, 4), t)
    return t.reshape(-1)


def apply_single_qubit_transposed(psi, n, q, U):
    t = psi.reshape((2 ** q, 2, 2 ** (n - q - 1)))
    t = np.einsum("st,xsy->xty", np.asarray(U), t)
    return t.reshape(-1)


def fidelity(a, b):
    a = np.asarray(a, dtype=np.complex128)
    b = np.asarray(b, dtype=np.complex128)
    return abs(np.vdot(a, b)) ** 2 / (np.vdot(a, a).real * np.vdot(b, b).real)
