"""MPO applied to an MPS, Pauli exponentials and the TDVP environment steps
against the reference's own outputs (tests/golden/mpo_apply.npz, written by
tests/golden/make_golden.py).  Tolerances: complex128 relative 1e-10,
complex64 relative 1e-5 (1e-6 against the reference's complex64 statevectors
of apply_mpo_to_mps).

Pauli exponentials: the reference's result is exp(i lam P)|psi> for strings
of length <= 2 and differs from it for longer strings (its two-rail MPO drops
the letters from the third site on; the fixture shows fidelity 0.83 for
"XYZ").  This build applies exp(i lam P) for every length, so it matches the
fixture for the short strings and the exact exponential for all of them.
"""
import numpy as np
import pytest
import torch

from conftest import load_golden, unpack_tensors

pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

import atlasq_gb300 as aq  # noqa: E402
from atlasq_gb300 import mpo_ops  # noqa: E402
from atlasq_gb300.circuits import haar_brickwork  # noqa: E402
from oracle import statevector as sv  # noqa: E402

DEV = "cuda:0"
C128 = torch.complex128
PAULI = {"I": np.eye(2), "X": np.array([[0, 1], [1, 0]]), "Y": np.array([[0, -1j], [1j, 0]]),
         "Z": np.diag([1.0, -1.0])}


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b))


def _mps128(tensors):
    n = len(tensors)
    m = aq.AdaptiveMPS(n, bond_dim=1, device=DEV, dtype=C128, dtype_policy=aq.DTypePolicy(default=C128))
    m.tensors = [torch.tensor(t).to(DEV) for t in tensors]
    m.bond_dims = [t.shape[2] for t in tensors[:-1]]
    return m


def test_apply_mpo_to_mps_matches_reference():
    g = load_golden("mpo_apply")
    ts = unpack_tensors(g["mpo_in_shapes"], g["mpo_in_flat"])
    n = len(ts)
    Z = torch.tensor([[1, 0], [0, -1]], dtype=C128)
    Y = torch.tensor([[0, -1j], [1j, 0]], dtype=C128)
    H = aq.MPOBuilder.sum_local_operators(n, [(i, Z) for i in range(n)] + [(2, Y)], device=DEV, dtype=C128)
    assert H.bond_dims == [2] * (n - 1)
    # the reference returns this statevector in complex64 (the dtype of the
    # AdaptiveMPS it builds for the result), so the bar is float32 rounding
    res = mpo_ops.apply_mpo_to_mps(H, _mps128(ts))
    assert rel(res.to_statevector().cpu().numpy(), g["mpo_sum_state"]) < 1e-6
    P = aq.MPOBuilder.local_operator(Y, 3, n, device=DEV, dtype=C128)
    res = mpo_ops.apply_mpo_to_mps(P, _mps128(ts))
    assert rel(res.to_statevector().cpu().numpy(), g["mpo_local_state"]) < 1e-6
    # left-canonical result, bond dimensions multiplied by the MPO's (no truncation)
    for t in res.tensors[:-1]:
        M = t.cpu().numpy().reshape(-1, t.shape[2])
        assert np.allclose(M.conj().T @ M, np.eye(M.shape[1]), atol=1e-10)


def test_pauli_exponential_matches_reference_and_exact():
    g = load_golden("mpo_apply")
    strings = [str(x) for x in g["pauli_strings"]]
    lam = 0.6 * 0.5
    for k, ps in enumerate(strings):
        n = len(ps)
        m = aq.AdaptiveMPS(n, bond_dim=1, device=DEV, dtype=C128, dtype_policy=aq.DTypePolicy(default=C128))
        Hd = torch.tensor([[1, 1], [1, -1]], dtype=C128) / np.sqrt(2)
        for q in range(n):
            m.apply_single_qubit_gate(q, Hd)
        m.apply_two_site_gate(0, haar_brickwork(2, 1, seed=9 + k)[0][2].to(C128))
        psi0 = m.to_statevector().cpu().numpy()
        assert rel(psi0, g[f"pauli{k}_in"]) < 1e-10
        mpo_ops.apply_pauli_exp_to_mps(m, ps, 1j * 0.5, 0.6)
        psi = m.to_statevector().cpu().numpy()
        Pm = np.array([[1.0]])
        for c in ps:
            Pm = np.kron(Pm, PAULI[c])
        exact = np.cos(lam) * psi0 + 1j * np.sin(lam) * (Pm @ psi0)
        assert rel(psi, exact) < 1e-10, ps
        ref = g[f"pauli{k}_out"]
        if n <= 2:
            assert rel(psi, ref) < 1e-10, ps
        else:
            assert sv.fidelity(ref, exact) < 0.99, ps  # the reference's deviation, recorded
        assert m.bond_dims == [t.shape[2] for t in m.tensors[:-1]]


@pytest.mark.parametrize("dt,tol", [(torch.complex128, 1e-10), (torch.complex64, 1e-5)])
def test_tdvp_environments_match_reference(dt, tol):
    g = load_golden("mpo_apply")
    A = torch.tensor(g["tdvp_A"]).to(DEV, dt)
    W = torch.tensor(g["tdvp_W"]).to(DEV, dt)
    L = torch.tensor(g["tdvp_L"]).to(DEV, dt)
    R = torch.tensor(g["tdvp_R"]).to(DEV, dt)
    Lin = torch.tensor(g["tdvp_left_in"]).to(DEV, dt)
    assert rel(mpo_ops.tdvp_left_environment(Lin, A, W).cpu().numpy(), g["tdvp_left"]) < tol
    assert rel(mpo_ops.tdvp_right_environment(R, A, W).cpu().numpy(), g["tdvp_right"]) < tol
    assert rel(mpo_ops.tdvp_apply_local_H(L, W, A, R).cpu().numpy(), g["tdvp_local"]) < tol


def test_general_mpo_expectation_uses_environments():
    """expectation_value of a bond-2 MPO equals the sum of the local terms, and
    the TDVP left environments of the identity-padded chain close to it."""
    ops_ = haar_brickwork(8, 4, seed=3)
    m = aq.AdaptiveMPS(8, bond_dim=1, eps_bond=1e-10, chi_max_per_bond=16, device=DEV, dtype=C128,
                       dtype_policy=aq.DTypePolicy(default=C128))
    for _, q, U in ops_:
        m.apply_two_site_gate(q, U.to(C128))
    Z = torch.tensor([[1, 0], [0, -1]], dtype=C128)
    X = torch.tensor([[0, 1], [1, 0]], dtype=C128)
    terms = [(i, Z) for i in range(8)] + [(i, 0.5 * X) for i in range(0, 8, 3)]
    H = aq.MPOBuilder.sum_local_operators(8, terms, device=DEV, dtype=C128)
    total = aq.expectation_value(H, m)
    parts = sum(aq.expectation_value(aq.MPOBuilder.local_operator(o, i, 8, device=DEV, dtype=C128), m)
                for i, o in terms)
    assert abs(total - parts) < 1e-10
    Lenv = torch.ones(1, 1, 1, dtype=C128, device=DEV)
    for A, W in zip(m.tensors, H.tensors):
        Lenv = mpo_ops.tdvp_left_environment(Lenv, A, W)
    N = torch.ones(1, 1, 1, dtype=C128, device=DEV)
    eye = aq.MPO.identity(8, device=DEV, dtype=C128)
    for A, W in zip(m.tensors, eye.tensors):
        N = mpo_ops.tdvp_left_environment(N, A, W)
    assert abs(complex(Lenv.reshape(-1)[0].item()) / complex(N.reshape(-1)[0].item()) - total) < 1e-10
