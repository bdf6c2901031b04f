"""Pin the CPU oracle against golden vectors produced by the reference itself."""
import numpy as np
import pytest

from conftest import load_golden, unpack_spectra, unpack_tensors
from oracle import mps_oracle as mo
from oracle import statevector as sv
from atlasq_gb300.circuits import haar_brickwork, hea_circuit

CIRCUITS = {
    "brickwork_n12_d10_chi32": lambda: haar_brickwork(12, 10, seed=1234),
    "brickwork_n8_d6_chi8": lambda: haar_brickwork(8, 6, seed=5),
    "brickwork_n10_d8_chi16_eps1e-3": lambda: haar_brickwork(10, 8, seed=11),
    "hea_n10_l3_chi16": lambda: hea_circuit(10, 3, seed=3),
}


def run_oracle(ops, n, chi, eps, dtype):
    m = mo.OracleMPS(n, bond_dim=1, eps_bond=eps, chi_max_per_bond=chi, dtype=dtype)
    spectra = []
    for kind, q, U in ops:
        if kind == "2q":
            spectra.append(m.apply_two_site_gate(q, U.numpy()))
        else:
            m.apply_single_qubit_gate(q, U.numpy())
    return m, spectra


def test_choose_rank_matches_reference():
    g = load_golden("choose_rank")
    vecs = unpack_spectra(g["lens"], g["flat"])
    for S, (eps, cap, k, el, ent, cond) in zip(vecs, g["meta"]):
        k2, el2, ent2, cond2 = mo.choose_rank_from_sigma(S.astype(np.float32), eps, int(cap))
        assert k2 == int(k), (eps, cap, S[:5])
        assert abs(el2 - el) <= 1e-6 * max(1.0, abs(el)) + 1e-12
        assert abs(ent2 - ent) <= 1e-5 * max(1.0, abs(ent))
        if np.isfinite(cond):
            assert abs(cond2 - cond) <= 1e-5 * cond
        else:
            assert not np.isfinite(cond2)


@pytest.mark.parametrize("name", sorted(CIRCUITS))
def test_oracle_complex64_matches_reference(name):
    g = load_golden(name)
    n, chi, eps = int(g["n"]), int(g["chi"]), float(g["eps"])
    m, spectra = run_oracle(CIRCUITS[name](), n, chi, eps, np.complex64)
    ref = unpack_spectra(g["sv_lens"], g["sv_flat"])
    assert len(ref) == len(spectra)
    ks = g["log_k_star"].astype(int)
    for s_ref, s, k in zip(ref, spectra, ks):
        assert s_ref.shape == s.shape
        # norm-wise relative error of the kept singular values
        assert np.max(np.abs(s_ref[:k] - s[:k])) <= 1e-5 * s_ref[0]
    assert list(m.bond_dims) == list(g["bond_dims"])
    assert sv.fidelity(m.to_statevector(), g["statevector"]) > 1 - 1e-6


@pytest.mark.parametrize("name", sorted(CIRCUITS))
def test_oracle_fp64_matches_reference_fp64(name):
    g = load_golden(name)
    n, chi, eps = int(g["n"]), int(g["chi"]), float(g["eps"])
    m, spectra = run_oracle(CIRCUITS[name](), n, chi, eps, np.complex128)
    ref = unpack_spectra(g["sv64_lens"], g["sv64_flat"])
    for s_ref, s in zip(ref, spectra):
        assert np.max(np.abs(s_ref - s)) <= 1e-12 * s_ref[0]
    assert list(m.bond_dims) == list(g["bond_dims64"])
    assert sv.fidelity(m.to_statevector(), g["statevector64"]) > 1 - 1e-12


@pytest.mark.parametrize("name", sorted(CIRCUITS))
def test_statevector_oracle_conventions(name):
    g = load_golden(name)
    n, chi = int(g["n"]), int(g["chi"])
    psi = sv.zero_state(n)
    for kind, q, U in CIRCUITS[name]():
        if kind == "2q":
            psi = sv.apply_two_qubit(psi, n, q, U.numpy().astype(np.complex128))
        else:
            psi = sv.apply_single_qubit_transposed(psi, n, q, U.numpy().astype(np.complex128))
    f = sv.fidelity(psi, g["statevector64"])
    ks = g["log_k_star"]
    if name == "hea_n10_l3_chi16" or name == "brickwork_n8_d6_chi8" and max(ks) < chi:
        assert f > 1 - 1e-8
    else:
        assert 0.0 < f <= 1.0 + 1e-12


def test_known_answers():
    g = load_golden("known_answers")
    m = mo.OracleMPS(2, dtype=np.complex64)
    th = 0.7
    RY = np.array([[np.cos(th / 2), -np.sin(th / 2)], [np.sin(th / 2), np.cos(th / 2)]])
    m.apply_single_qubit_gate(0, RY)
    assert np.allclose(m.to_statevector(), g["ry07_state"], atol=1e-6)
    # two-qubit ordering: U|00> = U[:, 0]
    m = mo.OracleMPS(2, eps_bond=1e-10, chi_max_per_bond=4, dtype=np.complex64)
    m.apply_two_site_gate(0, g["u4"])
    assert sv.fidelity(m.to_statevector(), g["u4_state"]) > 1 - 1e-6
    assert np.allclose(g["u4_state"], g["u4"][:, 0], atol=1e-5)
    H = np.array([[1, 1], [1, -1]]) / np.sqrt(2)
    CNOT = np.eye(4)[[0, 1, 3, 2]]
    m = mo.OracleMPS(6, eps_bond=1e-10, chi_max_per_bond=8, dtype=np.complex64)
    m.apply_single_qubit_gate(0, H)
    for i in range(5):
        m.apply_two_site_gate(i, CNOT)
    assert sv.fidelity(m.to_statevector(), g["ghz6_state"]) > 1 - 1e-6
    assert list(m.bond_dims) == list(g["ghz6_bonds"])


def test_expectations_match_reference():
    g = load_golden("expectations")
    n = int(g["n"])
    ts = unpack_tensors(g["tensor_shapes"], g["tensor_flat"])
    X = np.array([[0, 1], [1, 0]])
    Y = np.array([[0, -1j], [1j, 0]])
    Z = np.diag([1.0, -1.0])
    for i in range(n - 1):
        assert abs(mo.expectation_product(ts, {i: Z, i + 1: Z}) - g["zz"][i]) < 1e-5
    for i in range(n):
        assert abs(mo.expectation_product(ts, {i: X}) - g["x"][i]) < 1e-5
        assert abs(mo.expectation_product(ts, {i: Y}) - g["y"][i]) < 1e-5
    for i in range(n - 2):
        assert abs(mo.expectation_product(ts, {i: X, i + 2: Y}) - g["xy"][i]) < 1e-5
    # the reference evaluates <O^T>: <Y> from the dense state has the opposite sign
    psi = g["statevector"].astype(np.complex128)
    psi = psi / np.linalg.norm(psi)
    t = psi.reshape(2, 2 ** (n - 1))
    ydense = np.vdot(t, Y @ t)
    assert abs(ydense + g["y"][0]) < 1e-5


def test_canonical_sweeps_preserve_state():
    g = load_golden("canonical")
    ts = unpack_tensors(g["in_shapes"], g["in_flat"])
    rc = mo.right_canonicalize(ts)
    psi = rc[0]
    for t in rc[1:]:
        psi = np.einsum("...i,ijk->...jk", psi, t)
    assert sv.fidelity(psi.reshape(-1), g["right"]) > 1 - 1e-10
    for t in rc[1:]:
        l, p, r = t.shape
        M = t.reshape(l, p * r)
        assert np.allclose(M @ M.conj().T, np.eye(l), atol=1e-10)
    assert sv.fidelity(g["before"], g["mixed"]) > 1 - 1e-6
    assert sv.fidelity(g["before"], g["left"]) > 1 - 1e-6


def test_sampler_oracle_distribution():
    """The right-canonical Philox sampler reproduces |psi|^2 (TV distance at shot noise)."""
    g = load_golden("canonical")
    ts = unpack_tensors(g["in_shapes"], g["in_flat"])
    n = len(ts)
    rc = mo.right_canonicalize(ts)
    samples, _ = mo.batch_sweep_sample(rc, 40000, seed=123)
    p = np.abs(g["before"].astype(np.complex128)) ** 2
    p /= p.sum()
    h = np.bincount(samples, minlength=2 ** n) / len(samples)
    tv = 0.5 * np.abs(h - p).sum()
    assert tv < 0.04
