"""GPU parity tests: every kernel through the C ABI against the CPU oracle and the
reference's golden vectors.  Tolerances are written in each test:
  * contraction / GEMM / single-qubit gate: relative 1e-5 (complex64), 1e-12 (complex128)
  * eigensolver: residual ||HV - V diag(w)|| <= 5e-5 ||H||, ||V^H V - I|| <= 1e-5
  * two-site update vs reference: kept singular values within 1e-5 * sigma_0,
    identical bond dimensions, state fidelity >= 1 - 1e-6.
"""
import functools
import numpy as np
import pytest
import torch

from conftest import load_golden, unpack_spectra, unpack_tensors

pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

import atlasq_gb300 as aq  # noqa: E402
from atlasq_gb300 import ops  # noqa: E402
from atlasq_gb300.circuits import haar_brickwork, haar_unitary, hea_circuit  # noqa: E402
from oracle import mps_oracle as mo  # noqa: E402
from oracle import statevector as sv  # noqa: E402

DEV = "cuda:0"


def crandn(*shape, dtype=torch.complex64, gen=None):
    re = torch.randn(*shape, generator=gen, dtype=torch.float64)
    im = torch.randn(*shape, generator=gen, dtype=torch.float64)
    return torch.complex(re, im).to(dtype)


def rel(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


# ----------------------------------------------------------------------------- kernels
@pytest.mark.parametrize("chiL,chiM,chiR", [(1, 1, 1), (1, 2, 4), (3, 5, 7), (17, 33, 9), (64, 64, 64),
                                            (255, 17, 130)])
@pytest.mark.parametrize("dt", [torch.complex64, torch.complex128])
def test_contract_gate_matches_oracle(chiL, chiM, chiR, dt):
    g = torch.Generator().manual_seed(chiL * 1000 + chiM * 10 + chiR)
    A = crandn(chiL, 2, chiM, gen=g, dtype=dt)
    B = crandn(chiM, 2, chiR, gen=g, dtype=dt)
    U = haar_unitary(g).to(dt)
    X = ops.contract_gate(A.to(DEV), B.to(DEV), U.to(DEV)).cpu().numpy()
    ref = mo.fused_two_qubit_gate(A.numpy().astype(np.complex128), B.numpy().astype(np.complex128),
                                  U.numpy().astype(np.complex128))
    tol = 1e-5 if dt == torch.complex64 else 1e-12
    assert rel(X, ref) < tol


@pytest.mark.parametrize("opA,opB", [("N", "N"), ("C", "N"), ("N", "C"), ("T", "N"), ("N", "T"), ("C", "C")])
def test_cgemm_ops(opA, opB):
    g = torch.Generator().manual_seed(3)
    M, N, K = 70, 45, 129
    A = crandn(*((M, K) if opA == "N" else (K, M)), gen=g)
    B = crandn(*((K, N) if opB == "N" else (N, K)), gen=g)
    C = ops.cgemm(A.to(DEV), B.to(DEV), opA, opB).cpu().numpy()
    f = {"N": lambda x: x, "T": lambda x: x.T, "C": lambda x: x.conj().T}
    ref = f[opA](A.numpy().astype(np.complex128)) @ f[opB](B.numpy().astype(np.complex128))
    assert rel(C, ref) < 1e-5


@pytest.mark.parametrize("opA,opB,M,N,K,batch", [("N", "N", 70, 45, 129, 1), ("C", "N", 256, 256, 512, 3),
                                                  ("N", "C", 128, 64, 32, 2), ("T", "T", 200, 130, 77, 1),
                                                  ("N", "N", 512, 272, 512, 4), ("R", "T", 129, 65, 33, 2),
                                                  ("T", "R", 64, 200, 95, 1), ("C", "C", 300, 70, 1, 1)])
def test_cgemm_tensor_cores_3xtf32(opA, opB, M, N, K, batch):
    """tcgen05 3xTF32 complex GEMM against float64 numpy: FP32-class relative error
    (<= 1e-6 + 2e-9 K: the tensor core's fp32 accumulation error grows with K).
    Every op (N, T, C, R), ragged M / N / K (tile edges, one k slice, K = 1)."""
    g = torch.Generator().manual_seed(M + N + K)
    A = crandn(batch, *((M, K) if opA in ("N", "R") else (K, M)), gen=g)
    B = crandn(batch, *((K, N) if opB in ("N", "R") else (N, K)), gen=g)
    C = ops.cgemm_tc(A.to(DEV), B.to(DEV), opA, opB).cpu().numpy()
    f = {"N": lambda x: x, "T": lambda x: np.swapaxes(x, -1, -2), "C": lambda x: np.swapaxes(x, -1, -2).conj(),
         "R": lambda x: x.conj()}
    ref = f[opA](A.numpy().astype(np.complex128)) @ f[opB](B.numpy().astype(np.complex128))
    assert rel(C, ref) < 1e-6 + 2e-9 * K


def test_cgemm_tensor_cores_bounded_wait_expires_cleanly():
    """The GEMM's pipeline waits are bounded.  With their poll limit set to 0 no
    stage can be waited for, so every tile aborts: the synchronous entry returns
    AGB_ERR_TIMEOUT, the asynchronous one sets the device status word, which
    stays set through a later successful call; the context stays usable and the
    next call with the default limit is correct."""
    import ctypes
    from atlasq_gb300 import _lib
    lib = _lib.load()
    g = torch.Generator().manual_seed(5)
    A = crandn(2, 256, 96, gen=g).to(DEV)
    B = crandn(2, 96, 128, gen=g).to(DEV)
    bat, M, K, N = 2, 256, 96, 128
    C = torch.zeros(bat, M, N, dtype=torch.complex64, device=DEV)
    need = lib.agb_cgemm_tc_workspace(bat, M, N, K)
    ws = torch.empty(need, dtype=torch.uint8, device=DEV)
    stream = torch.cuda.current_stream().cuda_stream
    word = torch.zeros(1, dtype=torch.int32, device=DEV)

    def call(status_host=None, status_dev=None):
        args = (b"N", b"N", bat, M, N, K, A.data_ptr(), K, M * K, B.data_ptr(), N, K * N, C.data_ptr(), N, M * N,
                1.0, 0.0, 0.0, 0.0, ws.data_ptr(), need)
        if status_dev is None:
            return lib.agb_cgemm_tc(*args, ctypes.byref(status_host), stream)
        return lib.agb_cgemm_tc_async(*args, status_dev.data_ptr(), stream)

    assert lib.agb_set_gemm_wait_limit(0) == 0
    try:
        st = ctypes.c_int(0)
        assert call(status_host=st) == _lib.AGB_ERR_TIMEOUT
        assert st.value == _lib.AGB_ERR_TIMEOUT
        assert call(status_dev=word) == 0
        torch.cuda.synchronize()
        assert int(word.item()) == _lib.AGB_ERR_TIMEOUT
    finally:
        lib.agb_set_gemm_wait_limit(-1)
    st = ctypes.c_int(0)
    assert call(status_host=st) == 0 and st.value == 0
    ref = A.cpu().numpy().astype(np.complex128) @ B.cpu().numpy().astype(np.complex128)
    assert rel(C.cpu().numpy(), ref) < 1e-6
    assert call(status_dev=word) == 0
    torch.cuda.synchronize()
    assert int(word.item()) == _lib.AGB_ERR_TIMEOUT  # sticky: never cleared by the library


@functools.lru_cache(maxsize=1)
def _hermitian_cases():
    g = torch.Generator().manual_seed(11)
    cases = []
    for n in (1, 2, 5, 33, 128, 300, 512, 800, 1024):
        X = crandn(n + 3, n, gen=g, dtype=torch.complex128)
        cases.append(("gram", X.conj().T @ X))
    # rank deficient Gram (rank 40 of 96)
    X = crandn(40, 96, gen=g, dtype=torch.complex128)
    cases.append(("rankdef", X.conj().T @ X))
    # exactly degenerate spectrum (cluster of 30 equal eigenvalues)
    Q, _ = torch.linalg.qr(crandn(80, 80, gen=g, dtype=torch.complex128))
    w = torch.cat([torch.full((30,), 2.0), torch.linspace(1.0, 0.01, 50)]).to(torch.complex128)
    cases.append(("degenerate", (Q * w) @ Q.conj().T))
    # graded spectrum over 8 decades
    w = (10.0 ** -torch.linspace(0, 8, 64)).to(torch.complex128)
    Q, _ = torch.linalg.qr(crandn(64, 64, gen=g, dtype=torch.complex128))
    cases.append(("graded", (Q * w) @ Q.conj().T))
    # 100-fold degenerate cluster (CholeskyQR2 path, one chunk)
    Q, _ = torch.linalg.qr(crandn(160, 160, gen=g, dtype=torch.complex128))
    w = torch.cat([torch.full((100,), 1.0), torch.linspace(0.5, 0.01, 60)]).to(torch.complex128)
    cases.append(("bigcluster", (Q * w) @ Q.conj().T))
    # 300-wide near-degenerate tail (spread 1e-7 relative): block Gram-Schmidt over two chunks
    Q, _ = torch.linalg.qr(crandn(400, 400, gen=g, dtype=torch.complex128))
    w = torch.cat([torch.linspace(1.0, 0.1, 100), 1e-3 * (1 + 1e-7 * torch.rand(300, generator=g, dtype=torch.float64))]).to(torch.complex128)
    cases.append(("hugecluster", (Q * w) @ Q.conj().T))
    return cases


@pytest.mark.parametrize("n,ell", [(192, 50), (256, 35), (384, 24)])
@pytest.mark.parametrize("dt", [torch.complex64, torch.complex128])
def test_heevd_vector_phase_near_the_default_shared_memory_limit(n, ell, dt):
    """Sizes whose cluster inverse-iteration launch takes just under 48 KiB of
    dynamic shared memory: with the kernel's static shared memory the launch
    needs the opt-in, which was once granted only above 48 KiB of dynamic
    memory (the launch was refused with cudaErrorInvalidValue)."""
    g = torch.Generator().manual_seed(n + ell)
    Q, _ = torch.linalg.qr(crandn(n, n, gen=g, dtype=torch.complex128))
    w = torch.linspace(1.0, 0.01, n, dtype=torch.float64).to(torch.complex128)
    H = (Q * w) @ Q.conj().T
    H = (H + H.conj().T) / 2
    wv, V = ops.heevd(H.to(dt).to(DEV), ell=ell)
    wv = wv.cpu().double().numpy()
    V = V.cpu().to(torch.complex128).numpy()
    Hn = H.numpy()
    ref = np.linalg.eigvalsh(Hn)[::-1][:ell]
    tol = 5e-5 if dt == torch.complex64 else 1e-11
    assert np.max(np.abs(wv - ref)) <= tol
    assert np.linalg.norm(Hn @ V - V * wv[None, :]) <= tol * np.sqrt(ell)


@pytest.mark.parametrize("case", range(14))
@pytest.mark.parametrize("dt", [torch.complex64, torch.complex128])
def test_heevd_residual_and_orthonormality(case, dt):
    """Sizes 800 and 1024 (and 512 in complex128) exercise the cluster
    tridiagonalisation with rows overflowing shared memory into L2."""
    name, H = _hermitian_cases()[case]
    H = (H + H.conj().T) / 2
    n = H.shape[0]
    ell = n if name != "gram" or n < 100 else n // 2
    w, V = ops.heevd(H.to(dt).to(DEV), ell=ell)
    w = w.cpu().double().numpy()
    V = V.cpu().to(torch.complex128).numpy()
    Hn = H.numpy()
    ref = np.linalg.eigvalsh(Hn)[::-1][:ell]
    nrm = np.abs(ref).max()
    tol = 5e-5 if dt == torch.complex64 else 1e-11
    assert np.max(np.abs(w - ref)) <= tol * nrm
    assert np.linalg.norm(Hn @ V - V * w[None, :]) <= tol * nrm * np.sqrt(ell)
    assert np.max(np.abs(V.conj().T @ V - np.eye(ell))) <= (1e-5 if dt == torch.complex64 else 1e-12)


@pytest.mark.parametrize("M,N,trans", [(8, 4, False), (4, 8, False), (512, 256, False), (37, 37, False),
                                       (256, 512, True), (16, 64, True)])
def test_qr(M, N, trans):
    g = torch.Generator().manual_seed(M + N)
    A = crandn(*((N, M) if trans else (M, N)), gen=g)
    if M > 20 and not trans:
        A[:, 3] = A[:, 1] * 2.0  # rank deficiency
    Q, R = ops.qr(A.to(DEV), transA=trans, trans_out=trans)
    Q = Q.cpu().to(torch.complex128).numpy()
    R = R.cpu().to(torch.complex128).numpy()
    if trans:
        Q, R = Q.T, R.T
    Aop = A.numpy().astype(np.complex128)
    Aop = Aop.T if trans else Aop
    kk = min(M, N)
    assert Q.shape == (M, kk) and R.shape == (kk, N)
    assert rel(Q @ R, Aop) < 1e-5
    assert np.max(np.abs(Q.conj().T @ Q - np.eye(kk))) < 1e-5
    assert np.allclose(np.tril(R, -1), 0)


def test_single_qubit_gate_uses_transpose_convention():
    g = load_golden("known_answers")
    m = aq.AdaptiveMPS(2, bond_dim=1, device=DEV)
    th = 0.7
    m.ry(0, th)
    assert np.allclose(m.to_statevector().cpu().numpy(), g["ry07_state"], atol=1e-6)


# ----------------------------------------------------------------------------- two-site update
CIRCUITS = {
    "brickwork_n12_d10_chi32": lambda: haar_brickwork(12, 10, seed=1234),
    "brickwork_n8_d6_chi8": lambda: haar_brickwork(8, 6, seed=5),
    "brickwork_n10_d8_chi16_eps1e-3": lambda: haar_brickwork(10, 8, seed=11),
    "hea_n10_l3_chi16": lambda: hea_circuit(10, 3, seed=3),
}


def run_gpu(ops_, n, chi, eps, dtype=torch.complex64, flush_each=False):
    pol = aq.DTypePolicy(default=dtype)
    m = aq.AdaptiveMPS(n, bond_dim=1, eps_bond=eps, chi_max_per_bond=chi, device=DEV, dtype=dtype,
                       dtype_policy=pol)
    for kind, q, U in ops_:
        if kind == "2q":
            m.apply_two_site_gate(q, U)
        else:
            m.apply_single_qubit_gate(q, U)
        if flush_each:
            m.flush()
    m.flush()
    return m


@pytest.mark.parametrize("name", sorted(CIRCUITS))
def test_two_site_matches_reference_golden(name):
    """Ranks, bond dimensions and the final state match the reference complex64
    run.  Per-gate singular values / entropies are compared for the Haar
    circuits only: the HEA circuit has exactly degenerate spectra, and when the
    float32 rank rule drops one member of a degenerate pair the choice is
    arbitrary; in a non-canonical MPS the later X spectra then depend on that
    choice (the reference's own complex64 and complex128 runs differ there,
    bond 2 keeps 7 vs 8) while the physical state agrees to 1e-7."""
    g = load_golden(name)
    n, chi, eps = int(g["n"]), int(g["chi"]), float(g["eps"])
    m = run_gpu(CIRCUITS[name](), n, chi, eps)
    logs = m.statistics.logs
    psi = m.to_statevector().cpu().numpy()
    if name.startswith("brickwork"):
        assert list(m.bond_dims) == list(g["bond_dims"])
        assert logs["k_star"] == [int(x) for x in g["log_k_star"]]
        assert np.allclose(logs["eps_local"], g["log_eps_local"], atol=2e-6)
        assert np.allclose(logs["entropy"], g["log_entropy"], atol=1e-4)
    else:
        # the degenerate tail sits exactly at the float32 threshold: the reference's
        # complex64 and complex128 runs keep 7 and 8 on bond 2; either is a match
        assert list(m.bond_dims) in (list(g["bond_dims"]), list(g["bond_dims64"]))
        assert sv.fidelity(psi, g["statevector64"]) > 1 - 1e-6
    f = sv.fidelity(psi, g["statevector"])
    assert f > 1 - 1e-6, f


@pytest.mark.parametrize("name", sorted(CIRCUITS))
def test_two_site_fp64_matches_reference_fp64(name):
    g = load_golden(name)
    n, chi, eps = int(g["n"]), int(g["chi"]), float(g["eps"])
    m = run_gpu(CIRCUITS[name](), n, chi, eps, dtype=torch.complex128)
    assert list(m.bond_dims) == list(g["bond_dims64"])
    f = sv.fidelity(m.to_statevector().cpu().numpy(), g["statevector64"])
    assert f > 1 - 1e-10, f


def test_batched_equals_one_by_one():
    ops_ = haar_brickwork(10, 6, seed=21)
    a = run_gpu(ops_, 10, 16, 1e-8)
    b = run_gpu(ops_, 10, 16, 1e-8, flush_each=True)
    assert a.bond_dims == b.bond_dims
    f = mo.mps_fidelity([t.cpu().numpy() for t in a.tensors], [t.cpu().numpy() for t in b.tensors])
    assert f > 1 - 1e-10


def test_bell_ghz_known_answers():
    g = load_golden("known_answers")
    m = aq.AdaptiveMPS(2, bond_dim=1, eps_bond=1e-10, chi_max_per_bond=4, device=DEV)
    m.h(0)
    m.cnot(0, 1)
    assert np.allclose(m.to_statevector().cpu().numpy(), g["bell_state"], atol=1e-6)
    assert m.bond_dims == [2]
    assert m.global_error_bound() < 1e-5
    m = aq.AdaptiveMPS(6, bond_dim=1, eps_bond=1e-10, chi_max_per_bond=8, device=DEV)
    m.h(0)
    for i in range(5):
        m.cnot(i, i + 1)
    assert sv.fidelity(m.to_statevector().cpu().numpy(), g["ghz6_state"]) > 1 - 1e-6
    assert m.bond_dims == list(g["ghz6_bonds"])
    m = aq.AdaptiveMPS(2, bond_dim=1, eps_bond=1e-10, chi_max_per_bond=4, device=DEV)
    m.apply_two_site_gate(0, torch.tensor(g["u4"]))
    assert np.allclose(m.to_statevector().cpu().numpy(), g["u4"][:, 0], atol=1e-5)


def test_initial_state_shapes_match_reference():
    m = aq.AdaptiveMPS(5, bond_dim=8, device=DEV)
    assert m.bond_dims == [2, 4, 8, 8]
    psi = m.to_statevector().cpu().numpy()
    assert abs(psi[0] - 1) < 1e-6 and np.abs(psi[1:]).max() < 1e-6
    m = aq.AdaptiveMPS(4, bond_dim=2, device=DEV)
    assert m.bond_dims == [2, 2, 2]


def test_caps_and_budget_respected():
    ops_ = haar_brickwork(10, 8, seed=4)
    m = run_gpu(ops_, 10, 6, 1e-10)
    assert max(m.bond_dims) <= 6
    caps = [2, 3, 4, 5, 6, 5, 4, 3, 2]
    mm = aq.AdaptiveMPS(10, bond_dim=1, eps_bond=1e-10, chi_max_per_bond=caps, device=DEV)
    for kind, q, U in ops_:
        mm.apply_two_site_gate(q, U)
    assert all(d <= c for d, c in zip(mm.bond_dims, caps))


def test_fp64_oracle_fidelity_medium():
    """16 qubits, brickwork depth 12, chi 64: GPU complex64 vs FP64 oracle and exact state."""
    n, depth, chi = 16, 12, 64
    ops_ = haar_brickwork(n, depth, seed=99)
    m = run_gpu(ops_, n, chi, 1e-8)
    ref = mo.OracleMPS(n, bond_dim=1, eps_bond=1e-8, chi_max_per_bond=chi, dtype=np.complex128)
    for kind, q, U in ops_:
        ref.apply_two_site_gate(q, U.numpy())
    f = mo.mps_fidelity([t.cpu().numpy() for t in m.tensors], ref.tensors)
    assert f > 1 - 1e-6, f
    psi = sv.zero_state(n)
    for kind, q, U in ops_:
        psi = sv.apply_two_qubit(psi, n, q, U.numpy().astype(np.complex128))
    fe = sv.fidelity(m.to_statevector().cpu().numpy(), psi)
    fo = sv.fidelity(ref.to_statevector(), psi)
    # exact-state fidelity of the truncated states agrees to 1e-5 (complex64 vs FP64 truncation)
    assert abs(fe - fo) < 1e-5


# ----------------------------------------------------------------------------- canonical forms
def test_canonical_sweeps():
    g = load_golden("canonical")
    ts = unpack_tensors(g["in_shapes"], g["in_flat"])
    n = len(ts)
    m = aq.AdaptiveMPS(n, bond_dim=1, device=DEV)
    m.tensors = [torch.tensor(t).to(DEV) for t in ts]
    m.bond_dims = [t.shape[2] for t in ts[:-1]]
    m.canonicalize_right_to_left()
    assert sv.fidelity(m.to_statevector().cpu().numpy(), g["right"]) > 1 - 1e-6
    for t in m.tensors[1:]:
        M = t.cpu().to(torch.complex128).reshape(t.shape[0], -1).numpy()
        assert np.allclose(M @ M.conj().T, np.eye(M.shape[0]), atol=1e-5)
    m.to_mixed_canonical(3)
    assert sv.fidelity(m.to_statevector().cpu().numpy(), g["mixed"]) > 1 - 1e-6
    m.to_left_canonical()
    for t in m.tensors[:-1]:
        M = t.cpu().to(torch.complex128).reshape(-1, t.shape[2]).numpy()
        assert np.allclose(M.conj().T @ M, np.eye(M.shape[1]), atol=1e-5)
    assert sv.fidelity(m.to_statevector().cpu().numpy(), g["left"]) > 1 - 1e-6


# ----------------------------------------------------------------------------- sampling
def test_sampling_bit_exact_vs_oracle():
    """Same right-canonical tensors, same Philox stream: decisions agree except
    where |u - P(0)| is below the float32 probability resolution."""
    from atlasq_gb300.sampling import sample_tensors
    from oracle.philox import sample_uniforms
    g = load_golden("canonical")
    ts = unpack_tensors(g["in_shapes"], g["in_flat"])
    rc = mo.right_canonicalize(ts)
    shots, seed = 20000, 77
    bits, pz = sample_tensors([torch.tensor(t.astype(np.complex64)).to(DEV) for t in rc], shots, seed,
                              return_pz=True)
    bits = bits.cpu().numpy()
    ref_bits, ref_pz = mo.batch_sweep_sample(rc, shots, seed)
    n = len(rc)
    diff = bits != ref_bits
    if diff.any():
        # every disagreeing shot must have a near-threshold decision somewhere
        for s in np.nonzero(diff)[0]:
            near = min(abs(sample_uniforms(seed, np.array([s]), i)[0] - ref_pz[s, i]) for i in range(n))
            assert near < 1e-5
    assert diff.mean() < 1e-3
    p = np.abs(g["before"].astype(np.complex128)) ** 2
    p /= p.sum()
    h = np.bincount(bits, minlength=2 ** n) / shots
    assert 0.5 * np.abs(h - p).sum() < 0.05


def test_sample_api_distribution():
    ops_ = haar_brickwork(8, 6, seed=5)
    m = run_gpu(ops_, 8, 16, 1e-10)
    psi = m.to_statevector().cpu().numpy()
    p = np.abs(psi) ** 2
    p /= p.sum()
    s = m.sample(30000, seed=5)
    h = np.bincount(np.array(s), minlength=256) / len(s)
    assert 0.5 * np.abs(h - p).sum() < 0.05


# ----------------------------------------------------------------------------- expectations
def test_expectations_match_reference_golden():
    g = load_golden("expectations")
    n = int(g["n"])
    ts = unpack_tensors(g["tensor_shapes"], g["tensor_flat"])
    m = aq.AdaptiveMPS(n, bond_dim=1, device=DEV)
    m.tensors = [torch.tensor(t).to(DEV) for t in ts]
    m.bond_dims = [t.shape[2] for t in ts[:-1]]
    X = torch.tensor([[0, 1], [1, 0]], dtype=torch.complex64)
    Y = torch.tensor([[0, -1j], [1j, 0]], dtype=torch.complex64)
    Z = torch.tensor([[1, 0], [0, -1]], dtype=torch.complex64)
    for i in range(n - 1):
        assert abs(aq.correlation_function(Z, i, Z, i + 1, m) - g["zz"][i]) < 1e-5
    for i in range(n):
        assert abs(aq.expectation_value(aq.MPOBuilder.local_operator(X, i, n, device=DEV), m) - g["x"][i]) < 1e-5
        assert abs(aq.expectation_value(aq.MPOBuilder.local_operator(Y, i, n, device=DEV), m) - g["y"][i]) < 1e-5
    obs = [{i: Z, i + 1: Z} for i in range(n - 1)] + [{i: X} for i in range(n)] + \
          [{i: X, i + 2: Y} for i in range(n - 2)]
    vals = aq.local_expectations(m, obs)
    ref = list(g["zz"]) + list(g["x"]) + list(g["xy"])
    assert max(abs(a - b) for a, b in zip(vals, ref)) < 1e-5


def test_mpo_known_answers():
    Z = torch.tensor([[1, 0], [0, -1]], dtype=torch.complex64)
    X = torch.tensor([[0, 1], [1, 0]], dtype=torch.complex64)
    m = aq.AdaptiveMPS(5, bond_dim=2, device=DEV)
    assert abs(aq.expectation_value(aq.MPOBuilder.identity_mpo(5, device=DEV), m) - 1.0) < 1e-5
    assert abs(aq.correlation_function(Z, 0, Z, 2, m).real - 1.0) < 1e-5
    m = aq.AdaptiveMPS(3, bond_dim=2, device=DEV)
    m.x(1)
    assert abs(aq.expectation_value(aq.MPOBuilder.local_operator(Z, 1, 3, device=DEV), m) + 1.0) < 1e-5
    m = aq.AdaptiveMPS(10, bond_dim=2, device=DEV)
    for q in range(10):
        m.h(q)
    assert abs(aq.correlation_function(X, 0, X, 5, m).real - 1.0) < 1e-4
    # sum of local operators (MPO bond dimension > 1)
    Mz = aq.MPOBuilder.sum_local_operators(5, [(i, Z) for i in range(5)], device=DEV)
    m = aq.AdaptiveMPS(5, bond_dim=1, device=DEV)
    m.x(2)
    assert abs(aq.expectation_value(Mz, m) - 3.0) < 1e-4


# ----------------------------------------------------------------------------- misc API
def test_snapshot_roundtrip(tmp_path):
    ops_ = haar_brickwork(8, 4, seed=8)
    m = run_gpu(ops_, 8, 16, 1e-8)
    p = tmp_path / "s.pt"
    m.snapshot(str(p))
    m2 = aq.AdaptiveMPS.load_snapshot(str(p), device=DEV)
    assert m2.bond_dims == m.bond_dims
    assert sv.fidelity(m.to_statevector().cpu().numpy(), m2.to_statevector().cpu().numpy()) > 1 - 1e-10
    assert m2.statistics.logs["k_star"] == m.statistics.logs["k_star"]


def test_amplitudes_and_robust_svd():
    ops_ = haar_brickwork(6, 4, seed=2)
    m = run_gpu(ops_, 6, 16, 1e-10)
    psi = m.to_statevector().cpu().numpy()
    for b in (0, 5, 17, 63):
        assert abs(m.get_amplitude(b) - psi[b]) < 1e-5
    g = torch.Generator().manual_seed(5)
    X = crandn(40, 24, gen=g).to(DEV)
    U, S, Vh, drv = aq.robust_svd(X)
    ref = np.linalg.svd(X.cpu().numpy().astype(np.complex128), compute_uv=False)
    assert np.max(np.abs(S.cpu().numpy() - ref)) < 1e-5 * ref[0]
    assert rel(((U * S.to(U.dtype)) @ Vh).cpu().numpy(), X.cpu().numpy()) < 1e-5
    assert drv == "gb300_gram_heevd"


@pytest.mark.parametrize("chiM,eps", [(512, 1e-8), (96, 1e-8), (512, 1e-2)])
def test_two_site_chi512_matches_svd(chiM, eps):
    """chi_L = chi_R = 512 (X is 1024 x 1024, the chi_max=512 workload): kept rank,
    discarded weight and the truncated two-site block match a float64 SVD of the
    same X; chiM = 96 makes X rank-deficient (384 of 1024)."""
    gen = torch.Generator().manual_seed(chiM)
    A = crandn(512, 2, chiM, gen=gen, dtype=torch.complex128)
    B = crandn(chiM, 2, 512, gen=gen, dtype=torch.complex128)
    decay = torch.exp(-torch.arange(chiM, dtype=torch.float64) / 60.0)  # graded spectrum
    A = A * decay[None, None, :]
    A, B = A / A.norm(), B / B.norm()
    U = haar_unitary(gen).to(torch.complex128)
    m = aq.AdaptiveMPS(2, bond_dim=1, eps_bond=eps, chi_max_per_bond=512, device=DEV)
    m._tensors = [A.to(torch.complex64).to(DEV), B.to(torch.complex64).to(DEV)]
    m._bond_dims = [chiM]
    m.apply_two_site_gate(0, U.to(torch.complex64))
    m.flush()
    A32, B32 = A.to(torch.complex64).numpy(), B.to(torch.complex64).numpy()
    X = mo.fused_two_qubit_gate(A32.astype(np.complex128), B32.astype(np.complex128),
                                U.to(torch.complex64).numpy().astype(np.complex128))
    Uu, S, Vh = np.linalg.svd(X, full_matrices=False)
    k_ref = mo.choose_rank_from_sigma(S.astype(np.float32), eps, 512)[0]
    k = m.bond_dims[0]
    assert abs(k - k_ref) <= 1, (k, k_ref)
    Xt = (Uu[:, :k] * S[:k]) @ Vh[:k]
    Y = (m.tensors[0].cpu().numpy().reshape(1024, k).astype(np.complex128) @
         m.tensors[1].cpu().numpy().reshape(k, 1024).astype(np.complex128))
    f = abs(np.vdot(Xt, Y)) ** 2 / (np.vdot(Xt, Xt).real * np.vdot(Y, Y).real)
    assert f > 1 - 1e-6, f
    disc = np.sqrt(max(0.0, (S ** 2).sum() - (S[:k] ** 2).sum()))
    assert abs(m.statistics.logs["eps_local"][0] - disc) <= 1e-5 * S[0] + 1e-3 * disc


def test_autotuned_cluster_shape_keeps_results():
    """The autotuner picks an admissible cluster size, the library uses it for
    that shape, and the eigensolver still meets its residual bound."""
    from atlasq_gb300 import autotune
    C, ms = autotune.tune_tridiag(300, 2)
    assert C in (1, 2, 4, 6, 8, 16) and ms > 0
    assert autotune.tuned_cluster(300, 2) == C
    g = torch.Generator().manual_seed(77)
    X = crandn(303, 300, gen=g, dtype=torch.complex128)
    H = (X.conj().T @ X)
    w, V = ops.heevd(torch.stack([H, H]).to(torch.complex64).to(DEV), ell=150)
    ref = np.linalg.eigvalsh(H.numpy())[::-1][:150]
    nrm = np.abs(ref).max()
    for b in range(2):
        wb = w[b].cpu().double().numpy()
        Vb = V[b].cpu().to(torch.complex128).numpy()
        assert np.max(np.abs(wb - ref)) <= 5e-5 * nrm
        assert np.linalg.norm(H.numpy() @ Vb - Vb * wb[None, :]) <= 5e-5 * nrm * np.sqrt(150)


def test_near_degenerate_leading_group_keeps_every_direction():
    """A 58 x 56 two-site update whose ten leading eigenvalues of X^H X lie
    1e-5..4e-5 apart (tests/golden/collapse_case.npz, captured from a
    rank-predictor run).  With the former Sturm count (a pivot that cancelled
    to exactly 0 was counted as non-negative, then replaced by -pivmin) the
    bisection returned one leading eigenvalue midway between two neighbours
    and 68 of 80 runs gave overlapping eigenvectors (relative error up to
    0.26).  Every seed must reproduce X up to the truncation (relative error
    ~7e-4 at eps 1e-3) at the default cluster tolerance, without the
    orthogonality guard's repair (AGB_D_REPAIR bit 1)."""
    import atlasq_gb300.adaptive_mps as amod
    g = load_golden("collapse_case")
    A = torch.tensor(g["A"]).to(DEV)
    B = torch.tensor(g["B"]).to(DEV)
    U = torch.tensor(g["U"]).to(DEV)
    i, nq, chi, eps = int(g["bond"]), int(g["n_qubits"]), int(g["chi_max"]), float(g["eps"])
    th = torch.einsum("apm,mqb->apqb", A.to(torch.complex128), B.to(torch.complex128))
    X = torch.einsum("PQpq,apqb->aPQb", U.to(torch.complex128).reshape(2, 2, 2, 2), th)
    for oc in range(40):  # the operation counter enters the inverse-iteration seed
        for all_vectors in (True, False):
            m = aq.AdaptiveMPS(nq, bond_dim=1, eps_bond=eps, chi_max_per_bond=chi, device=DEV)
            m._operation_counter = oc
            m._tensors[i] = A.clone()
            m._tensors[i + 1] = B.clone()
            r = amod._run_pipeline([(m, i, U)], torch.complex64, None, all_vectors=all_vectors)[0]
            rec = torch.einsum("apk,kqb->apqb", r["A"].to(torch.complex128), r["B"].to(torch.complex128))
            err = float(torch.linalg.norm(X - rec) / torch.linalg.norm(X))
            assert err < 2e-3, (oc, all_vectors, err, r["k"])
            assert not (r["repair"] & 2), (oc, all_vectors, r["repair"])


def _planted(n_half, lead, rest, seed):
    """Site tensors A [n_half, 2, 2n_half], B [2n_half, 2, n_half] whose
    contraction is X = W_L diag(sqrt(lam)) W_R^H (gate = identity), with the
    leading eigenvalues of X^H X given by `lead` and the rest by `rest`."""
    rng = np.random.default_rng(seed)
    nn = 2 * n_half
    lam = np.concatenate([lead, rest])

    def haar(k):
        z = (rng.standard_normal((k, k)) + 1j * rng.standard_normal((k, k))) / np.sqrt(2)
        q, r = np.linalg.qr(z)
        return q * (np.diag(r) / np.abs(np.diag(r)))[None, :]
    WL, WR = haar(nn), haar(nn)
    A = (WL * np.sqrt(lam)[None, :]).reshape(n_half, 2, nn).astype(np.complex64)
    B = WR.conj().T.reshape(nn, 2, n_half).astype(np.complex64)
    return A, B


def _run_planted(A, B, cap, eps, oc, all_vectors, cluster_tol=None):
    import atlasq_gb300.adaptive_mps as amod
    m = aq.AdaptiveMPS(2, bond_dim=1, eps_bond=eps, chi_max_per_bond=cap, device=DEV)
    m._operation_counter = oc
    m._tensors = [torch.tensor(A).to(DEV), torch.tensor(B).to(DEV)]
    m._bond_dims = [A.shape[2]]
    U = torch.eye(4, dtype=torch.complex64, device=DEV)
    r = amod._run_pipeline([(m, 0, U)], torch.complex64, None, all_vectors=all_vectors, cluster_tol=cluster_tol)[0]
    X = np.einsum("apm,mqb->apqb", A.astype(np.complex128), B.astype(np.complex128)).reshape(2 * A.shape[0], -1)
    rec = np.einsum("apk,kqb->apqb", r["A"].cpu().numpy().astype(np.complex128),
                    r["B"].cpu().numpy().astype(np.complex128)).reshape(X.shape)
    s = np.linalg.svd(X, compute_uv=False)
    k = r["k"]
    opt = np.sqrt(max(0.0, (s ** 2).sum() - (s[:k] ** 2).sum()) / (s ** 2).sum())
    return r, np.linalg.norm(X - rec) / np.linalg.norm(X), opt


def test_near_degenerate_leading_group_n512():
    """The headline's Gram size (n = 512, chi_max 256): ten leading eigenvalues
    of X^H X spaced 1e-5..4e-5 apart (relative), straddling the 1e-5 cluster
    tolerance, then a decaying tail.  For 40 inverse-iteration seeds and both
    eigenvector-count modes the kept factors reproduce X to within twice the
    optimal truncation error, with no orthogonality repair."""
    rng = np.random.default_rng(7)
    gaps = 1e-5 * (1 + 3 * rng.random(9))
    lead = 1 - np.concatenate([[0], np.cumsum(gaps)])
    rest = 0.5 * np.exp(-np.arange(502) / 40.0)
    A, B = _planted(256, lead, rest, seed=11)
    for oc in range(40):
        for allv in (True, False):
            r, err, opt = _run_planted(A, B, 256, 1e-8, oc, allv)
            assert r["k"] == 256
            assert err <= 2 * opt + 1e-5, (oc, allv, err, opt)
            assert not (r["repair"] & 2), (oc, allv, r["repair"])


def test_orthogonality_guard_repairs_overlapping_vectors():
    """With the cluster tolerance forced to ~0 (AGB_D_CTOL), four leading
    eigenvalues of X^H X spaced 2e-7 apart (below the float32 Gram's
    resolution) are solved one by one by inverse iteration, which returns
    vectors mixed inside their common subspace.  The guard on the first
    Newton-Schulz product V^H V flags overlaps above 0.3, the repair pass
    re-runs the vector phase with the 1e-2 cluster tolerance, and every result
    is again the optimal truncation."""
    lead = 1.0 - 2e-7 * np.arange(4)
    rest = 0.6 * np.exp(-np.arange(60) / 6.0)
    A, B = _planted(32, lead, rest, seed=5)
    repaired = 0
    for oc in range(8):
        r, err, opt = _run_planted(A, B, 24, 1e-8, oc, True, cluster_tol=1e-30)
        repaired += bool(r["repair"] & 2)
        assert r["status"] == 0, (oc, r["status"])
        assert err <= 2 * opt + 1e-5, (oc, err, opt)
    assert repaired >= 1, repaired


@pytest.mark.parametrize("resident", [False, True])
def test_precision_promotion_matches_oracle(resident):
    """adaptive_mps.py:266-274: a gate whose kept spectrum spans more than
    promote_if_cond_gt (sigma_0 / sigma_{k-1}) is factorised again in
    complex128 and its two site tensors become complex128.  With the threshold
    lowered to 3, 14 of the 27 gates of a 10-qubit brickwork promote (their
    sigma_0 / sigma_{k-1} run from 1 to ~20, none within 7% of 3); the promoted
    gates, the kept ranks, the site dtypes and the state match the oracle run
    with the same policy.  Asked for device-resident execution, an instance
    whose threshold the rank rule can reach runs host-synchronised instead."""
    n = 10
    ops_ = haar_brickwork(n, 6, seed=21)
    pol = aq.DTypePolicy(default=torch.complex64, promote_if_cond_gt=3.0)
    m = aq.AdaptiveMPS(n, bond_dim=1, eps_bond=1e-6, chi_max_per_bond=16, device=DEV, dtype_policy=pol,
                       device_resident=resident)
    assert m.promotion_reachable()
    o = mo.OracleMPS(n, bond_dim=1, eps_bond=1e-6, chi_max_per_bond=16, dtype=np.complex64,
                     promote_if_cond_gt=3.0)
    for _, q, U in ops_:
        m.apply_two_site_gate(q, U)
        o.apply_two_site_gate(q, U.numpy())
    m.flush()
    assert m._res is None and m.unpromoted == 0
    logs = m.statistics.logs
    ours = [d == "gb300_gram_heevd_c128" for d in logs["svd_driver"]]
    ref = [d == "complex128" for d in o.logs["dtype"]]
    assert sum(ref) >= 8
    assert ours == ref
    assert logs["k_star"] == o.logs["k_star"]
    assert [t.dtype for t in m.tensors] == [torch.complex128 if t.dtype == np.complex128 else torch.complex64
                                            for t in o.tensors]
    f = mo.mps_fidelity([t.cpu().numpy() for t in m.tensors], o.tensors)
    assert f > 1 - 1e-6, f
