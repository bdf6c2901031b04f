"""CPU-side checks: the C-ABI library loads and exports every declared symbol,
host planning logic, error mapping, and host-side policy code.  No kernel is
launched here."""
import ctypes
import os
import re

import numpy as np
import pytest
import torch

from conftest import ROOT, load_golden, unpack_spectra

import atlasq_gb300
from atlasq_gb300 import _build, _lib


def header_symbols():
    src = open(os.path.join(ROOT, "include", "atlasq_gb300.h")).read()
    return sorted(set(re.findall(r"\b(agb_[a-z0-9_]+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    _build.build()
    return _lib.load(build_if_missing=False)


def test_library_exports_every_declared_symbol(lib):
    declared = header_symbols()
    assert len(declared) >= 10
    for name in declared:
        assert hasattr(lib, name), name
    assert set(_lib.exported_symbols()) == set(declared)


def test_version(lib):
    assert lib.agb_version() >= 100


def _desc(rows):
    d = torch.zeros(len(rows), _lib.D_NFIELDS, dtype=torch.int64)
    for g, (l, m, r, cap, ell) in enumerate(rows):
        d[g, _lib.D_CHIL], d[g, _lib.D_CHIM], d[g, _lib.D_CHIR] = l, m, r
        d[g, _lib.D_CAP], d[g, _lib.D_ELL] = cap, ell
    return d


def test_two_site_plan_host_logic(lib):
    d = _desc([(256, 256, 256, 256, 0), (1, 1, 1, 4, 0), (4, 8, 16, 8, 3), (8, 8, 2, 64, 100)])
    ws = _lib.SZ(0)
    _lib.check(lib.agb_two_site_plan(_lib.AGB_C64, 4, _lib.ptr(d), ws))
    ells = d[:, _lib.D_ELL].tolist()
    assert ells == [256, 2, 3, 4]          # min(2chiL, 2chiR, cap) or the requested ell
    offs = d[:, _lib.D_WS].tolist()
    assert offs == sorted(offs) and all(o % 256 == 0 for o in offs)
    assert ws.value > offs[-1]
    # 512x512 Gram slab needs at least X + G complex64 planes
    assert offs[1] - offs[0] >= 2 * 512 * 512 * 8
    # complex128 has no tensor-core tail; its slab is about twice the complex64 slab
    ws128 = _lib.SZ(0)
    d2 = _desc([(256, 256, 256, 256, 0)])
    _lib.check(lib.agb_two_site_plan(_lib.AGB_C128, 1, _lib.ptr(d2), ws128))
    slab64 = offs[1] - offs[0]
    assert ws128.value > 1.9 * slab64
    # complex64 workspaces end with the tensor-core GEMMs' scratch token (the
    # split operands live in shared memory, not in the workspace)
    assert offs[-1] < ws.value < offs[-1] + slab64


def test_plan_rejects_bad_shapes(lib):
    ws = _lib.SZ(0)
    d = _desc([(0, 2, 2, 4, 0)])
    assert lib.agb_two_site_plan(_lib.AGB_C64, 1, _lib.ptr(d), ws) == _lib.AGB_ERR_ARG
    d = _desc([(2, 2, 600, 1024, 0)])
    assert lib.agb_two_site_plan(_lib.AGB_C64, 1, _lib.ptr(d), ws) == _lib.AGB_ERR_UNSUPPORTED
    assert lib.agb_two_site_plan(7, 1, _lib.ptr(d), ws) == _lib.AGB_ERR_ARG
    with pytest.raises(ValueError):
        _lib.check(_lib.AGB_ERR_ARG, "x")
    with pytest.raises(NotImplementedError):
        _lib.check(_lib.AGB_ERR_UNSUPPORTED, "x")


def test_entry_points_validate_arguments_without_a_gpu(lib):
    # argument checks return before any CUDA call
    assert lib.agb_contract_gate(5, None, None, None, None, 1, 1, 1, None) == _lib.AGB_ERR_ARG
    assert lib.agb_single_qubit_gate(0, None, None, 1, 1, None) == _lib.AGB_ERR_ARG
    assert lib.agb_heevd(0, 1, 4, 5, None, None, None, None, 0, 0, None) == _lib.AGB_ERR_ARG
    assert lib.agb_qr(0, None, 4, 4, 0, None, None, 0, None, 0, None) == _lib.AGB_ERR_ARG
    assert lib.agb_cgemm_batched(0, b"X", b"N", 1, 1, 1, 1, None, 1, 1, None, 1, 1, None, 1, 1,
                                 1.0, 0.0, 0.0, 0.0, None) == _lib.AGB_ERR_ARG
    assert lib.agb_heevd_workspace(0, 512, 272) > 512 * 272 * 8


@pytest.mark.skipif(torch.cuda.is_available(), reason="checks the no-GPU failure mode")
def test_product_path_fails_loudly_without_cuda():
    with pytest.raises(RuntimeError):
        atlasq_gb300.AdaptiveMPS(4, bond_dim=1, device="cuda")
    with pytest.raises(RuntimeError):
        atlasq_gb300.AdaptiveMPS(4, bond_dim=1, device="cpu")


def test_host_choose_rank_matches_reference():
    g = load_golden("choose_rank")
    vecs = unpack_spectra(g["lens"], g["flat"])
    for S, (eps, cap, k, el, ent, cond) in zip(vecs, g["meta"]):
        k2, el2, ent2, cond2 = atlasq_gb300.choose_rank_from_sigma(torch.tensor(S), eps, int(cap))
        assert k2 == int(k)
        assert abs(el2 - el) <= 1e-6 * max(1.0, abs(el)) + 1e-12
        assert abs(ent2 - ent) <= 1e-5 * max(1.0, abs(ent))


def test_statistics_api_matches_reference_semantics():
    st = atlasq_gb300.MPSStatistics()
    st.record(step=0, bond=0, k_star=4, chi_before=8, chi_after=4, eps_local=1e-6, entropy=1.5,
              svd_driver="gb300_gram_heevd", dtype="complex64", ms_elapsed=10.0, condS=100.0)
    st.record(step=1, bond=1, k_star=6, chi_before=8, chi_after=6, eps_local=2e-6, entropy=2.0,
              svd_driver="gb300_gram_heevd", dtype="complex64", ms_elapsed=12.0, condS=150.0)
    s = st.summary()
    assert s["total_operations"] == 2 and s["max_chi"] == 6 and s["total_time_ms"] == 22.0
    assert s["cuda_svd_pct"] == 100.0 and s["cpu_fallback_pct"] == 0.0
    assert abs(st.global_error_bound() - np.sqrt(1e-12 + 4e-12)) < 1e-15
    assert abs(atlasq_gb300.bond_entropy_from_S(torch.ones(4) / 2.0) - 2.0) < 1e-6
    assert atlasq_gb300.effective_rank(torch.tensor([1.0, 0.1, 0.01, 0.001]), 0.99) <= 2
    assert set(atlasq_gb300.get_adaptive_mps()) >= {"AdaptiveMPS", "robust_svd", "choose_rank_from_sigma"}


def test_circuit_generators_are_deterministic():
    from atlasq_gb300.circuits import count_two_site, haar_brickwork, hea_circuit, layers_of
    a = haar_brickwork(40, 20, seed=1234)
    b = haar_brickwork(40, 20, seed=1234)
    assert count_two_site(a) == 390
    assert all(torch.equal(x[2], y[2]) for x, y in zip(a, b))
    U = a[0][2].to(torch.complex128)
    assert torch.allclose(U.conj().T @ U, torch.eye(4, dtype=torch.complex128), atol=1e-6)
    h = hea_circuit(64, 12, seed=3)
    assert count_two_site(h) == 756
    lays = layers_of(a)
    assert len(lays) == 20 and sum(len(x) for x in lays) == 390


def test_new_entry_points_validate_arguments_without_a_gpu(lib):
    """Argument checks run before any CUDA call, so they work on a CPU host."""
    P = None
    # batched site mix: bad dtype, null buffers, negative count
    assert lib.agb_site_mix(7, P, P, P, 1, 4, 4, P) == _lib.AGB_ERR_ARG
    assert lib.agb_site_mix(_lib.AGB_C64, P, P, P, 1, 4, 4, P) == _lib.AGB_ERR_ARG
    assert lib.agb_site_mix(_lib.AGB_C64, P, P, P, -1, 4, 4, P) == _lib.AGB_ERR_ARG
    # asynchronous tensor-core GEMM: the device status word is required
    assert lib.agb_cgemm_tc_async(b"N", b"N", 1, 8, 8, 8, P, 8, 64, P, 8, 64, P, 8, 64,
                                  1.0, 0.0, 0.0, 0.0, P, 0, P, P) == _lib.AGB_ERR_ARG
    # the GEMM's wait-limit hook is host state: set, restore (negative = default)
    assert lib.agb_set_gemm_wait_limit(0) == _lib.AGB_OK
    assert lib.agb_set_gemm_wait_limit(-1) == _lib.AGB_OK
    # tridiagonalisation switch: modes 0 and 1 only
    assert lib.agb_set_tridiag_stages(2) == _lib.AGB_ERR_ARG
    assert lib.agb_set_tridiag_stages(1) == _lib.AGB_OK
    # no launch has failed in this process
    assert lib.agb_last_error() == b""


def test_samples_to_counts_formats_like_the_reference():
    """adapters.samples_to_counts: format(sample, '0{n}b') keys (qubit 0 leftmost)."""
    from atlasq_gb300.adapters import samples_to_counts
    c = samples_to_counts(np.array([0, 5, 5, 7]), 3)
    assert c == {"000": 1, "101": 2, "111": 1}
    assert samples_to_counts({"01": 3}) == {"01": 3}
    assert samples_to_counts([2, 2], None) == {"10": 2}


def test_svd_event_log_roundtrip(tmp_path, monkeypatch):
    """svd_log writes the reference's record fields (tools_qih/tn_core.py:247-274)
    to svd_events_*.jsonl.gz under $QIH_SVD_LOG_DIR, and read_events reads them."""
    from atlasq_gb300 import svd_log
    monkeypatch.setenv("QIH_SVD_LOG_DIR", str(tmp_path))
    lg = svd_log.get_logger()
    lg.spectrum(bond=3, pre_rank=16, chi_max=32, tol=1e-8, total_weight=2.0, sigma=[1.0, 0.5, 0.25], keep=2,
                step=7, chi_left=8, chi_right=16, features=[0.1, 0.2, 0.3, 0.4, 0.5], full=16)
    lg.close()
    recs = list(svd_log.read_events(str(tmp_path)))
    assert len(recs) == 1
    r = recs[0]
    for key in ("host", "pid", "run_ts", "kind", "i", "j", "pre_rank", "chi_max", "tol", "adaptive", "entangler",
                "total_weight", "S_top128", "adaptive_keep"):
        assert key in r
    assert r["kind"] == "svd_spectrum" and r["i"] == 3 and r["j"] == 4 and r["adaptive_keep"] == 2
    assert len(r["S_top128"]) == 128 and r["S_top128"][:3] == [1.0, 0.5, 0.25] and r["S_top128"][3] == 0.0
    assert r["features"] == [0.1, 0.2, 0.3, 0.4, 0.5] and r["full"] == 16
    monkeypatch.delenv("QIH_SVD_LOG_DIR")
    assert svd_log.get_logger() is None


def test_pauli_fixture_records_the_reference_deviation():
    """The reference's exp(i lam P) is exact for Pauli strings of length <= 2 and
    not for longer ones (tests/golden/mpo_apply.npz); the package's MPO builder
    (pauli_exp_mpo, CPU tensors) contracts to the exact operator for all."""
    import torch
    from atlasq_gb300.mpo_ops import pauli_exp_mpo
    g = load_golden("mpo_apply")
    P = {"I": np.eye(2), "X": np.array([[0, 1], [1, 0]]), "Y": np.array([[0, -1j], [1j, 0]]), "Z": np.diag([1., -1.])}
    lam = 0.3
    for k, ps in enumerate(str(x) for x in g["pauli_strings"]):
        Pm = np.array([[1.0]])
        for c in ps:
            Pm = np.kron(Pm, P[c])
        op = np.cos(lam) * np.eye(2 ** len(ps)) + 1j * np.sin(lam) * Pm
        exact = op @ g[f"pauli{k}_in"]
        f = abs(np.vdot(exact, g[f"pauli{k}_out"])) ** 2
        assert (f > 1 - 1e-10) == (len(ps) <= 2), (ps, f)
        mpo = pauli_exp_mpo(ps, lam, device="cpu", dtype=torch.complex128)
        T = None
        for W in mpo.tensors:
            T = W if T is None else torch.einsum("...a,astr->...str", T, W)
        n = len(ps)
        T = T.reshape([2] * (2 * n)).permute([2 * i for i in range(n)] + [2 * i + 1 for i in range(n)])
        assert np.allclose(T.reshape(2 ** n, 2 ** n).numpy(), op, atol=1e-12)


def test_promotion_reachability_bound():
    """Resident execution is allowed only where the float32 rank rule cannot
    reach the promotion threshold: sigma_0 / sigma_{k-1} <= sqrt(2 chi_cap 2^26)."""
    import types
    import torch
    from atlasq_gb300.adaptive_mps import AdaptiveMPS, DTypePolicy

    def reach(dt, thr, caps):
        o = types.SimpleNamespace(dtype_policy=DTypePolicy(default=dt, promote_if_cond_gt=thr), chi_max_per_bond=caps)
        return AdaptiveMPS.promotion_reachable(o)
    assert not reach(torch.complex64, 1e6, [256] * 39)      # the default policy at chi 256
    assert not reach(torch.complex64, 1e6, [512] * 63)
    assert reach(torch.complex64, 1e5, [256] * 39)
    assert reach(torch.complex64, 3.0, [16] * 9)
    assert not reach(torch.complex128, 3.0, [16] * 9)        # complex128 never promotes
