"""Rank-predictor MLP: CPU checks of the float64 oracle and of the gate
features; GPU checks of the forward / backward / AdamW kernels against the
oracle, of training, and of the predictor's gain on a Trotter circuit.

The reference's predictor (src/atlas_q/tools_qih/ai_rank_predictor.py:14-89)
has no GPU kernels to pin against; the kernels are pinned to the oracle here,
and the oracle's gradient to central finite differences.
"""
import math

import numpy as np
import pytest
import torch

from oracle import mlp_oracle as mo


def _batch(seed, B):
    rng = np.random.default_rng(seed)
    X = rng.uniform(0, 1, size=(B, 5))
    T = rng.uniform(0.05, 0.95, size=B)
    return X, T


def test_oracle_gradient_finite_differences():
    p = mo.init_params(3)
    X, T = _batch(1, 16)
    _, g = mo.loss_and_grad(p, X, T)
    rng = np.random.default_rng(7)
    idx = rng.choice(mo.NPARAM, size=60, replace=False)
    h = 1e-6
    for j in idx:
        e = np.zeros_like(p)
        e[j] = h
        fd = (mo.loss_and_grad(p + e, X, T)[0] - mo.loss_and_grad(p - e, X, T)[0]) / (2 * h)
        assert abs(fd - g[j]) <= 1e-6 * max(1.0, abs(g[j])) + 1e-9, (j, fd, g[j])


def test_oracle_layout_matches_header():
    from atlasq_gb300 import _lib
    assert mo.NPARAM == _lib.MLP_NPARAM == 8769


def test_entangling_power_known_values():
    from atlasq_gb300.rank_predictor import entangling_power
    from atlasq_gb300.circuits import CZ, rzz
    cnot = np.eye(4)[[0, 1, 3, 2]]
    swap = np.eye(4)[[0, 2, 1, 3]]
    ep = entangling_power(np.stack([np.eye(4), cnot, CZ.numpy(), swap, np.kron(np.eye(2), np.eye(2)[[1, 0]])]))
    np.testing.assert_allclose(ep, [0, 2 / 9, 2 / 9, 0, 0], atol=1e-12)
    # RZZ(theta): e_p = (2/9) sin^2(theta)
    for th in (0.1, 0.7, 1.3):
        np.testing.assert_allclose(entangling_power(rzz(th).numpy()), [(2 / 9) * math.sin(th) ** 2], atol=1e-7)


# ---------------------------------------------------------------- GPU kernels
def _kernel_predictor(seed=3):
    from atlasq_gb300.rank_predictor import RankPredictor
    return RankPredictor(params=torch.from_numpy(mo.init_params(seed)).float())


@pytest.mark.gpu
def test_mlp_forward_matches_oracle():
    rp = _kernel_predictor()
    X, _ = _batch(2, 1000)
    y = rp.predict_fraction(X).cpu().numpy()
    p = rp.params.cpu().double().numpy()
    yo, _ = mo.forward(p, X.astype(np.float32))
    np.testing.assert_allclose(y, yo, rtol=2e-5, atol=2e-6)


@pytest.mark.gpu
@pytest.mark.parametrize("B", [1, 37, 128, 1000])
def test_mlp_backward_matches_oracle(B):
    rp = _kernel_predictor()
    X, T = _batch(4 + B, B)
    loss, g = rp.loss_and_grad(X, T)
    p = rp.params.cpu().double().numpy()
    lo, go = mo.loss_and_grad(p, X.astype(np.float32), T.astype(np.float32))
    g = g.cpu().double().numpy()
    assert abs(float(loss) - lo) <= 1e-5 * lo + 1e-9
    # relative error of the full gradient vector (fp32 kernels vs float64 oracle)
    assert np.linalg.norm(g - go) <= 1e-4 * np.linalg.norm(go), np.linalg.norm(g - go) / np.linalg.norm(go)


@pytest.mark.gpu
def test_mlp_training_is_deterministic():
    """The gradient reductions run in a fixed order (no float atomics): two
    trainings from the same start on the same minibatches end bit-identical."""
    from atlasq_gb300.rank_predictor import RankPredictor
    X, T = _batch(11, 3000)
    outs = []
    for _ in range(2):
        rp = RankPredictor(seed=3)
        rp.train(X, T, steps=60, batch=1000, lr=3e-3)
        outs.append(rp.params.cpu().numpy().copy())
    assert np.array_equal(outs[0], outs[1])


@pytest.mark.gpu
def test_mlp_adam_matches_oracle():
    from atlasq_gb300 import _lib
    from atlasq_gb300._lib import check, ptr, stream_ptr
    import ctypes
    lib = _lib.load()
    rng = np.random.default_rng(5)
    p0 = rng.standard_normal(mo.NPARAM).astype(np.float32)
    pd = torch.from_numpy(p0).cuda()
    md = torch.zeros_like(pd)
    vd = torch.zeros_like(pd)
    p, m, v = p0.astype(np.float64), np.zeros(mo.NPARAM), np.zeros(mo.NPARAM)
    for step in range(1, 6):
        g = rng.standard_normal(mo.NPARAM).astype(np.float32)
        gd = torch.from_numpy(g).cuda()
        check(lib.agb_mlp_adam(ptr(pd), ptr(gd), ptr(md), ptr(vd), step, ctypes.c_float(1e-2), ctypes.c_float(0.9),
                               ctypes.c_float(0.999), ctypes.c_float(1e-8), ctypes.c_float(1e-3),
                               stream_ptr(pd.device)), "adam")
        p, m, v = mo.adam_step(p, g.astype(np.float64), m, v, step, 1e-2, wd=1e-3)
    np.testing.assert_allclose(pd.cpu().numpy(), p, rtol=1e-5, atol=1e-6)


@pytest.mark.gpu
def test_mlp_training_reduces_loss():
    from atlasq_gb300.rank_predictor import RankPredictor
    rng = np.random.default_rng(0)
    X = rng.uniform(0, 1, size=(4096, 5)).astype(np.float32)
    T = (0.2 + 0.6 * X[:, 0] * X[:, 2] + 0.1 * np.sin(6 * X[:, 1])).astype(np.float32)
    rp = RankPredictor(seed=1)
    hist = rp.train(X, T, steps=300, batch=512, lr=3e-3)
    assert hist[-1] < 0.1 * hist[0], hist
    assert hist[-1] < 2e-3, hist


def _run(ops, n, chi, eps, predictor=None):
    from atlasq_gb300 import AdaptiveMPS
    m = AdaptiveMPS(n, bond_dim=1, eps_bond=eps, chi_max_per_bond=chi, device="cuda")
    m.rank_predictor = predictor
    for kind, q, U in ops:
        if kind == "2q":
            m.apply_two_site_gate(q, U)
        else:
            m.apply_single_qubit_gate(q, U)
    m.flush()
    return m


@pytest.mark.gpu
def test_rank_predictor_gain_on_trotter_circuit():
    """Trained on plain runs of six circuits, the predictor sizes the
    eigensolver of a seventh: fewer eigenpairs in total (fallback re-runs
    included), few fallbacks, and the same fidelity to the exact state as the
    plain run.  (Bond dimensions are not compared one by one: with float32
    spectra a rank at the cutoff moves by one or two with the order of
    floating-point sums, in the reference's own complex64 vs complex128 runs
    too, and a truncated circuit amplifies such differences.)"""
    from atlasq_gb300.circuits import trotter_ising
    from atlasq_gb300.rank_predictor import RankPredictor, collect_training_data
    from oracle import statevector as sv
    n, chi, eps, steps, dtr = 16, 128, 1e-3, 20, (0.05, 0.25)
    circ = lambda sd: trotter_ising(n, steps, sd, dt_range=dtr)  # noqa: E731
    X, T = collect_training_data(circ, range(6), n, chi, eps)
    assert len(T) > 1000
    rp = RankPredictor(seed=0)
    hist = rp.train(X, T, steps=600, batch=512, lr=3e-3)
    assert hist[-1] < 0.5 * hist[0], hist
    ops = circ(11)
    plain = _run(ops, n, chi, eps)
    pred = _run(ops, n, chi, eps, predictor=rp)
    gates = sum(1 for op in ops if op[0] == "2q")
    assert pred.ell_total <= 0.92 * plain.ell_total, (pred.ell_total, plain.ell_total)
    assert pred.rank_fallbacks <= 0.15 * gates, pred.rank_fallbacks
    exact = sv.zero_state(n)
    for kind, q, U in ops:
        U = U.numpy().astype(np.complex128)
        exact = sv.apply_two_qubit(exact, n, q, U) if kind == "2q" else sv.apply_single_qubit_transposed(exact, n, q, U)
    fa = sv.fidelity(plain.to_statevector().cpu().numpy(), exact)
    fb = sv.fidelity(pred.to_statevector().cpu().numpy(), exact)
    assert abs(fa - fb) <= 2e-3, (fa, fb)


@pytest.mark.gpu
def test_rank_fallback_reruns_match_plain_run():
    """A predictor that always under-sizes (ell = 1) sends every truncating gate
    through the re-run at full size: the state must equal the plain run's."""
    from atlasq_gb300.circuits import trotter_ising
    from oracle.mps_oracle import mps_fidelity
    n, chi, eps = 12, 64, 1e-3
    ops = trotter_ising(n, 10, 3)
    plain = _run(ops, n, chi, eps)
    low = _run(ops, n, chi, eps, predictor=lambda mps, gates: [1] * len(gates))
    assert low.rank_fallbacks > 0
    assert low.bond_dims == plain.bond_dims
    ta = [t.cpu().numpy().astype(np.complex128) for t in plain.tensors]
    tb = [t.cpu().numpy().astype(np.complex128) for t in low.tensors]
    assert mps_fidelity(ta, tb) >= 1 - 1e-6


def test_training_data_from_svd_events(tmp_path):
    """The training pairs are read back from the SVD-event log: features and
    kept rank / full size from records that carry them, others skipped."""
    from atlasq_gb300 import svd_log
    from atlasq_gb300.rank_predictor import training_data_from_events
    lg = svd_log.SVDEventLogger(str(tmp_path))
    lg.spectrum(bond=1, pre_rank=4, chi_max=32, tol=1e-8, total_weight=1.0, sigma=[1.0], keep=6, step=0,
                chi_left=4, chi_right=8, features=[0.2, 0.3, 0.5, 0.1, 1.0], full=8)
    lg.spectrum(bond=2, pre_rank=4, chi_max=32, tol=1e-8, total_weight=1.0, sigma=[1.0], keep=3, step=1,
                chi_left=4, chi_right=8)
    lg.spectrum(bond=3, pre_rank=8, chi_max=32, tol=1e-8, total_weight=1.0, sigma=[1.0], keep=16, step=2,
                chi_left=8, chi_right=8, features=[0.3, 0.3, 0.9, 0.2, 0.5], full=16)
    lg.close()
    X, T = training_data_from_events(svd_log.read_events(str(tmp_path)))
    assert X.shape == (2, 5) and X.dtype == np.float32
    np.testing.assert_allclose(T, [0.75, 1.0])
    np.testing.assert_allclose(X[1], [0.3, 0.3, 0.9, 0.2, 0.5], rtol=1e-6)


@pytest.mark.gpu
def test_training_pipeline_logs_trains_and_saves(tmp_path):
    """log_plain_runs -> training_data_from_events -> train -> save / load on
    a small hardware-efficient ansatz: one event per two-site gate, and the
    reloaded network predicts what the trained one does."""
    from atlasq_gb300 import svd_log
    from atlasq_gb300.circuits import hea_circuit
    from atlasq_gb300.rank_predictor import (RankPredictor, load_predictor, log_plain_runs, save_predictor,
                                             training_data_from_events)
    n, layers = 12, 4
    path = log_plain_runs(lambda sd: hea_circuit(n, layers, seed=sd), [1, 2, 3], n, 32, 1e-8, str(tmp_path))
    X, T = training_data_from_events(svd_log.read_events(path))
    assert len(T) == 3 * layers * (n - 1)
    assert np.all((T > 0) & (T <= 1))
    rp = RankPredictor(seed=0)
    hist = rp.train(X, T, steps=200)
    assert hist[-1] < hist[0]
    out = str(tmp_path / "w.npz")
    save_predictor(rp, out, note="test")
    rp2 = load_predictor(out)
    a = rp.predict_fraction(X).cpu().numpy()
    b = rp2.predict_fraction(X).cpu().numpy()
    assert np.array_equal(a, b)
