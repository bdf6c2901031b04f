"""Generate golden fixtures by running the reference ATLAS-Q implementation.

Run in a container that has the reference source checked out (read-only):

    python tests/golden/make_golden.py [/path/to/ATLAS-Q]

It imports the reference's own ``atlas_q`` package on the CPU (torch), issues
seeded call sequences and stores inputs and outputs as small ``.npz`` files in
this directory.  The reference imports matplotlib through ``vqe_qaoa``; a
do-nothing stand-in is registered in ``sys.modules`` before the import (it is
never called on the paths used here).  Nothing here is needed at test time:
the committed ``.npz`` files are the fixtures.
"""
import os
import sys
import types

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
REF = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"


def _stub_matplotlib():
    mpl = types.ModuleType("matplotlib")
    mpl.use = lambda *a, **k: None
    plt = types.ModuleType("matplotlib.pyplot")
    plt.__getattr__ = lambda name: (lambda *a, **k: None)
    mpl.pyplot = plt
    sys.modules.setdefault("matplotlib", mpl)
    sys.modules.setdefault("matplotlib.pyplot", plt)


_stub_matplotlib()
sys.path.insert(0, os.path.join(REF, "src"))
sys.path.insert(0, REPO)
import atlas_q.adaptive_mps as am  # noqa: E402
from atlas_q.adaptive_mps import AdaptiveMPS, DTypePolicy  # noqa: E402
from atlas_q.mpo_ops import MPOBuilder, correlation_function, expectation_value  # noqa: E402
from atlas_q.truncation import choose_rank_from_sigma  # noqa: E402

from atlasq_gb300.circuits import haar_brickwork, hea_circuit  # noqa: E402

assert am.fused_two_qubit_gate_pytorch is not None, "reference must use the fused two-qubit path"
torch.set_num_threads(max(1, os.cpu_count() or 1))

_REC = []
_orig_svd = am.robust_svd


def _recording_svd(X):
    U, S, Vh, d = _orig_svd(X)
    _REC.append(S.detach().cpu().numpy().copy())
    return U, S, Vh, d


am.robust_svd = _recording_svd


def run_ref(ops, n, chi, eps, dtype=torch.complex64):
    _REC.clear()
    policy = DTypePolicy(default=dtype)
    mps = AdaptiveMPS(n, bond_dim=1, eps_bond=eps, chi_max_per_bond=chi, device="cpu",
                      dtype=dtype, dtype_policy=policy)
    for kind, q, U in ops:
        if kind == "2q":
            mps.apply_two_site_gate(q, U.to(dtype))
        else:
            mps.apply_single_qubit_gate(q, U.to(dtype))
    spectra = list(_REC)
    return mps, spectra


def pack_spectra(spectra):
    lens = np.array([len(s) for s in spectra], dtype=np.int64)
    flat = np.concatenate(spectra) if spectra else np.zeros(0)
    return lens, flat


def pack_tensors(tensors):
    shapes = np.array([t.shape for t in tensors], dtype=np.int64)
    flat = np.concatenate([t.detach().cpu().numpy().reshape(-1) for t in tensors])
    return shapes, flat


def circuit_record(name, ops, n, chi, eps, with_fp64=True):
    out = {}
    mps, spectra = run_ref(ops, n, chi, eps)
    lens, flat = pack_spectra(spectra)
    out["sv_lens"], out["sv_flat"] = lens, flat
    logs = mps.statistics.logs
    for key in ("k_star", "chi_before", "eps_local", "entropy", "condS", "bond"):
        out["log_" + key] = np.array(logs[key], dtype=np.float64)
    out["bond_dims"] = np.array(mps.bond_dims, dtype=np.int64)
    out["tensor_shapes"], out["tensor_flat"] = pack_tensors(mps.tensors)
    if n <= 20:
        out["statevector"] = mps.to_statevector().detach().cpu().numpy()
    if with_fp64:
        mps64, spectra64 = run_ref(ops, n, chi, eps, dtype=torch.complex128)
        l64, f64 = pack_spectra(spectra64)
        out["sv64_lens"], out["sv64_flat"] = l64, f64
        out["bond_dims64"] = np.array(mps64.bond_dims, dtype=np.int64)
        if n <= 20:
            out["statevector64"] = mps64.to_statevector().detach().cpu().numpy()
    np.savez_compressed(os.path.join(HERE, name + ".npz"), n=n, chi=chi, eps=eps, **out)
    print(name, "gates", len(spectra), "bond_dims", list(mps.bond_dims))


def choose_rank_cases():
    rng = np.random.default_rng(7)
    cases = []
    vecs = [np.array([1.0, 0.5, 0.1, 0.01, 0.001]), np.ones(10), np.ones(4) / 2.0,
            np.array([1.0, 0.0, 0.0, 0.0]), np.array([1e-20, 1e-21])]
    for _ in range(12):
        m = int(rng.integers(2, 300))
        s = np.sort(np.abs(rng.standard_normal(m)) * 10.0 ** rng.uniform(-6, 0, m))[::-1]
        vecs.append(s)
    for s in vecs:
        for eps in (1e-1, 1e-2, 1e-3, 1e-6, 1e-8, 1e-10):
            for cap in (3, 64, 1000):
                S = torch.tensor(np.ascontiguousarray(s), dtype=torch.float32)
                k, el, ent, cond = choose_rank_from_sigma(S, eps, cap)
                cases.append((S.numpy().copy(), eps, cap, k, el, ent, cond))
    lens = np.array([len(c[0]) for c in cases])
    flat = np.concatenate([c[0] for c in cases]).astype(np.float32)
    meta = np.array([[c[1], c[2], c[3], c[4], c[5], c[6]] for c in cases], dtype=np.float64)
    np.savez_compressed(os.path.join(HERE, "choose_rank.npz"), lens=lens, flat=flat, meta=meta)
    print("choose_rank cases", len(cases))


def known_answers():
    out = {}
    X = torch.tensor([[0, 1], [1, 0]], dtype=torch.complex64)
    H = torch.tensor([[1, 1], [1, -1]], dtype=torch.complex64) / np.sqrt(2)
    CNOT = torch.tensor([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 0, 1], [0, 0, 1, 0]], dtype=torch.complex64)
    # RY convention (single-qubit gates apply U^T)
    m = AdaptiveMPS(2, bond_dim=1, device="cpu")
    th = 0.7
    RY = torch.tensor([[np.cos(th / 2), -np.sin(th / 2)], [np.sin(th / 2), np.cos(th / 2)]],
                      dtype=torch.complex64)
    m.apply_single_qubit_gate(0, RY)
    out["ry07_state"] = m.to_statevector().numpy()
    # Bell pair
    m = AdaptiveMPS(2, bond_dim=1, eps_bond=1e-10, chi_max_per_bond=4, device="cpu")
    m.apply_single_qubit_gate(0, H)
    m.apply_two_site_gate(0, CNOT)
    out["bell_state"] = m.to_statevector().numpy()
    out["bell_bond"] = np.array(m.bond_dims)
    out["bell_entropy"] = np.array(m.statistics.logs["entropy"])
    # GHZ(6)
    m = AdaptiveMPS(6, bond_dim=1, eps_bond=1e-10, chi_max_per_bond=8, device="cpu")
    m.apply_single_qubit_gate(0, H)
    for i in range(5):
        m.apply_two_site_gate(i, CNOT)
    out["ghz6_state"] = m.to_statevector().numpy()
    out["ghz6_bonds"] = np.array(m.bond_dims)
    # two-qubit gate ordering: U applied to |00> gives U[:,0]
    g = torch.Generator().manual_seed(99)
    from atlasq_gb300.circuits import haar_unitary
    U = haar_unitary(g)
    m = AdaptiveMPS(2, bond_dim=1, eps_bond=1e-10, chi_max_per_bond=4, device="cpu")
    m.apply_two_site_gate(0, U)
    out["u4"] = U.numpy()
    out["u4_state"] = m.to_statevector().numpy()
    # expectation known answers (reference tests/unit/test_mpo_ops.py:213-283)
    Z = torch.tensor([[1, 0], [0, -1]], dtype=torch.complex64)
    m = AdaptiveMPS(3, bond_dim=2, device="cpu")
    m.apply_single_qubit_gate(1, X)
    out["z1_on_010"] = np.array([expectation_value(MPOBuilder.local_operator(Z, 1, 3, device="cpu"), m)])
    np.savez_compressed(os.path.join(HERE, "known_answers.npz"), **out)
    print("known answers written")


def expectations_record():
    """Pauli expectations on a seeded entangled state, via the reference's
    correlation_function / expectation_value.  Includes Y to pin the transpose
    convention of the expectation einsum."""
    n, chi = 10, 16
    ops = haar_brickwork(n, 6, seed=2024)
    mps, _ = run_ref(ops, n, chi, 1e-8)
    Xo = torch.tensor([[0, 1], [1, 0]], dtype=torch.complex64)
    Yo = torch.tensor([[0, -1j], [1j, 0]], dtype=torch.complex64)
    Zo = torch.tensor([[1, 0], [0, -1]], dtype=torch.complex64)
    zz = [correlation_function(Zo, i, Zo, i + 1, mps) for i in range(n - 1)]
    xs = [expectation_value(MPOBuilder.local_operator(Xo, i, n, device="cpu"), mps) for i in range(n)]
    ys = [expectation_value(MPOBuilder.local_operator(Yo, i, n, device="cpu"), mps) for i in range(n)]
    xy = [correlation_function(Xo, i, Yo, i + 2, mps) for i in range(n - 2)]
    shapes, flat = pack_tensors(mps.tensors)
    np.savez_compressed(os.path.join(HERE, "expectations.npz"), n=n, tensor_shapes=shapes,
                        tensor_flat=flat, zz=np.array(zz), x=np.array(xs), y=np.array(ys),
                        xy=np.array(xy), statevector=mps.to_statevector().numpy())
    print("expectations written")


def canonical_record():
    """Reference canonical sweeps on a seeded state (state must be unchanged,
    tensors orthonormal)."""
    n, chi = 8, 8
    ops = haar_brickwork(n, 5, seed=77)
    mps, _ = run_ref(ops, n, chi, 1e-8)
    before = mps.to_statevector().numpy()
    mps.canonicalize_right_to_left()
    right = mps.to_statevector().numpy()
    rshapes, rflat = pack_tensors(mps.tensors)
    mps.to_mixed_canonical(3)
    mixed = mps.to_statevector().numpy()
    mps.to_left_canonical()
    left = mps.to_statevector().numpy()
    mps2, _ = run_ref(ops, n, chi, 1e-8)
    ishapes, iflat = pack_tensors(mps2.tensors)
    np.savez_compressed(os.path.join(HERE, "canonical.npz"), n=n, before=before, right=right,
                        mixed=mixed, left=left, right_shapes=rshapes, right_flat=rflat,
                        in_shapes=ishapes, in_flat=iflat)
    print("canonical written")


def mpo_record():
    """apply_mpo_to_mps and apply_pauli_exp_to_mps (src/atlas_q/mpo_ops.py:1034-1082,
    1296-1358) and the three TDVP contractions of
    src/triton_kernels/tdvp_mpo_ops.py:38-106, run by the reference on seeded
    inputs.  The Pauli cases include strings of length >= 3, where the
    reference's two-rail MPO drops the letters from the third site on."""
    from atlas_q.mpo_ops import apply_mpo_to_mps, apply_pauli_exp_to_mps
    import triton_kernels.tdvp_mpo_ops as tdo
    out = {}
    n = 6
    ops = haar_brickwork(n, 4, seed=314)
    mps, _ = run_ref(ops, n, 8, 1e-10, dtype=torch.complex128)
    out["mpo_in_shapes"], out["mpo_in_flat"] = pack_tensors(mps.tensors)
    Zo = torch.tensor([[1, 0], [0, -1]], dtype=torch.complex128)
    Xo = torch.tensor([[0, 1], [1, 0]], dtype=torch.complex128)
    Yo = torch.tensor([[0, -1j], [1j, 0]], dtype=torch.complex128)
    H = MPOBuilder.sum_local_operators(n, [(i, Zo) for i in range(n)] + [(2, Yo)], device="cpu",
                                       dtype=torch.complex128)
    res = apply_mpo_to_mps(H, mps)
    out["mpo_sum_state"] = res.to_statevector().numpy()
    P = MPOBuilder.local_operator(Yo, 3, n, device="cpu", dtype=torch.complex128)
    out["mpo_local_state"] = apply_mpo_to_mps(P, mps).to_statevector().numpy()
    strings = ["XY", "ZX", "XYZ", "ZXXY"]
    for k, ps in enumerate(strings):
        m = AdaptiveMPS(len(ps), bond_dim=1, device="cpu", dtype=torch.complex128,
                        dtype_policy=DTypePolicy(default=torch.complex128))
        Hd = torch.tensor([[1, 1], [1, -1]], dtype=torch.complex128) / np.sqrt(2)
        for q in range(len(ps)):
            m.apply_single_qubit_gate(q, Hd)
        m.apply_two_site_gate(0, haar_brickwork(2, 1, seed=9 + k)[0][2].to(torch.complex128))
        out[f"pauli{k}_in"] = m.to_statevector().numpy()
        apply_pauli_exp_to_mps(m, ps, 1j * 0.5, 0.6)
        out[f"pauli{k}_out"] = m.to_statevector().numpy()
    out["pauli_strings"] = np.array(strings)
    g = torch.Generator().manual_seed(2718)

    def cr(*shape):
        return torch.complex(torch.randn(*shape, generator=g, dtype=torch.float64),
                             torch.randn(*shape, generator=g, dtype=torch.float64))
    L, A, W, R = cr(7, 3, 5), cr(5, 2, 6), cr(3, 2, 2, 4), cr(6, 4, 6)
    out["tdvp_L"], out["tdvp_A"], out["tdvp_W"], out["tdvp_R"] = (t.numpy() for t in (L, A, W, R))
    out["tdvp_left"] = tdo.tdvp_left_environment_init_optimized(cr(5, 3, 5) * 0 + L[:5], A, W).numpy()
    out["tdvp_left_in"] = L[:5].numpy()
    out["tdvp_right"] = tdo.tdvp_right_environment_init_optimized(R, A, W).numpy()
    out["tdvp_local"] = tdo.tdvp_apply_local_H_optimized(L, W, A, R).numpy()
    np.savez_compressed(os.path.join(HERE, "mpo_apply.npz"), **out)
    print("mpo / pauli / tdvp written")


def qiskit_record():
    """The reference backend's MPS route (ATLASQBackend._run_mps,
    src/atlas_q/adapters/qiskit_adapter.py:383-404) on tests/qiskit_like.py's
    six-qubit circuit: its statevector (the counts are torch.multinomial
    draws and are compared by distribution only)."""
    import warnings
    sys.path.insert(0, os.path.join(REPO, "tests"))
    from qiskit_like import sample_circuit
    import importlib.util
    # the adapters package also imports its Cirq adapter, which needs Cirq;
    # load the Qiskit adapter's module file on its own
    spec = importlib.util.spec_from_file_location(
        "qiskit_adapter_ref", os.path.join(REF, "src", "atlas_q", "adapters", "qiskit_adapter.py"))
    qa = importlib.util.module_from_spec(spec)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        spec.loader.exec_module(qa)
    fake = types.SimpleNamespace(_max_bond_dim=128)
    fake._apply_gate_to_mps = lambda mps, name, qubits, params: qa.ATLASQBackend._apply_gate_to_mps(
        fake, mps, name, qubits, params)
    fake._samples_to_counts = lambda samples, n=None: qa.ATLASQBackend._samples_to_counts(fake, samples, n)
    angle = lambda v: torch.tensor(v, dtype=torch.float64)  # noqa: E731
    counts, sv = qa.ATLASQBackend._run_mps(fake, sample_circuit(angle), 4000, 7)
    np.savez_compressed(os.path.join(HERE, "qiskit_mps.npz"), statevector=sv.numpy(), shots=4000,
                        count_keys=np.array(sorted(counts)), count_vals=np.array([counts[k] for k in sorted(counts)]))
    print("qiskit route written")


def headline_record(seeds=(1234, 1235, 1236), pinned=150, checkpoints=(150, 250, 330, 390)):
    """The 40-qubit Haar brickwork (depth 20, chi_max 256, eps 1e-8) through the
    reference in complex64 and in complex128, gate by gate in lockstep.  Kept:
    for the first seed, the per-gate kept singular values (complex64) and logs
    of the first `pinned` gates, and the kept ranks of every gate in both
    precisions; for every seed, the complex64-vs-complex128 fidelity at the
    checkpoints (the reference's own float32 drift once the chi cap binds)."""
    from oracle import mps_oracle as mo
    out = {"seeds": np.array(seeds), "checkpoints": np.array(checkpoints)}
    fids = np.zeros((len(seeds), len(checkpoints)))
    for si, seed in enumerate(seeds):
        ops = haar_brickwork(40, 20, seed=seed)
        runs = {}
        for dt in (torch.complex64, torch.complex128):
            runs[dt] = AdaptiveMPS(40, bond_dim=1, eps_bond=1e-8, chi_max_per_bond=256, device="cpu", dtype=dt,
                                   dtype_policy=DTypePolicy(default=dt))
        spectra = []
        for g, (_, q, U) in enumerate(ops):
            _REC.clear()
            runs[torch.complex64].apply_two_site_gate(q, U.to(torch.complex64))
            if g < pinned:
                spectra.append(_REC[-1].astype(np.float32))
            runs[torch.complex128].apply_two_site_gate(q, U.to(torch.complex128))
            if g + 1 in checkpoints:
                a = [t.numpy() for t in runs[torch.complex64].tensors]
                b = [t.numpy() for t in runs[torch.complex128].tensors]
                fids[si, list(checkpoints).index(g + 1)] = mo.mps_fidelity(a, b)
        print("headline seed", seed, "fidelity c64 vs c128 at", list(checkpoints), fids[si])
        if si == 0:
            l64 = runs[torch.complex64].statistics.logs
            k = [int(x) for x in l64["k_star"]]
            out["k64"] = np.array(k, dtype=np.int64)
            out["k128"] = np.array(runs[torch.complex128].statistics.logs["k_star"], dtype=np.int64)
            kept = [sp[:kk] for sp, kk in zip(spectra, k[:pinned])]
            out["sv_lens"], out["sv_flat"] = pack_spectra(kept)
            for key in ("eps_local", "entropy", "condS"):
                out["log_" + key] = np.array(l64[key][:pinned], dtype=np.float64)
    out["fid_c64_c128"] = fids
    np.savez_compressed(os.path.join(HERE, "brickwork_n40_d20_chi256.npz"), n=40, chi=256, eps=1e-8,
                        depth=20, pinned=pinned, **out)


if __name__ == "__main__":
    choose_rank_cases()
    known_answers()
    circuit_record("brickwork_n12_d10_chi32", haar_brickwork(12, 10, seed=1234), 12, 32, 1e-10)
    circuit_record("brickwork_n8_d6_chi8", haar_brickwork(8, 6, seed=5), 8, 8, 1e-6)
    circuit_record("brickwork_n10_d8_chi16_eps1e-3", haar_brickwork(10, 8, seed=11), 10, 16, 1e-3)
    circuit_record("hea_n10_l3_chi16", hea_circuit(10, 3, seed=3), 10, 16, 1e-8)
    expectations_record()
    canonical_record()
    mpo_record()
    qiskit_record()
    headline_record()
