"""Device-resident mode (no host synchronisation between gate batches) and
whole-circuit CUDA-graph capture of many instances: same results as the
host-synchronised path and as the reference's golden runs."""
import numpy as np
import pytest
import torch

from conftest import load_golden
from oracle import mps_oracle as mo
from oracle import statevector as sv

pytestmark = pytest.mark.gpu

aq = pytest.importorskip("atlasq_gb300")
from atlasq_gb300.circuits import haar_brickwork, hea_circuit, ry, rz  # noqa: E402

GOLDEN = {
    "brickwork_n12_d10_chi32": lambda: haar_brickwork(12, 10, seed=1234),
    "brickwork_n10_d8_chi16_eps1e-3": lambda: haar_brickwork(10, 8, seed=11),
    "hea_n10_l3_chi16": lambda: hea_circuit(10, 3, seed=3),
}


def _run(ops, n, chi, eps, resident):
    m = aq.AdaptiveMPS(n, bond_dim=1, eps_bond=eps, chi_max_per_bond=chi, device="cuda",
                       device_resident=resident)
    for kind, q, U in ops:
        (m.apply_two_site_gate if kind == "2q" else m.apply_single_qubit_gate)(q, U)
    return m


def _fid(a, b):
    return mo.mps_fidelity([t.cpu().numpy().astype(np.complex128) for t in a.tensors],
                           [t.cpu().numpy().astype(np.complex128) for t in b.tensors])


@pytest.mark.parametrize("name", sorted(GOLDEN))
def test_resident_matches_reference_golden(name):
    g = load_golden(name)
    n, chi, eps = int(g["n"]), int(g["chi"]), float(g["eps"])
    m = _run(GOLDEN[name](), n, chi, eps, resident=True)
    assert m._res is not None  # nothing synchronised yet
    psi = m.to_statevector().cpu().numpy()
    assert m._res is None
    if name.startswith("brickwork"):
        assert list(m.bond_dims) == list(g["bond_dims"])
        assert m.statistics.logs["k_star"] == [int(x) for x in g["log_k_star"]]
        assert np.allclose(m.statistics.logs["eps_local"], g["log_eps_local"], atol=2e-6)
    else:
        assert list(m.bond_dims) in (list(g["bond_dims"]), list(g["bond_dims64"]))
    assert sv.fidelity(psi, g["statevector"]) > 1 - 1e-6


def test_resident_interleaved_reads_and_gates():
    """Reading the state leaves resident mode; the next gate re-enters it."""
    ops = haar_brickwork(10, 6, seed=8)
    a = _run(ops, 10, 16, 1e-8, resident=False)
    b = aq.AdaptiveMPS(10, bond_dim=1, eps_bond=1e-8, chi_max_per_bond=16, device="cuda", device_resident=True)
    for j, (kind, q, U) in enumerate(ops):
        b.apply_two_site_gate(q, U)
        if j % 7 == 3:
            _ = b.bond_dims  # synchronise mid-circuit
    assert a.bond_dims == b.bond_dims
    assert _fid(a, b) > 1 - 1e-6
    assert len(b.statistics.logs["k_star"]) == len(ops)


def test_resident_batch_and_graph_capture_match_host_path():
    rng = np.random.default_rng(12)
    specs = []
    for b in range(10):
        n = int(rng.integers(6, 15))
        chi = int(rng.choice([8, 16, 32]))
        specs.append((n, chi, hea_circuit(n, 3, seed=300 + b)))
    host = [aq.AdaptiveMPS(n, bond_dim=1, eps_bond=1e-8, chi_max_per_bond=chi, device="cuda") for n, chi, _ in specs]
    aq.MPSBatch(host).run([o for _, _, o in specs])
    res = [aq.AdaptiveMPS(n, bond_dim=1, eps_bond=1e-8, chi_max_per_bond=chi, device="cuda", device_resident=True)
           for n, chi, _ in specs]
    aq.MPSBatch(res).run([o for _, _, o in specs]).synchronize()
    # the host path sizes the eigenvector phase from the eigenvalues, the resident
    # path computes every vector: with eps 1e-8 the float32 rule's cut sits at the
    # rounding level, where the two orders of summation may keep one value more
    for a, b in zip(host, res):
        assert max(abs(x - y) for x, y in zip(a.bond_dims, b.bond_dims)) <= 2
        assert _fid(a, b) > 1 - 1e-5
    # whole circuit as one graph, replayed twice from the same start state
    gr = [aq.AdaptiveMPS(n, bond_dim=1, eps_bond=1e-8, chi_max_per_bond=chi, device="cuda", device_resident=True)
          for n, chi, _ in specs]
    cap = aq.MPSBatch(gr).capture([o for _, _, o in specs])
    assert cap.kernels_per_replay > 0
    cap.replay()
    cap.replay()
    cap.finish()
    # the graph replays the resident launches, with the eigensolver's cluster shape
    # autotuned at capture (a different summation order at the rounding level)
    for (n, chi, ops), a, b in zip(specs, res, gr):
        assert max(abs(x - y) for x, y in zip(a.bond_dims, b.bond_dims)) <= 2
        assert _fid(a, b) > 1 - 1e-5
        assert len(b.statistics.logs["k_star"]) == sum(1 for op in ops if op[0] == "2q")


def test_graph_replay_with_rewritten_angles():
    """Same circuit structure, new rotation angles written into the captured
    gate buffers: the replay equals a fresh run with those angles."""
    n, chi = 8, 16
    gen = torch.Generator().manual_seed(2)
    angles = torch.rand(2, n, 2, generator=gen, dtype=torch.float64) * 6.28

    def circuit(a):
        ops = []
        for layer in range(2):
            for q in range(n):
                ops.append(("1q", q, ry(float(a[layer, q, 0])).cuda()))
                ops.append(("1q", q, rz(float(a[layer, q, 1])).cuda()))
            for b in range(n - 1):
                ops.append(("2q", b, torch.diag(torch.tensor([1, 1, 1, -1], dtype=torch.complex64)).cuda()))
        return ops
    ops0 = circuit(angles)
    m = aq.AdaptiveMPS(n, bond_dim=1, eps_bond=1e-8, chi_max_per_bond=chi, device="cuda", device_resident=True)
    cap = aq.MPSBatch([m]).capture([ops0])
    new = angles + 0.3
    ops1 = circuit(new)
    cap.update_gates([ops1])
    cap.replay()
    cap.finish()
    ref = _run(ops1, n, chi, 1e-8, resident=False)
    assert m.bond_dims == ref.bond_dims
    assert _fid(m, ref) > 1 - 1e-6


@pytest.mark.parametrize("resident", [False, True])
def test_complex64_matches_complex128_before_the_cap_binds(resident):
    """40-qubit Haar brickwork, first 150 gates (bonds below chi_max = 256, so
    only the eps = 1e-8 rule truncates): complex64 against complex128 must
    agree to float32 accuracy in both execution modes.  Guards the eigenvector
    phase (a too-short inverse iteration once cost 4e-4 here in one mode)."""
    ops = [op for op in haar_brickwork(40, 20, seed=1234)][:150]
    a = _run(ops, 40, 256, 1e-8, resident)
    pol = aq.DTypePolicy(default=torch.complex128)
    b = aq.AdaptiveMPS(40, bond_dim=1, eps_bond=1e-8, chi_max_per_bond=256, device="cuda",
                       dtype=torch.complex128, dtype_policy=pol)
    for _, q, U in ops:
        b.apply_two_site_gate(q, U)
    assert _fid(a, b) > 1 - 1e-6
