"""Many MPS instances per launch sequence (MPSBatch): every instance must give
the result it gives alone, and the reference's golden results where it has
them."""
import numpy as np
import pytest
import torch

from conftest import load_golden
from oracle import mps_oracle as mo
from oracle import statevector as sv

pytestmark = pytest.mark.gpu

aq = pytest.importorskip("atlasq_gb300")
from atlasq_gb300.circuits import haar_brickwork, hea_circuit  # noqa: E402

GOLDEN = {
    "brickwork_n12_d10_chi32": lambda: haar_brickwork(12, 10, seed=1234),
    "brickwork_n8_d6_chi8": lambda: haar_brickwork(8, 6, seed=5),
    "brickwork_n10_d8_chi16_eps1e-3": lambda: haar_brickwork(10, 8, seed=11),
    "hea_n10_l3_chi16": lambda: hea_circuit(10, 3, seed=3),
}


def _solo(ops, n, chi, eps):
    m = aq.AdaptiveMPS(n, bond_dim=1, eps_bond=eps, chi_max_per_bond=chi, device="cuda")
    for kind, q, U in ops:
        (m.apply_two_site_gate if kind == "2q" else m.apply_single_qubit_gate)(q, U)
    m.flush()
    return m


def test_batch_matches_reference_golden():
    names = sorted(GOLDEN)
    insts, circs, gold = [], [], []
    for nm in names:
        g = load_golden(nm)
        n, chi, eps = int(g["n"]), int(g["chi"]), float(g["eps"])
        insts.append(aq.AdaptiveMPS(n, bond_dim=1, eps_bond=eps, chi_max_per_bond=chi, device="cuda"))
        circs.append(GOLDEN[nm]())
        gold.append(g)
    batch = aq.MPSBatch(insts).run(circs)
    assert batch.rounds < sum(sum(1 for op in c if op[0] == "2q") for c in circs)
    for nm, m, g in zip(names, insts, gold):
        psi = m.to_statevector().cpu().numpy()
        if nm.startswith("brickwork"):
            assert list(m.bond_dims) == list(g["bond_dims"]), nm
            assert m.statistics.logs["k_star"] == [int(x) for x in g["log_k_star"]], nm
        else:
            assert list(m.bond_dims) in (list(g["bond_dims"]), list(g["bond_dims64"])), nm
        assert sv.fidelity(psi, g["statevector"]) > 1 - 1e-6, nm


def test_uneven_instances_match_solo_runs():
    rng = np.random.default_rng(4)
    specs = []
    for b in range(12):
        n = int(rng.integers(6, 17))
        chi = int(rng.choice([8, 16, 32, 64]))
        ops = hea_circuit(n, 4, seed=100 + b) if b % 2 else haar_brickwork(n, 6, seed=100 + b)
        specs.append((n, chi, 1e-8, ops))
    insts = [aq.AdaptiveMPS(n, bond_dim=1, eps_bond=eps, chi_max_per_bond=chi, device="cuda")
             for n, chi, eps, _ in specs]
    aq.MPSBatch(insts).run([s[3] for s in specs])
    for (n, chi, eps, ops), m in zip(specs, insts):
        s = _solo(ops, n, chi, eps)
        assert m.bond_dims == s.bond_dims
        f = mo.mps_fidelity([t.cpu().numpy().astype(np.complex128) for t in m.tensors],
                            [t.cpu().numpy().astype(np.complex128) for t in s.tensors])
        assert f > 1 - 1e-6, (n, chi, f)
        if 2 ** (n // 2) <= chi:  # no truncation by the cap: compare with the exact state
            ref = sv.zero_state(n)
            for kind, q, U in ops:
                if kind == "2q":
                    ref = sv.apply_two_qubit(ref, n, q, U.numpy().astype(np.complex128))
                else:
                    ref = sv.apply_single_qubit_transposed(ref, n, q, U.numpy().astype(np.complex128))
            assert sv.fidelity(m.to_statevector().cpu().numpy(), ref) > 1 - 1e-5


def test_batch_statistics_are_per_instance():
    a = aq.AdaptiveMPS(8, bond_dim=1, eps_bond=1e-8, chi_max_per_bond=16, device="cuda")
    b = aq.AdaptiveMPS(11, bond_dim=1, eps_bond=1e-8, chi_max_per_bond=8, device="cuda")
    ca, cb = haar_brickwork(8, 4, seed=1), haar_brickwork(11, 5, seed=2)
    aq.MPSBatch([a, b]).run([ca, cb])
    assert len(a.statistics.logs["k_star"]) == sum(1 for op in ca if op[0] == "2q")
    assert len(b.statistics.logs["k_star"]) == sum(1 for op in cb if op[0] == "2q")
    assert max(b.bond_dims) <= 8 and max(a.bond_dims) <= 16


@pytest.mark.parametrize("dt", [torch.complex64, torch.complex128])
def test_single_qubit_batch_equals_sequential(dt):
    """Queued single-qubit gates (one launch for all sites and instances) give
    bit-identical tensors to applying each gate with its own launch."""
    from atlasq_gb300 import ops
    from atlasq_gb300.adaptive_mps import apply_single_qubit_entries
    gen = torch.Generator().manual_seed(9)
    insts = [aq.AdaptiveMPS(n, bond_dim=1, device="cuda", dtype=dt) for n in (5, 7)]
    entries, ref = [], []
    for m in insts:
        ts = []
        for q in range(m.num_qubits):
            l, r = int(torch.randint(1, 40, (1,), generator=gen)), int(torch.randint(1, 40, (1,), generator=gen))
            T = torch.randn(l, 2, r, dtype=dt, generator=gen)
            ts.append(T.cuda())
        m._tensors = [t.clone() for t in ts]
        ref.append(ts)
        for j in range(25):
            q = int(torch.randint(0, m.num_qubits, (1,), generator=gen))
            U = torch.randn(2, 2, dtype=dt, generator=gen)
            U = U.cuda() if j % 2 else U  # host and device gate matrices
            entries.append((m, q, U))
    for m, q, U in entries:
        ops.single_qubit_gate_(ref[insts.index(m)][q], U.to("cuda", dt))
    apply_single_qubit_entries(entries)
    for m, ts in zip(insts, ref):
        for a, b in zip(m._tensors, ts):
            assert torch.equal(a, b)


def test_config4_shaped_graph_batch_matches_fp64_oracle():
    """The batched workload's shape at oracle-checkable sizes: hardware-efficient
    ansatz instances of uneven qubit counts and chi caps, 10 layers, eps 1e-8,
    device-resident and captured as one CUDA graph, each against the FP64
    oracle run of that instance alone.  The caps equal 2^(n/2), so only eps
    truncates and the float32 result stays within 1 - 1e-6 of FP64."""
    specs = [(12, 64, 700), (14, 128, 701), (16, 256, 702)]
    insts = [aq.AdaptiveMPS(n, bond_dim=1, eps_bond=1e-8, chi_max_per_bond=chi, device="cuda", device_resident=True)
             for n, chi, _ in specs]
    circs = [hea_circuit(n, 10, seed=sd) for n, _, sd in specs]
    cap = aq.MPSBatch(insts).capture(circs)
    cap.replay()
    cap.finish()
    for (n, chi, _), m, c in zip(specs, insts, circs):
        o = mo.OracleMPS(n, bond_dim=1, eps_bond=1e-8, chi_max_per_bond=chi, dtype=np.complex128)
        for kind, q, U in c:
            (o.apply_two_site_gate if kind == "2q" else o.apply_single_qubit_gate)(q, U.numpy())
        f = mo.mps_fidelity([t.cpu().numpy() for t in m.tensors], o.tensors)
        assert f > 1 - 1e-6, (n, chi, f)
