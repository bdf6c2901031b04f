"""The Qiskit MPS route (adapters.run_circuit) against the reference
backend's _run_mps on the same circuit (tests/golden/qiskit_mps.npz):
statevector fidelity > 1 - 1e-6 (complex64), counts keyed like the reference
(qubit 0 leftmost) and distributed like |psi|^2 (total variation < 0.05 at
4000 shots; the reference's own counts are not, see below), and the
reference's error for an unknown gate."""
import numpy as np
import pytest
import torch

from conftest import load_golden
from qiskit_like import Circuit, sample_circuit

pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

from atlasq_gb300 import adapters  # noqa: E402
from oracle import statevector as sv  # noqa: E402


def test_run_circuit_matches_reference_mps_route():
    g = load_golden("qiskit_mps")
    out = adapters.run_circuit(sample_circuit(), shots=int(g["shots"]), seed=7, device="cuda:0")
    assert out["backend_used"] == "mps"
    assert sv.fidelity(out["statevector"], g["statevector"]) > 1 - 1e-6
    counts = out["counts"]
    assert sum(counts.values()) == int(g["shots"])
    assert all(len(k) == 6 for k in counts)
    p = np.abs(g["statevector"].astype(np.complex128)) ** 2
    p /= p.sum()
    h = np.zeros(64)
    for k, v in counts.items():
        h[int(k, 2)] = v / int(g["shots"])
    assert 0.5 * np.abs(h - p).sum() < 0.05
    # the reference's own counts are not compared: for <= 10 qubits its sampler
    # canonicalises to the left before a left-to-right conditional sweep
    # (src/atlas_q/mps_pytorch.py:166-171), so they do not follow |psi|^2
    ref = np.zeros(64)
    for k, v in zip(g["count_keys"], g["count_vals"]):
        ref[int(str(k), 2)] = v / int(g["shots"])
    assert 0.5 * np.abs(ref - p).sum() > 0.2


def test_unknown_gate_raises_like_the_reference():
    c = Circuit(2).append("h", [0]).append("u3", [1], [0.1, 0.2, 0.3])
    with pytest.raises(ValueError, match="Unknown single-qubit gate"):
        adapters.run_circuit(c, shots=10, device="cuda:0")
    c = Circuit(3).append("ccx", [0, 1])
    with pytest.raises(ValueError, match="Unknown two-qubit gate"):
        adapters.run_circuit(c, shots=10, device="cuda:0")
