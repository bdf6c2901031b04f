"""Qiskit front end for the MPS path: the reference backend's MPS route
(ATLASQBackend._run_mps, src/atlas_q/adapters/qiskit_adapter.py:383-404, with
its gate dispatch _apply_gate_to_mps :505-553 and count conversion
_samples_to_counts :729-746) on this package's AdaptiveMPS.

Qiskit itself is not needed: a circuit is read through the attributes every
qiskit.QuantumCircuit has (``num_qubits``, ``data`` of instructions with
``.operation.name`` / ``.operation.params`` / ``.qubits``, and
``find_bit(qubit).index``), so a QuantumCircuit and any object shaped like
one both work.

Behaviour kept from the reference: the MPS starts as
AdaptiveMPS(n, bond_dim=max_bond_dim) with its default truncation; measure
and barrier instructions are skipped; an unknown gate raises ValueError;
counts keys are ``format(sample, '0{n}b')`` (qubit 0 the leftmost bit, the
MPS sampler's order); the statevector is returned for n <= 20.  Sampling
right-canonicalises first (the conditional sampler is exact only then) and
draws from Philox4x32-10 seeded by ``seed``.
"""
from typing import Dict, Optional

import numpy as np

from .adaptive_mps import AdaptiveMPS

_ONE = {"h": "h", "x": "x", "y": "y", "z": "z", "s": "s", "sdg": "sdg", "t": "t", "tdg": "tdg"}
_ROT = {"rx": "rx", "ry": "ry", "rz": "rz"}
_TWO = {"cx": "cnot", "cnot": "cnot", "cz": "cz", "cy": "cy", "swap": "swap"}


def apply_gate(mps: AdaptiveMPS, name: str, qubits, params) -> None:
    """One instruction on the MPS by name (the reference's _apply_gate_to_mps)."""
    g = name.lower()
    if g in ("measure", "barrier"):
        return
    if len(qubits) == 1:
        q = qubits[0]
        if g in _ONE:
            getattr(mps, _ONE[g])(q)
        elif g in _ROT:
            getattr(mps, _ROT[g])(q, float(params[0]))
        else:
            raise ValueError(f"Unknown single-qubit gate: {g}")
    elif len(qubits) == 2:
        if g not in _TWO:
            raise ValueError(f"Unknown two-qubit gate: {g}")
        getattr(mps, _TWO[g])(qubits[0], qubits[1])


def samples_to_counts(samples, n_qubits: Optional[int] = None) -> Dict[str, int]:
    if isinstance(samples, dict):
        return samples
    keys, cnt = np.unique(np.asarray(samples, dtype=np.int64), return_counts=True)
    fmt = (lambda v: format(int(v), f"0{n_qubits}b")) if n_qubits else (lambda v: bin(int(v))[2:])
    return {fmt(k): int(c) for k, c in zip(keys, cnt)}


class MPSCircuitRunner:
    """Runs circuits on the GB300 MPS path (the MPS branch of the reference backend)."""

    def __init__(self, max_bond_dim: int = 128, device: str = "cuda", **mps_kwargs):
        self.max_bond_dim = max_bond_dim
        self.device = device
        self.mps_kwargs = mps_kwargs

    def build(self, circuit) -> AdaptiveMPS:
        mps = AdaptiveMPS(circuit.num_qubits, bond_dim=self.max_bond_dim, device=self.device, **self.mps_kwargs)
        for inst in circuit.data:
            op = inst.operation
            qubits = [circuit.find_bit(q).index for q in inst.qubits]
            apply_gate(mps, op.name, qubits, list(getattr(op, "params", [])))
        return mps

    def run(self, circuit, shots: int = 1024, seed: Optional[int] = None) -> dict:
        mps = self.build(circuit)
        n = circuit.num_qubits
        samples = mps.sample(shots, seed=0 if seed is None else int(seed))
        counts = samples_to_counts(np.asarray(samples), n)
        sv = mps.to_statevector().cpu().numpy() if n <= 20 else None
        return {"counts": counts, "statevector": sv, "backend_used": "mps", "success": True, "mps": mps}


def run_circuit(circuit, shots: int = 1024, seed: Optional[int] = None, max_bond_dim: int = 128,
                device: str = "cuda") -> dict:
    """Counts (and the statevector for n <= 20) of a Qiskit-style circuit on the MPS path."""
    return MPSCircuitRunner(max_bond_dim=max_bond_dim, device=device).run(circuit, shots=shots, seed=seed)
