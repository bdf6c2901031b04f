"""A minimal object with the QuantumCircuit attributes the MPS route reads
(num_qubits, data[i].operation.{name, params}, data[i].qubits, find_bit),
for tests without Qiskit installed."""
from types import SimpleNamespace


class Circuit:
    def __init__(self, n):
        self.num_qubits = n
        self._qubits = [SimpleNamespace(tag=i) for i in range(n)]
        self.data = []

    def find_bit(self, q):
        return SimpleNamespace(index=q.tag)

    def append(self, name, qubits, params=()):
        self.data.append(SimpleNamespace(operation=SimpleNamespace(name=name, params=list(params)),
                                         qubits=[self._qubits[q] for q in qubits]))
        return self


def sample_circuit(angle=float):
    """Six qubits, every gate name the MPS route dispatches, plus measure and
    barrier.  `angle` wraps the rotation parameters (the reference's rotation
    gates need torch tensors, its fixture passes torch.tensor)."""
    c = Circuit(6)
    for q in range(6):
        c.append("h", [q])
    c.append("rx", [0], [angle(0.3)]).append("ry", [1], [angle(1.1)]).append("rz", [2], [angle(-0.7)])
    c.append("cx", [0, 1]).append("cz", [1, 2]).append("cy", [2, 3]).append("swap", [3, 4])
    c.append("x", [4]).append("y", [5]).append("z", [0]).append("s", [1]).append("sdg", [2])
    c.append("t", [3]).append("tdg", [4]).append("barrier", [0, 1, 2])
    c.append("cnot", [4, 5]).append("ry", [3], [angle(0.4)]).append("cx", [2, 3])
    for q in range(6):
        c.append("measure", [q])
    return c
