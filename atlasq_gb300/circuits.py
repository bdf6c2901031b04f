"""Seeded circuit generators for the MPS workloads.

All gate matrices are produced on the host from a ``torch.Generator`` so that the
same seed yields the same circuit for the GPU path, the reference and the CPU
oracle.  A circuit is a list of operations:

    ("2q", bond, U4)      two-site gate on (bond, bond+1), U4 complex64 [4,4]
    ("1q", qubit, U2)     single-qubit gate, U2 complex64 [2,2]

Workloads:
  * Haar brickwork: layer L applies Haar-random 4x4 unitaries on bonds
    L%2, L%2+2, ...  (n=40, depth 20 -> 390 gates; n=12, depth 10 -> 55 gates).
    Haar unitaries are the Q of a complex Gaussian QR with the Mezzadri phase
    fix, drawn in float64 and cast to complex64.
  * Hardware-efficient ansatz (HEA): per layer RY(theta) then RZ(phi) on every
    qubit (theta, phi ~ U[0, 2pi)), then CZ on (i, i+1) for i = 0..n-2 in order.
"""
import math

import torch

CZ = torch.diag(torch.tensor([1, 1, 1, -1], dtype=torch.complex64))


def haar_unitary(gen, dim=4):
    z = torch.complex(torch.randn(dim, dim, generator=gen, dtype=torch.float64),
                      torch.randn(dim, dim, generator=gen, dtype=torch.float64)) / math.sqrt(2.0)
    q, r = torch.linalg.qr(z)
    d = torch.diagonal(r)
    return (q * (d / torch.abs(d)).unsqueeze(0)).to(torch.complex64).contiguous()


def ry(theta):
    c, s = math.cos(theta / 2), math.sin(theta / 2)
    return torch.tensor([[c, -s], [s, c]], dtype=torch.complex64)


def rz(phi):
    return torch.tensor([[complex(math.cos(-phi / 2), math.sin(-phi / 2)), 0],
                         [0, complex(math.cos(phi / 2), math.sin(phi / 2))]], dtype=torch.complex64)


def haar_brickwork(n, depth, seed):
    gen = torch.Generator().manual_seed(seed)
    ops = []
    for layer in range(depth):
        for b in range(layer % 2, n - 1, 2):
            ops.append(("2q", b, haar_unitary(gen)))
    return ops


def hea_circuit(n, layers, seed):
    gen = torch.Generator().manual_seed(seed)
    ops = []
    for _ in range(layers):
        ang = torch.rand(n, 2, generator=gen, dtype=torch.float64) * (2 * math.pi)
        for q in range(n):
            ops.append(("1q", q, ry(float(ang[q, 0]))))
            ops.append(("1q", q, rz(float(ang[q, 1]))))
        for b in range(n - 1):
            ops.append(("2q", b, CZ.clone()))
    return ops


def rx(theta):
    c, s = math.cos(theta / 2), math.sin(theta / 2)
    return torch.tensor([[c, complex(0, -s)], [complex(0, -s), c]], dtype=torch.complex64)


def rzz(theta):
    """exp(-i theta/2 Z(x)Z) in the basis 2*q_i + q_{i+1}."""
    m, p = complex(math.cos(theta / 2), -math.sin(theta / 2)), complex(math.cos(theta / 2), math.sin(theta / 2))
    return torch.diag(torch.tensor([m, p, p, m], dtype=torch.complex64))


def trotter_ising(n, steps, seed, dt_range=(0.05, 0.6)):
    """Transverse-field Ising Trotter circuit with disordered couplings:
    per step, RZZ(2 J_b dt) on every bond (even bonds, then odd) and RX(2 h_q dt)
    on every qubit; J, h uniform in [0.5, 1.5], dt uniform in dt_range per step.
    Entanglement grows at a rate set by J dt, so kept ranks sit well below the
    full two-site size (the workload the rank predictor is meant for)."""
    gen = torch.Generator().manual_seed(seed)
    ops = []
    for _ in range(steps):
        dt = dt_range[0] + (dt_range[1] - dt_range[0]) * float(torch.rand(1, generator=gen, dtype=torch.float64))
        J = 0.5 + torch.rand(n - 1, generator=gen, dtype=torch.float64)
        h = 0.5 + torch.rand(n, generator=gen, dtype=torch.float64)
        for par in (0, 1):
            for b in range(par, n - 1, 2):
                ops.append(("2q", b, rzz(2 * float(J[b]) * dt)))
        for q in range(n):
            ops.append(("1q", q, rx(2 * float(h[q]) * dt)))
    return ops


def layers_of(ops):
    """Split an op list into maximal runs whose two-site gates touch disjoint
    sites (single-qubit gates end a run only if they touch a pending site)."""
    out, cur, busy = [], [], set()
    for op in ops:
        sites = {op[1], op[1] + 1} if op[0] == "2q" else {op[1]}
        if sites & busy:
            out.append(cur)
            cur, busy = [], set()
        cur.append(op)
        busy |= sites
    if cur:
        out.append(cur)
    return out


def count_two_site(ops):
    return sum(1 for op in ops if op[0] == "2q")
