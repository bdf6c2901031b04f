"""MPO expectations, API-compatible with the in-scope part of src/atlas_q/mpo_ops.py.

Conventions kept from the reference: an MPO tensor is W[l, s, t, r]; the sweep
contracts the ket on s and the bra on t (einsum 'Lab,atr,LstR,bsB->RrB',
mpo_ops.py:1145), so a non-symmetric local operator O is evaluated as <O^T>;
the result is divided by <psi|psi> from a second (identity) sweep
(mpo_ops.py:1152-1169).

All contractions run as this package's GEMM and mix kernels.  ``local_expectations``
evaluates many product observables at once from cached left and right
environments (one left and one right sweep, then O(support) work each).
"""
import ctypes
from dataclasses import dataclass
from typing import Dict, List, Sequence, Tuple

import torch

from . import _lib, ops
from ._lib import check, dtype_code, ptr, stream_ptr


@dataclass
class MPO:
    """mpo_ops.py:35-141 (container + identity / from_local_ops / sum)."""

    tensors: List[torch.Tensor]
    n_sites: int

    def __post_init__(self):
        assert len(self.tensors) == self.n_sites
        for i, W in enumerate(self.tensors):
            assert len(W.shape) == 4, f"MPO tensor {i} must be 4D"
            assert W.shape[1] == W.shape[2], f"Physical dims must match at site {i}"

    @staticmethod
    def identity(n_sites: int, device: str = "cuda", dtype=torch.complex64) -> "MPO":
        W = torch.zeros(1, 2, 2, 1, dtype=dtype, device=device)
        W[0, 0, 0, 0] = 1.0
        W[0, 1, 1, 0] = 1.0
        return MPO([W.clone() for _ in range(n_sites)], n_sites)

    @staticmethod
    def from_local_ops(ops_: List[torch.Tensor], device: str = "cuda") -> "MPO":
        tensors = []
        for i, op in enumerate(ops_):
            assert op.shape == (2, 2), f"Operator {i} must be 2x2"
            tensors.append(op.reshape(1, 2, 2, 1).to(device))
        return MPO(tensors, len(ops_))

    @staticmethod
    def from_operators(ops_: List[torch.Tensor], device: str = "cuda") -> "MPO":
        return MPO.from_local_ops(ops_, device=device)

    def __add__(self, other: "MPO") -> "MPO":
        """mpo_ops.py:88-141 (bond-dimension concatenation)."""
        assert self.n_sites == other.n_sites
        out = []
        for i in range(self.n_sites):
            A, B = self.tensors[i], other.tensors[i]
            la, d, _, ra = A.shape
            lb, _, _, rb = B.shape
            if i == 0:
                W = torch.zeros(max(la, lb), d, d, ra + rb, dtype=A.dtype, device=A.device)
                W[:la, :, :, :ra] = A
                W[:lb, :, :, ra:ra + rb] = B
            elif i == self.n_sites - 1:
                W = torch.zeros(la + lb, d, d, max(ra, rb), dtype=A.dtype, device=A.device)
                W[:la, :, :, :ra] = A
                W[la:la + lb, :, :, :rb] = B
            else:
                W = torch.zeros(la + lb, d, d, ra + rb, dtype=A.dtype, device=A.device)
                W[:la, :, :, :ra] = A
                W[la:, :, :, ra:] = B
            out.append(W)
        return MPO(out, self.n_sites)


class MPOBuilder:
    """mpo_ops.py:144-199 (identity / local operator / sum of local operators)."""

    @staticmethod
    def identity_mpo(n_sites: int, device: str = "cuda", dtype=torch.complex64) -> MPO:
        return MPO.identity(n_sites, device=device, dtype=dtype)

    @staticmethod
    def local_operator(op: torch.Tensor, site: int, n_sites: int, device: str = "cuda",
                       dtype=torch.complex64) -> MPO:
        I = torch.eye(2, dtype=dtype, device=device)
        ops_ = [I] * n_sites
        ops_[site] = op.to(device=device, dtype=dtype)
        return MPO.from_local_ops(ops_, device=device)

    @staticmethod
    def sum_local_operators(n_sites: int, local_ops: List[Tuple[int, torch.Tensor]], device: str = "cuda",
                            dtype=torch.complex64) -> MPO:
        result = None
        for site, op in local_ops:
            m = MPOBuilder.local_operator(op, site, n_sites, device=device, dtype=dtype)
            result = m if result is None else result + m
        return result


def _site_step(E, A, W):
    """E' for one site.  E: [Lw, chiA, chiA] (bra, ket), A: [chiA, 2, chiB], W: [Lw, 2, 2, Rw]."""
    lib = _lib.load()
    Lw, chiA, _ = E.shape
    chiB = A.shape[2]
    Rw = W.shape[3]
    A_mat = A.reshape(chiA, 2 * chiB)
    M = ops.cgemm(E.contiguous(), A_mat.unsqueeze(0).expand(Lw, -1, -1).contiguous())  # [Lw, chiA, 2chiB]
    N = torch.empty(Rw, chiA, 2, chiB, dtype=A.dtype, device=A.device)
    Wc = W.to(dtype=A.dtype, device=A.device).contiguous()
    check(lib.agb_mpo_mix(dtype_code(A.dtype), ptr(M), ptr(Wc), ptr(N), Lw, Rw, chiA, chiB,
                          stream_ptr(A.device)), "mpo_mix")
    A2 = A.reshape(2 * chiA, chiB)
    out = ops.cgemm(A2.unsqueeze(0).expand(Rw, -1, -1).contiguous(), N.reshape(Rw, 2 * chiA, chiB),
                    opA="C", opB="N")
    return out


def _gemm(A, B, opA="N", opB="N"):
    """complex64 products with every dimension >= 32 go to the tcgen05 GEMM
    (3xTF32, float32 accuracy); the rest to the SIMT GEMM."""
    ra, ca = A.shape[-2], A.shape[-1]
    rb, cb = B.shape[-2], B.shape[-1]
    M, K = (ra, ca) if opA == "N" else (ca, ra)
    N = cb if opB == "N" else rb
    if A.dtype == torch.complex64 and min(M, N, K) >= 32:
        return ops.cgemm_tc(A, B, opA=opA, opB=opB, sync=False)
    return ops.cgemm(A, B, opA=opA, opB=opB)


def _norm_step(E, A):
    """Identity step: E' = sum_s A_s^H E A_s as two GEMMs (no mixing needed)."""
    chiA, _, chiB = A.shape
    M = _gemm(E, A.reshape(chiA, 2 * chiB))            # [chiA, 2chiB] == [(a,t), B] layout
    return _gemm(A.reshape(2 * chiA, chiB), M.reshape(2 * chiA, chiB), opA="C", opB="N")


@torch.no_grad()
def expectation_value(mpo: MPO, mps, use_gpu_optimized: bool = True) -> complex:
    """mpo_ops.py:1085-1169 (standard MPO contraction path)."""
    n = mpo.n_sites
    assert n == mps.num_qubits
    tensors = [t.contiguous() for t in mps.tensors]
    dt = tensors[0].dtype
    dev = tensors[0].device
    E = torch.ones(1, 1, 1, dtype=dt, device=dev)
    N = torch.ones(1, 1, dtype=dt, device=dev)
    for i in range(n):
        A = tensors[i] if tensors[i].dtype == dt else tensors[i].to(dt).contiguous()
        E = _site_step(E, A, mpo.tensors[i])
        N = _norm_step(N, A)
    val = complex(E.reshape(-1)[0].item() / N.reshape(-1)[0].item())
    ops.check_tc_status(dev)
    return val


def correlation_function(op1: torch.Tensor, site1: int, op2: torch.Tensor, site2: int, mps) -> complex:
    """mpo_ops.py:1172-1207."""
    n = mps.num_qubits
    assert 0 <= site1 < n and 0 <= site2 < n
    if site1 > site2:
        site1, site2, op1, op2 = site2, site1, op2, op1
    dev = mps.tensors[0].device
    dt = mps.tensors[0].dtype
    I = torch.eye(2, dtype=dt, device=dev)
    ops_ = [I] * n
    ops_[site1] = op1.to(device=dev, dtype=dt)
    ops_[site2] = op2.to(device=dev, dtype=dt)
    return expectation_value(MPO.from_local_ops(ops_, device=dev), mps)


def pauli_string_to_mpo(pauli_string: str, device: str = "cuda", dtype=torch.complex128) -> MPO:
    """mpo_ops.py:1210-1233."""
    table = {"I": [[1, 0], [0, 1]], "X": [[0, 1], [1, 0]], "Y": [[0, -1j], [1j, 0]], "Z": [[1, 0], [0, -1]]}
    return MPO.from_local_ops([torch.tensor(table[p], dtype=dtype, device=device) for p in pauli_string],
                              device=device)


@torch.no_grad()
def environments(mps):
    """Left identity environments Lenv[i] (before site i, [bra, ket]) and right
    environments Renv[i] (after site i-1, stored as [ket, bra]) for i = 0..n."""
    tensors = [t.contiguous() for t in mps.tensors]
    dt = tensors[0].dtype
    dev = tensors[0].device
    n = len(tensors)
    Lenv = [torch.ones(1, 1, dtype=dt, device=dev)]
    for A in tensors:
        Lenv.append(_norm_step(Lenv[-1], A if A.dtype == dt else A.to(dt).contiguous()))
    Renv = [None] * (n + 1)
    Renv[n] = torch.ones(1, 1, dtype=dt, device=dev)
    for i in range(n - 1, -1, -1):
        A = tensors[i] if tensors[i].dtype == dt else tensors[i].to(dt).contiguous()
        chi, _, chi2 = A.shape
        X = _gemm(A.reshape(2 * chi, chi2), Renv[i + 1])          # [(B,s), r']
        Renv[i] = _gemm(X.reshape(chi, 2 * chi2), A.reshape(chi, 2 * chi2), opA="N", opB="C")
    return tensors, Lenv, Renv


@torch.no_grad()
def local_expectations(mps, observables: Sequence[Dict[int, torch.Tensor]]) -> List[complex]:
    """<psi|prod_i O_i^T|psi>/<psi|psi> for many product observables (site -> 2x2),
    with the reference's transpose convention (the per-site einsum of
    expectation_value, src/atlas_q/mpo_ops.py:1145, with [1,2,2,1] MPO tensors).

    One left and one right environment sweep; then every observable advances
    one site of its support per round, starting from the left environment of
    its first site: the items of a round whose site tensors have the same shape
    share one batched GEMM pair (E A, then A^H (mixed E A)) and one site-mix
    launch (agb_site_mix; sites inside the support without an operator mix with
    the identity).  Each finished item is closed with the right environment."""
    lib = _lib.load()
    tensors, Lenv, Renv = environments(mps)
    dt = tensors[0].dtype
    dev = tensors[0].device
    code = dtype_code(dt)
    nobs = len(observables)
    out2 = torch.zeros(nobs + 1, 2, dtype=torch.float64, device=dev)
    stream = stream_ptr(dev)
    # norm = tr(Lenv[n]) (1x1)
    check(lib.agb_trace_prod(code, ptr(Lenv[-1]), ptr(Renv[-1]), 1,
                             ctypes.c_void_p(out2.data_ptr() + 16 * nobs), stream), "trace_prod")
    eye = torch.eye(2, dtype=dt, device=dev)
    # [index, next site, last site, environment, operators]
    active = []
    for k, obs in enumerate(observables):
        sites = sorted(obs)
        ops_dev = {i: obs[i].to(device=dev, dtype=dt) for i in sites}
        active.append([k, sites[0], sites[-1], Lenv[sites[0]], ops_dev])
    while active:
        groups = {}
        for it in active:
            groups.setdefault(tuple(tensors[it[1]].shape), []).append(it)
        for (chiA, _, chiB), its in groups.items():
            G = len(its)
            E = torch.stack([it[3] for it in its])                               # [G, chiA, chiA]
            A = torch.stack([tensors[it[1]] for it in its])                      # [G, chiA, 2, chiB]
            W = torch.stack([it[4].get(it[1], eye) for it in its]).contiguous()  # [G, 2, 2]
            M = _gemm(E, A.view(G, chiA, 2 * chiB))                              # [G, chiA, (s, chiB)]
            X = torch.empty_like(M)
            check(lib.agb_site_mix(code, ptr(M), ptr(W), ptr(X), G, chiA, chiB, stream), "site_mix")
            En = _gemm(A.view(G, 2 * chiA, chiB), X.view(G, 2 * chiA, chiB), opA="C")  # [G, chiB, chiB]
            for g, it in enumerate(its):
                it[3] = En[g]
                it[1] += 1
        still = []
        for it in active:
            if it[1] > it[2]:
                check(lib.agb_trace_prod(code, ptr(it[3]), ptr(Renv[it[2] + 1]), it[3].shape[0],
                                         ctypes.c_void_p(out2.data_ptr() + 16 * it[0]), stream), "trace_prod")
            else:
                still.append(it)
        active = still
    host = out2.cpu()
    ops.check_tc_status(dev)
    norm = complex(host[-1, 0].item(), host[-1, 1].item())
    return [complex(host[k, 0].item(), host[k, 1].item()) / norm for k in range(nobs)]
