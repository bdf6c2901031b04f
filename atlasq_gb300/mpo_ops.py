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
import math
from typing import Dict, List, Sequence, Tuple

import torch

from . import _lib, ops
from ._lib import check, dtype_code, ptr, stream_ptr


def _as_site(W, i):
    if not isinstance(W, torch.Tensor) or W.dim() != 4:
        raise ValueError(f"MPO site {i}: expected a 4-index tensor [left, phys_out, phys_in, right]")
    if W.shape[1] != 2 or W.shape[2] != 2:
        raise ValueError(f"MPO site {i}: physical dimensions must be 2 x 2, got {tuple(W.shape[1:3])}")
    return W


class MPO:
    """Matrix product operator over qubits.

    Site tensors are W[l, s, t, r] (l, r the operator bonds; s, t the physical
    indices), the layout of src/atlas_q/mpo_ops.py:35-141.  A local operator
    O enters as W[l, s, t, r] = O[s, t]; expectation_value contracts the ket on
    s and the bra on t (so it evaluates <O^T>, as the reference does) and
    apply_mpo_to_mps applies O with s the output index."""

    def __init__(self, tensors: Sequence[torch.Tensor], n_sites: int = None):
        tensors = [_as_site(W, i) for i, W in enumerate(tensors)]
        if n_sites is None:
            n_sites = len(tensors)
        if len(tensors) != n_sites:
            raise ValueError(f"MPO has {len(tensors)} site tensors for {n_sites} sites")
        if n_sites and (tensors[0].shape[0] != 1 or tensors[-1].shape[3] != 1):
            raise ValueError("MPO boundary bonds must have dimension 1")
        for i in range(n_sites - 1):
            if tensors[i].shape[3] != tensors[i + 1].shape[0]:
                raise ValueError(f"MPO bond {i}: {tensors[i].shape[3]} != {tensors[i + 1].shape[0]}")
        self.tensors = tensors
        self.n_sites = n_sites

    @property
    def bond_dims(self) -> List[int]:
        return [int(W.shape[3]) for W in self.tensors[:-1]]

    @staticmethod
    def identity(n_sites: int, device: str = "cuda", dtype=torch.complex64) -> "MPO":
        eye = torch.eye(2, dtype=dtype, device=device).reshape(1, 2, 2, 1)
        return MPO([eye.clone() for _ in range(n_sites)], n_sites)

    @staticmethod
    def from_local_ops(ops_: Sequence[torch.Tensor], device: str = "cuda") -> "MPO":
        """Product operator O_0 x O_1 x ... (bond dimension 1)."""
        sites = []
        for i, o in enumerate(ops_):
            if tuple(o.shape) != (2, 2):
                raise ValueError(f"local operator {i} must be 2 x 2, got {tuple(o.shape)}")
            sites.append(o.to(device).reshape(1, 2, 2, 1))
        return MPO(sites, len(sites))

    @staticmethod
    def from_operators(ops_: Sequence[torch.Tensor], device: str = "cuda") -> "MPO":
        return MPO.from_local_ops(ops_, device=device)

    def __add__(self, other: "MPO") -> "MPO":
        """The operator sum as the direct sum of the two chains: the bonds of
        `other` are appended after those of `self` (block-diagonal inner
        sites; the first site joins the two rows, the last the two columns)."""
        if self.n_sites != other.n_sites:
            raise ValueError(f"cannot add MPOs on {self.n_sites} and {other.n_sites} sites")
        n = self.n_sites
        out = []
        for i, (A, B) in enumerate(zip(self.tensors, other.tensors)):
            B = B.to(device=A.device, dtype=A.dtype)
            if n == 1:
                out.append(A + B)
                continue
            la, _, _, ra = A.shape
            lb, _, _, rb = B.shape
            rows = 1 if i == 0 else la + lb
            cols = 1 if i == n - 1 else ra + rb
            W = torch.zeros(rows, 2, 2, cols, dtype=A.dtype, device=A.device)
            r0 = 0 if i == 0 else la          # where B's left bonds start
            c0 = 0 if i == n - 1 else ra      # where B's right bonds start
            W[:la, :, :, :ra] += A
            W[r0:r0 + lb, :, :, c0:c0 + rb] += B
            out.append(W)
        return MPO(out, n)


class MPOBuilder:
    """Constructors of src/atlas_q/mpo_ops.py:144-199."""

    @staticmethod
    def identity_mpo(n_sites: int, device: str = "cuda", dtype=torch.complex64) -> MPO:
        return MPO.identity(n_sites, device=device, dtype=dtype)

    @staticmethod
    def local_operator(op: torch.Tensor, site: int, n_sites: int, device: str = "cuda",
                       dtype=torch.complex64) -> MPO:
        """I x ... x op (at `site`) x ... x I."""
        if not 0 <= site < n_sites:
            raise ValueError(f"site {site} outside 0..{n_sites - 1}")
        eye = torch.eye(2, dtype=dtype, device=device)
        return MPO.from_local_ops([op.to(device=device, dtype=dtype) if k == site else eye
                                   for k in range(n_sites)], device=device)

    @staticmethod
    def sum_local_operators(n_sites: int, local_ops: Sequence[Tuple[int, torch.Tensor]], device: str = "cuda",
                            dtype=torch.complex64) -> MPO:
        """sum_k I x ... x O_k (at site_k) x ... x I as a two-channel finite-state
        MPO: channel 0 = "term not placed yet", channel 1 = "term placed"; every
        site carries I on 0 -> 0 and 1 -> 1 and the sum of its local terms on
        0 -> 1, the first site starts in channel 0 and the last ends in channel 1
        (bond dimension 2 for any number of terms).  None for no terms, as the
        reference returns."""
        if not local_ops:
            return None
        terms = [torch.zeros(2, 2, dtype=dtype, device=device) for _ in range(n_sites)]
        for site, op in local_ops:
            if not 0 <= site < n_sites:
                raise ValueError(f"site {site} outside 0..{n_sites - 1}")
            terms[site] = terms[site] + op.to(device=device, dtype=dtype)
        if n_sites == 1:
            return MPO([terms[0].reshape(1, 2, 2, 1)], 1)
        eye = torch.eye(2, dtype=dtype, device=device)
        sites = []
        for k in range(n_sites):
            W = torch.zeros(2, 2, 2, 2, dtype=dtype, device=device)
            W[0, :, :, 0] = eye
            W[1, :, :, 1] = eye
            W[0, :, :, 1] = terms[k]
            if k == 0:
                W = W[0:1]
            if k == n_sites - 1:
                W = W[..., 1:2]
            sites.append(W.contiguous())
        return MPO(sites, n_sites)


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


# ---------------------------------------------------------------- MPO applied to an MPS (f4)
@torch.no_grad()
def apply_mpo_to_mps(mpo: MPO, mps, chi_max: int = 128, eps: float = 1e-8):
    """|psi'> = O |psi> (src/atlas_q/mpo_ops.py:1034-1082): per site
    out[(l, a), s, (r, b)] = sum_t W[l, s, t, r] A[a, t, b] (agb_mpo_apply_site),
    then a left-canonical QR sweep of the result.  As in the reference, the
    bond dimensions multiply by the MPO's and nothing is truncated:
    `chi_max` and `eps` are accepted for signature compatibility only.
    Returns a new AdaptiveMPS holding the product state's tensors (same dtype
    and device as `mps`)."""
    from .adaptive_mps import AdaptiveMPS, DTypePolicy
    if mpo.n_sites != mps.num_qubits:
        raise ValueError(f"MPO on {mpo.n_sites} sites applied to an MPS of {mps.num_qubits} qubits")
    lib = _lib.load()
    src = [t.contiguous() for t in mps.tensors]
    dt, dev = src[0].dtype, src[0].device
    code = dtype_code(dt)
    stream = stream_ptr(dev)
    out = []
    for W, A in zip(mpo.tensors, src):
        W = W.to(device=dev, dtype=dt).contiguous()
        A = A if A.dtype == dt else A.to(dt).contiguous()
        Dl, _, _, Dr = W.shape
        ca, _, cb = A.shape
        M = torch.empty(Dl * ca, 2, Dr * cb, dtype=dt, device=dev)
        check(lib.agb_mpo_apply_site(code, ptr(W), ptr(A), ptr(M), Dl, Dr, ca, cb, stream), "mpo_apply_site")
        out.append(M)
    res = AdaptiveMPS(mps.num_qubits, bond_dim=1, eps_bond=mps.eps_bond, chi_max_per_bond=mps.chi_max_per_bond,
                      dtype_policy=DTypePolicy(default=dt), device=str(dev), dtype=dt)
    res.tensors = out
    res.bond_dims = [int(t.shape[2]) for t in out[:-1]]
    res.to_left_canonical()
    return res


_PAULI = {"I": ((1, 0), (0, 1)), "X": ((0, 1), (1, 0)), "Y": ((0, -1j), (1j, 0)), "Z": ((1, 0), (0, -1))}


def _pauli(letter, dtype, device):
    if letter not in _PAULI:
        raise ValueError(f"Invalid Pauli letter: {letter}")
    return torch.tensor(_PAULI[letter], dtype=dtype, device=device)


def pauli_exp_mpo(pauli_string: str, lam: float, device: str = "cuda", dtype=torch.complex64) -> MPO:
    """exp(i lam P) = cos(lam) I + i sin(lam) P for a Pauli string P as a
    two-rail MPO: rail 0 carries cos(lam) I x I x ..., rail 1 carries
    i sin(lam) P_0 x P_1 x ...; the rails never mix, so every letter of P acts.
    (The reference's builder, mpo_ops.py:1250-1293, routes rail 1 back onto
    rail 0 after the second site, which drops the letters from the third site
    on; this builder applies the operator its docstring names.)"""
    n = len(pauli_string)
    if n == 0:
        raise ValueError("empty Pauli string")
    c, s = math.cos(lam), math.sin(lam)
    eye = torch.eye(2, dtype=dtype, device=device)
    if n == 1:
        return MPO([(c * eye + 1j * s * _pauli(pauli_string[0], dtype, device)).reshape(1, 2, 2, 1)], 1)
    sites = []
    for k, letter in enumerate(pauli_string):
        P = _pauli(letter, dtype, device)
        W = torch.zeros(2, 2, 2, 2, dtype=dtype, device=device)
        W[0, :, :, 0] = (c if k == 0 else 1.0) * eye
        W[1, :, :, 1] = (1j * s if k == 0 else 1.0) * P
        if k == 0:
            W = (W[0] + W[1]).unsqueeze(0)   # one left bond: both rails start here
        if k == n - 1:
            W = (W[..., 0] + W[..., 1]).unsqueeze(-1)  # one right bond: both rails end here
        sites.append(W.contiguous())
    return MPO(sites, n)


@torch.no_grad()
def apply_pauli_exp_to_mps(mps, pauli_string: str, coeff: complex, theta: float, chi_max: int = 128) -> None:
    """In place: |psi> <- exp(i lam P)|psi> with lam = theta * Im(coeff) when
    coeff is imaginary, else theta * Re(coeff) (src/atlas_q/mpo_ops.py:1296-1358);
    nothing happens for |lam| < 1e-12.  The bond dimension doubles (no
    truncation, as in the reference; `chi_max` is accepted for compatibility)."""
    coeff = complex(coeff)
    lam = theta * (coeff.imag if abs(coeff.imag) > 1e-14 else coeff.real)
    if abs(lam) < 1e-12:
        return
    if len(pauli_string) != mps.num_qubits:
        raise ValueError(f"Pauli string of length {len(pauli_string)} for {mps.num_qubits} qubits")
    t0 = mps.tensors[0]
    out = apply_mpo_to_mps(pauli_exp_mpo(pauli_string, lam, device=t0.device, dtype=t0.dtype), mps,
                           chi_max=chi_max)
    mps.tensors = [t.clone() for t in out.tensors]
    mps.bond_dims = list(out.bond_dims)


# ---------------------------------------------------------------- TDVP environments (f1)
@torch.no_grad()
def tdvp_left_environment(L_prev: torch.Tensor, A: torch.Tensor, W: torch.Tensor) -> torch.Tensor:
    """L_next[u, n, j] = sum L_prev[q, l, i] conj(A[q, t, u]) W[l, s, t, n] A[i, s, j]
    (src/triton_kernels/tdvp_mpo_ops.py:38-60; L: [bra, mpo, ket]).  Three
    launches: a strided GEMM per MPO bond l (T[l, q, (s, j)] = L[q, l, :] A),
    the MPO mix (agb_mpo_mix), and a strided GEMM per bond n that writes
    L_next in its [u, n, j] order."""
    lib = _lib.load()
    A = A.contiguous()
    dt, dev = A.dtype, A.device
    W = W.to(device=dev, dtype=dt).contiguous()
    L_prev = L_prev.to(dt).contiguous()
    cq, Dl, ci = L_prev.shape
    ci2, _, cj = A.shape
    Wl, _, _, Dn = W.shape
    if ci2 != ci or Wl != Dl or A.shape[0] != ci:
        raise ValueError("tdvp_left_environment: bond dimensions do not match")
    cu = A.shape[2]
    T = torch.empty(Dl, cq, 2 * cj, dtype=dt, device=dev)
    ops.cgemm_strided(Dl, cq, 2 * cj, ci, L_prev, 0, Dl * ci, ci, A, 0, 2 * cj, 0, T, 0, 2 * cj, cq * 2 * cj)
    N = torch.empty(Dn, cq, 2, cj, dtype=dt, device=dev)
    check(lib.agb_mpo_mix(dtype_code(dt), ptr(T), ptr(W), ptr(N), Dl, Dn, cq, cj, stream_ptr(dev)), "mpo_mix")
    out = torch.empty(cu, Dn, cj, dtype=dt, device=dev)
    ops.cgemm_strided(Dn, cu, cj, 2 * cq, A, 0, cu, 0, N, 0, cj, 2 * cq * cj, out, 0, Dn * cj, cj, opA="C")
    return out


@torch.no_grad()
def tdvp_right_environment(R_next: torch.Tensor, A: torch.Tensor, W: torch.Tensor) -> torch.Tensor:
    """R_prev[q, l, i] = sum R_next[u, n, j] conj(A[q, t, u]) W[l, s, t, n] A[i, s, j]
    (src/triton_kernels/tdvp_mpo_ops.py:63-86; R: [bra, mpo, ket]).  A strided
    GEMM per bond n with A conjugated in place (P[n, (q, t), j]), the MPO mix
    with the tensor's index roles exchanged (Q[l, q, (s, j)]), and a strided GEMM
    per bond l that writes R_prev in its [q, l, i] order."""
    lib = _lib.load()
    A = A.contiguous()
    dt, dev = A.dtype, A.device
    W = W.to(device=dev, dtype=dt)
    R_next = R_next.to(dt).contiguous()
    cu, Dn, cj = R_next.shape
    cq, _, cu2 = A.shape
    Dl = W.shape[0]
    if cu2 != cu or W.shape[3] != Dn or A.shape[2] != cj:
        raise ValueError("tdvp_right_environment: bond dimensions do not match")
    ci = cq
    P = torch.empty(Dn, 2 * cq, cj, dtype=dt, device=dev)
    ops.cgemm_strided(Dn, 2 * cq, cj, cu, A, 0, cu, 0, R_next, 0, Dn * cj, cj, P, 0, cj, 2 * cq * cj, opA="R")
    Wx = W.permute(3, 2, 1, 0).contiguous()  # Wx[n, t, s, l] = W[l, s, t, n]
    Q = torch.empty(Dl, cq, 2, cj, dtype=dt, device=dev)
    check(lib.agb_mpo_mix(dtype_code(dt), ptr(P), ptr(Wx), ptr(Q), Dn, Dl, cq, cj, stream_ptr(dev)), "mpo_mix")
    out = torch.empty(cq, Dl, ci, dtype=dt, device=dev)
    ops.cgemm_strided(Dl, cq, ci, 2 * cj, Q, 0, 2 * cj, cq * 2 * cj, A, 0, 2 * cj, 0, out, 0, Dl * ci, ci, opB="T")
    return out


@torch.no_grad()
def tdvp_apply_local_H(L_site: torch.Tensor, W_site: torch.Tensor, A: torch.Tensor,
                       R_site_plus1: torch.Tensor) -> torch.Tensor:
    """H_A[i, t, j] with the reference's index pattern 'qli, lstn, isj, unj -> itj'
    (src/triton_kernels/tdvp_mpo_ops.py:89-106): i and j are shared with the
    environments' ket indices, the bra indices q and u are summed
    (agb_tdvp_local_h)."""
    lib = _lib.load()
    A = A.contiguous()
    dt, dev = A.dtype, A.device
    L = L_site.to(dt).contiguous()
    R = R_site_plus1.to(dt).contiguous()
    W = W_site.to(device=dev, dtype=dt).contiguous()
    cq, Dl, ci = L.shape
    cu, Dn, cj = R.shape
    if A.shape[0] != ci or A.shape[2] != cj or W.shape[0] != Dl or W.shape[3] != Dn:
        raise ValueError("tdvp_apply_local_H: bond dimensions do not match")
    H = torch.empty(ci, 2, cj, dtype=dt, device=dev)
    need = lib.agb_tdvp_local_h_workspace(dtype_code(dt), Dl, Dn, ci, cj)
    ws = ops.workspace(need, dev, "tdvp")
    check(lib.agb_tdvp_local_h(dtype_code(dt), ptr(L), ptr(W), ptr(A), ptr(R), ptr(H), cq, Dl, ci, Dn, cu, cj,
                               ptr(ws), ws.numel(), stream_ptr(dev)), "tdvp_local_h")
    return H
