"""NumPy restatement of the reference AdaptiveMPS hot path (test infrastructure only).

Every function cites the reference file:line it restates (paths relative to the
followthesapper/ATLAS-Q 0.7.0 project root).  Two precisions are supported:

* ``complex64``  -- mirrors the reference's default complex64 arithmetic
  (reference-parity mode);
* ``complex128`` -- the FP64 oracle (the reference run with
  ``DTypePolicy(default=torch.complex128)``).

Conventions reproduced on purpose (they differ from textbook physics):
  * single-qubit gates apply U^T  (adaptive_mps.py:177, einsum "st,asb->atb");
  * two-qubit gates apply U in the fused-path order, site i = high bit
    (mps_complex.py:343-368);
  * singular values are absorbed into the LEFT factor (adaptive_mps.py:281-285);
  * MPO expectations contract W[l, s, t, r] with the ket on s and the bra on t,
    i.e. they evaluate <psi| O^T |psi> (mpo_ops.py:1145).
"""
import math

import numpy as np

from .philox import sample_uniforms

F32 = np.float32


# --------------------------------------------------------------------------
# truncation.py:21-83  choose_rank_from_sigma
# --------------------------------------------------------------------------
def choose_rank_from_sigma(S, eps_bond, chi_cap, budget_ok=lambda k: True):
    """Restates truncation.py:21-83 with torch-CPU float32 semantics.

    * ``E = (S*S).cumsum(0)``: torch CPU accumulates a float32 cumsum in double
      and rounds each partial sum to float32 (truncation.py:52).
    * ``thresh = (1 - eps^2) * total`` is float32 (python scalar x float32 tensor).
    * ``k_tol = searchsorted(E, thresh) + 1`` (left search), capped by len(S)
      and chi_cap, then reduced while ``budget_ok`` fails (truncation.py:59-67).
    * eps_local = sqrt(clamp(total - E[k-1], 0)) (:70); entropy in nats over the
      kept part (:73-75); condS = S[0]/S[k-1] (:78-81).
    Float64 input (complex128 oracle) uses float64 throughout.
    """
    S = np.asarray(S)
    if S.size == 0:
        return 0, 0.0, 0.0, float("inf")
    if S.dtype == np.float32:
        sq = (S * S).astype(np.float32)
        E = np.cumsum(sq.astype(np.float64)).astype(np.float32)
        total = E[-1]
        if total < 1e-30:
            return 1, 0.0, 0.0, float("inf")
        thresh = np.float32(np.float32(1.0 - eps_bond ** 2) * total)
    else:
        sq = S * S
        E = np.cumsum(sq)
        total = E[-1]
        if total < 1e-30:
            return 1, 0.0, 0.0, float("inf")
        thresh = (1.0 - eps_bond ** 2) * total
    k_tol = int(np.searchsorted(E, thresh, side="left")) + 1
    k_tol = min(k_tol, S.size)
    k = min(k_tol, chi_cap)
    while k > 1 and not budget_ok(k):
        k -= 1
    eps_local = float(np.sqrt(max(total - E[k - 1], 0.0)))
    kept = S[:k].astype(np.float64)
    p = kept * kept / np.sum(kept * kept)
    entropy = float(-(p * np.log(np.clip(p, 1e-30, None))).sum())
    if k > 1 and S[k - 1] > 0:
        condS = float(S[0] / S[k - 1])
    else:
        condS = float("inf")
    return k, eps_local, entropy, condS


def check_entropy_sanity(entropy, chi_left, chi_right):
    """truncation.py:104-122."""
    return entropy <= math.log2(min(chi_left * 2, 2 * chi_right)) + 1e-6


# --------------------------------------------------------------------------
# mps_complex.py:343-368  fused_two_qubit_gate_pytorch
# --------------------------------------------------------------------------
def fused_two_qubit_gate(A, B, U):
    """X[(l,p),(q,j)] = sum_{p'q'} U[2p+q, 2p'+q'] sum_r A[l,p',r] B[r,q',j]."""
    li, _, _ = A.shape
    _, _, rj = B.shape
    psi = np.einsum("lpr,rqj->lpqj", A, B)
    psi = psi.transpose(1, 2, 0, 3).reshape(4, li * rj)
    out = U @ psi
    return out.reshape(2, 2, li, rj).transpose(2, 0, 1, 3).reshape(li * 2, 2 * rj)


def thin_svd(X):
    """Thin SVD (reference: robust_svd, linalg_robust.py:17-52)."""
    U, S, Vh = np.linalg.svd(X, full_matrices=False)
    return U, S.astype(np.float32 if X.dtype == np.complex64 else np.float64), Vh


class OracleMPS:
    """AdaptiveMPS restated (adaptive_mps.py:51-623, mps_pytorch.py:44-655)."""

    def __init__(self, num_qubits, bond_dim=1, eps_bond=1e-6, chi_max_per_bond=256,
                 dtype=np.complex128, promote_if_cond_gt=1e6, budget_global_mb=None):
        self.num_qubits = num_qubits
        self.dtype = np.dtype(dtype)
        self.eps_bond = eps_bond
        self.promote_if_cond_gt = promote_if_cond_gt
        self.budget_global_mb = budget_global_mb
        if isinstance(chi_max_per_bond, int):
            self.chi_max_per_bond = [chi_max_per_bond] * (num_qubits - 1)
        else:
            assert len(chi_max_per_bond) == num_qubits - 1
            self.chi_max_per_bond = list(chi_max_per_bond)
        self.bond_dims = [bond_dim] * (num_qubits - 1)
        self.logs = {k: [] for k in ("step", "bond", "k_star", "chi_before", "chi_after",
                                     "eps_local", "entropy", "svd_driver", "dtype",
                                     "ms_elapsed", "condS")}
        self._op = 0
        self.is_canonical = False
        self._init_zero_state(bond_dim)

    # mps_pytorch.py:59-89 shapes, adaptive_mps.py:128-139 zero state, :595-604 normalise
    def _init_zero_state(self, b):
        n = self.num_qubits
        shapes = []
        if n == 1:
            shapes = [(1, 2, b)]
        else:
            shapes = [(1, 2, b)] + [(b, 2, b)] * (n - 2) + [(b, 2, 1)]
        self.tensors = []
        for (l, p, r) in shapes:
            T = np.zeros((l, p, r), dtype=self.dtype)
            T[:, 0, :] = np.eye(l, r, dtype=self.dtype)
            self.tensors.append(T)
        self.to_left_canonical()
        last = self.tensors[-1]
        nrm2 = np.sum(np.abs(last) ** 2)
        if nrm2 > 0:
            self.tensors[-1] = (last / np.sqrt(nrm2)).astype(self.dtype)

    # adaptive_mps.py:159-180 (applies U^T)
    def apply_single_qubit_gate(self, q, U2):
        T = self.tensors[q]
        self.tensors[q] = np.einsum("st,asb->atb", np.asarray(U2, dtype=T.dtype), T)
        self.is_canonical = False

    def memory_usage(self):
        return sum(t.nbytes for t in self.tensors)

    # adaptive_mps.py:182-308
    def apply_two_site_gate(self, i, U4):
        A, B = self.tensors[i], self.tensors[i + 1]
        chiL, chiM, chiR = A.shape[0], A.shape[2], B.shape[2]
        local = self.dtype
        A = A.astype(local)
        B = B.astype(local)
        U = np.asarray(U4).reshape(4, 4).astype(local)
        X = fused_two_qubit_gate(A, B, U)
        Uu, S, Vh = thin_svd(X)
        cap = self.chi_max_per_bond[i]

        def budget_ok(k):
            if self.budget_global_mb is None:
                return True
            bpe = np.dtype(local).itemsize // 2
            before = (chiL * chiM + chiM * chiR) * 2 * bpe
            after = (chiL * k + k * chiR) * 2 * bpe
            delta = max(0, after - before)
            cur = self.memory_usage() / (1024 ** 2)
            return (cur + delta / (1024 ** 2)) < self.budget_global_mb

        k, eps_loc, entropy, condS = choose_rank_from_sigma(S, self.eps_bond, cap, budget_ok)
        if math.isfinite(condS) and condS > self.promote_if_cond_gt:
            X = X.astype(np.complex128)
            Uu, S, Vh = thin_svd(X)
            k, eps_loc, entropy, condS = choose_rank_from_sigma(S, self.eps_bond, cap, budget_ok)
            local = np.complex128
        US = Uu[:, :k] * S[:k]
        self.tensors[i] = US.reshape(chiL, 2, k)
        self.tensors[i + 1] = Vh[:k, :].reshape(k, 2, chiR)
        self.bond_dims[i] = k
        for key, val in (("step", self._op), ("bond", i), ("k_star", k), ("chi_before", chiM),
                         ("chi_after", k), ("eps_local", eps_loc), ("entropy", entropy),
                         ("svd_driver", "oracle_numpy"), ("dtype", str(np.dtype(local))),
                         ("ms_elapsed", 0.0), ("condS", condS)):
            self.logs[key].append(val)
        self._op += 1
        self.is_canonical = False
        return S

    # adaptive_mps.py:310-339  (QR; R absorbed into the right neighbour)
    def to_left_canonical(self):
        for i in range(self.num_qubits - 1):
            A = self.tensors[i]
            l, p, r = A.shape
            Q, R = np.linalg.qr(A.reshape(l * p, r))
            m = Q.shape[1]
            self.tensors[i] = Q.reshape(l, p, m)
            self.tensors[i + 1] = np.einsum("ij,jkl->ikl", R, self.tensors[i + 1])
            if i < len(self.bond_dims):
                self.bond_dims[i] = m
        self.is_canonical = True

    canonicalize_left_to_right = to_left_canonical

    # mps_pytorch.py:123-152
    def canonicalize_right_to_left(self):
        for i in range(self.num_qubits - 1, 0, -1):
            T = self.tensors[i]
            l, p, r = T.shape
            Q, R = np.linalg.qr(T.reshape(l, p * r).T)
            Q = Q.T
            R = R.T
            self.tensors[i] = Q.reshape(Q.shape[0], p, r)
            prev = self.tensors[i - 1]
            pl, pp, pr = prev.shape
            self.tensors[i - 1] = (prev.reshape(pl * pp, pr) @ R).reshape(pl, pp, R.shape[1])

    # adaptive_mps.py:346-385
    def to_mixed_canonical(self, center):
        for i in range(center):
            A = self.tensors[i]
            l, p, r = A.shape
            Q, R = np.linalg.qr(A.reshape(l * p, r))
            self.tensors[i] = Q.reshape(l, p, Q.shape[1])
            self.tensors[i + 1] = np.einsum("ij,jkl->ikl", R, self.tensors[i + 1])
        for i in range(self.num_qubits - 1, center, -1):
            B = self.tensors[i]
            l, p, r = B.shape
            Q, R = np.linalg.qr(B.transpose(1, 2, 0).reshape(p * r, l))
            self.tensors[i] = Q.T.reshape(Q.shape[1], p, r)
            self.tensors[i - 1] = np.einsum("ijk,kl->ijl", self.tensors[i - 1], R.T)

    # adaptive_mps.py:444-481
    def to_statevector(self):
        res = self.tensors[0]
        for t in self.tensors[1:]:
            res = np.einsum("...i,ijk->...jk", res, t)
        return res.reshape(-1)

    # mps_pytorch.py:606-627 (qubit 0 = most significant bit)
    def get_amplitude(self, basis_state):
        n = self.num_qubits
        bits = [(basis_state >> (n - 1 - i)) & 1 for i in range(n)]
        res = self.tensors[0][:, bits[0], :]
        for i in range(1, n):
            res = res @ self.tensors[i][:, bits[i], :]
        return complex(res[0, 0])


# --------------------------------------------------------------------------
# Free functions on tensor lists
# --------------------------------------------------------------------------
def right_canonicalize(tensors):
    """mps_pytorch.py:123-152 on a list (returns a new list, FP64)."""
    ts = [np.asarray(t, dtype=np.complex128) for t in tensors]
    for i in range(len(ts) - 1, 0, -1):
        l, p, r = ts[i].shape
        Q, R = np.linalg.qr(ts[i].reshape(l, p * r).T)
        Q, R = Q.T, R.T
        ts[i] = Q.reshape(Q.shape[0], p, r)
        pl, pp, pr = ts[i - 1].shape
        ts[i - 1] = (ts[i - 1].reshape(pl * pp, pr) @ R).reshape(pl, pp, R.shape[1])
    return ts


def batch_sweep_sample(tensors, num_shots, seed, shot_offset=0, chunk=4096):
    """FP64 restatement of mps_pytorch.py:247-355 with Philox uniforms replacing
    ``torch.multinomial``.  Returns (samples int64[num_shots], pzero float64
    [num_shots, n]) where pzero is the normalised P(0) used at each decision
    (kept to count near-threshold decision flips).  Qubit 0 is the MSB (:321).
    """
    n = len(tensors)
    ts = [np.asarray(t, dtype=np.complex128) for t in tensors]
    out = np.zeros(num_shots, dtype=np.int64)
    pz_all = np.zeros((num_shots, n), dtype=np.float64)
    for c0 in range(0, num_shots, chunk):
        c1 = min(num_shots, c0 + chunk)
        ns = c1 - c0
        shot_ids = np.arange(c0, c1, dtype=np.uint64) + np.uint64(shot_offset)
        left = np.ones((ns, 1), dtype=np.complex128)
        samples = np.zeros(ns, dtype=np.int64)
        for i in range(n):
            T = ts[i]
            t0 = left @ T[:, 0, :]
            t1 = left @ T[:, 1, :]
            p0 = np.sum(np.abs(t0) ** 2, axis=-1) + 1e-15
            p1 = np.sum(np.abs(t1) ** 2, axis=-1) + 1e-15
            pz = p0 / (p0 + p1)
            u = sample_uniforms(seed, shot_ids, i)
            outc = (u >= pz).astype(np.int64)
            pz_all[c0:c1, i] = pz
            samples = (samples << 1) | outc
            left = np.where(outc[:, None] == 1, t1, t0)
        out[c0:c1] = samples
    return out, pz_all


def expectation_product(tensors, ops):
    """mpo_ops.py:1085-1169 for a bond-1 MPO built from 2x2 local operators
    (``MPO.from_local_ops``, mpo_ops.py:70-86).  Evaluates the reference einsum
    'Lab,atr,LstR,bsB->RrB' (W[s,t] with ket s, bra t) and divides by the norm
    sweep.  ``ops`` maps site -> 2x2 operator; identity elsewhere."""
    E = np.ones((1, 1), dtype=np.complex128)
    N = np.ones((1, 1), dtype=np.complex128)
    for i, A in enumerate(tensors):
        A = np.asarray(A, dtype=np.complex128)
        W = np.asarray(ops.get(i, np.eye(2)), dtype=np.complex128)
        E = _env_step(E, A, W)
        N = _env_step(N, A, None)
    return complex(E[0, 0] / N[0, 0])


def _env_step(E, A, W):
    """E'[r, B] = sum conj(A[a, t, r]) W[s, t] E[a, b] A[b, s, B] (the reference's
    per-site einsum with a [1, 2, 2, 1] MPO tensor; W = None is the identity)."""
    la, _, ra = A.shape
    M = (E @ A.reshape(la, -1)).reshape(E.shape[0], 2, ra)       # [a, s, B]
    if W is not None:
        M = np.einsum("st,asB->atB", W, M)                        # ket s -> bra t
    return A.reshape(la * 2, ra).conj().T @ M.reshape(la * 2, ra)


def local_expectations(tensors, observables):
    """<psi| prod_i O_i^T |psi> / <psi|psi> for product observables (site -> 2x2)
    with the reference's convention (expectation_product), evaluated from left
    and right identity environments: each observable costs the sites of its
    support instead of a whole sweep (same contractions, other association)."""
    ts = [np.asarray(t, dtype=np.complex128) for t in tensors]
    n = len(ts)
    Lenv = [np.ones((1, 1), dtype=np.complex128)]
    for A in ts:
        Lenv.append(_env_step(Lenv[-1], A, None))
    Renv = [None] * (n + 1)
    Renv[n] = np.ones((1, 1), dtype=np.complex128)
    for i in range(n - 1, -1, -1):
        A = ts[i]
        la, _, ra = A.shape
        X = (A.reshape(la * 2, ra) @ Renv[i + 1]).reshape(la, 2 * ra)   # [(b, s), r'] -> [b, (s, r')]
        Renv[i] = X @ A.reshape(la, 2 * ra).conj().T                    # [ket b, bra a]
    norm = complex(np.trace(Lenv[n] @ Renv[n]))
    out = []
    for obs in observables:
        sites = sorted(obs)
        E = Lenv[sites[0]]
        for i in range(sites[0], sites[-1] + 1):
            E = _env_step(E, ts[i], np.asarray(obs[i], np.complex128) if i in obs else None)
        out.append(complex(np.trace(E @ Renv[sites[-1] + 1])) / norm)
    return out


def mps_overlap(ta, tb):
    """<a|b> for two MPS given as tensor lists."""
    E = np.ones((1, 1), dtype=np.complex128)
    for A, B in zip(ta, tb):
        A = np.asarray(A, np.complex128)
        B = np.asarray(B, np.complex128)
        la, _, ra = A.shape
        lb, _, rb = B.shape
        T = (E @ B.reshape(lb, 2 * rb)).reshape(la * 2, rb)   # sum_b E[a,b] B[b,s,B]
        E = A.reshape(la * 2, ra).conj().T @ T                 # sum_{a,s} conj(A[a,s,r]) T[a,s,B]
    return complex(E[0, 0])


def mps_fidelity(ta, tb):
    """|<a|b>|^2 / (<a|a><b|b>)."""
    ab = mps_overlap(ta, tb)
    aa = mps_overlap(ta, ta).real
    bb = mps_overlap(tb, tb).real
    return abs(ab) ** 2 / (aa * bb)
