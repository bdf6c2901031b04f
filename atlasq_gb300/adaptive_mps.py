"""AdaptiveMPS on GB300: drop-in for src/atlas_q/adaptive_mps.py (ATLAS-Q 0.7.0).

Same constructor, attributes and methods as the reference class.  Differences
that a caller can observe are documented where they occur:

* two-site gates are queued and applied as one batched GPU launch per set of
  gates on disjoint bonds (a brickwork layer).  Gates on disjoint bonds act on
  different site tensors, so the result equals applying them one by one.  Any
  read of ``tensors``, ``bond_dims`` or ``statistics``, any single-qubit gate on
  a queued site, and any gate overlapping a queued one flushes the queue first.
* the SVD is a Gram/eigensolver factorisation on the GPU (driver tag
  ``gb300_gram_heevd``); singular values are absorbed to the left exactly as in
  adaptive_mps.py:281-285.
* ``sample()`` right-canonicalises a copy of the state before sampling (the
  reference's left-to-right sampler is only correct on a right-canonical MPS,
  mps_pytorch.py:154-355) and draws Philox4x32-10 uniforms.
"""
import ctypes
import math
import time
from dataclasses import dataclass
from typing import Dict, List, Optional, Union

import numpy as np
import torch

from . import _lib, ops, resident, svd_log
from ._lib import check, dtype_code, ptr, stream_ptr
from .diagnostics import MPSStatistics
from .truncation import check_entropy_sanity

_C64, _C128 = torch.complex64, torch.complex128


@dataclass
class DTypePolicy:
    """adaptive_mps.py:43-48."""

    default: torch.dtype = torch.complex64
    promote_if_cond_gt: float = 1e6


def _dbits(x: float) -> int:
    return int(np.array([x], dtype=np.float64).view(np.int64)[0])


def _bitsd(v: int) -> float:
    return float(np.array([v], dtype=np.int64).view(np.float64)[0])


class AdaptiveMPS:
    """Adaptive-bond MPS with batched GPU two-site updates (adaptive_mps.py:51-623)."""

    def __init__(self, num_qubits: int, bond_dim: int = 8, *, eps_bond: float = 1e-6,
                 chi_max_per_bond: Optional[Union[int, List[int]]] = 256,
                 budget_global_mb: Optional[float] = None, dtype_policy: DTypePolicy = DTypePolicy(),
                 device: str = "cuda", dtype: Optional[torch.dtype] = None, seed: int = 0,
                 device_resident: bool = False):
        if dtype is None:
            dtype = dtype_policy.default
        self.device = _lib.require_cuda(device)
        _lib.load()
        self.num_qubits = num_qubits
        self.dim = 2 ** num_qubits
        self.bond_dim = bond_dim
        self.dtype = dtype
        self.eps_bond = eps_bond
        self.dtype_policy = dtype_policy
        self.budget_global_mb = budget_global_mb
        if isinstance(chi_max_per_bond, int):
            self.chi_max_per_bond = [chi_max_per_bond] * (num_qubits - 1)
        else:
            assert len(chi_max_per_bond) == num_qubits - 1, f"chi_max_per_bond must have length {num_qubits-1}"
            self.chi_max_per_bond = list(chi_max_per_bond)
        self._statistics = MPSStatistics()
        self._log_queue = []
        self._operation_counter = 0
        self._seed = int(seed)
        self._pending = []
        self._pending_sites = set()
        self._pending_1q = []        # queued single-qubit gates (site, U) in order
        # optional callable(mps, [(bond, U4x4), ...]) -> list of ell (eigenpairs to compute per gate)
        self.rank_predictor = None
        self.feature_log = None      # list -> (features, k, full) per gate is appended (predictor training data)
        # SVD-event log (svd_log.py): on when $QIH_SVD_LOG_DIR is set, or assign a logger
        self.svd_logger = svd_log.get_logger()
        self.spectrum_log = None     # list -> (step, bond, singular values computed) per gate
        self._last_entropy = {}      # bond -> entanglement entropy at its last update
        self.rank_fallbacks = 0      # gates re-run at full size after a too-small predicted ell
        # device-resident mode (see resident.py): gates run without host synchronisation
        self.device_resident = device_resident
        self._res = None
        self.unpromoted = 0
        self.ell_total = 0           # eigenpairs computed, summed over gates (fallback runs included)
        self.batch_log = []          # per-flush (n_gates, seconds) for profiling
        self._initialize_zero_state(bond_dim)

    # ------------------------------------------------------------ state / views
    def _initialize_zero_state(self, b: int):
        """|0...0> with the reference's shapes after its QR normalisation
        (adaptive_mps.py:128-139 + mps_pytorch.py:595-604): bond i has
        min(2 * bond_{i-1}, b) with bond_{-1} = 1.  Each site is the isometric
        embedding (a, s) -> c = 2a + s, and the last site selects the all-zero
        path, which is left-canonical and represents |0...0> exactly."""
        n = self.num_qubits
        dims, prev = [], 1
        for i in range(n - 1):
            prev = min(2 * prev, b)
            dims.append(prev)
        self._bond_dims = list(dims) if n > 1 else []
        tensors = []
        for i in range(n):
            l = 1 if i == 0 else dims[i - 1]
            r = 1 if i == n - 1 else dims[i]
            T = torch.zeros(l, 2, r, dtype=self.dtype)
            if i == n - 1:
                T[0, 0, 0] = 1.0
            else:
                for a in range(l):
                    for s in range(2):
                        c = 2 * a + s
                        if c < r:
                            T[a, s, c] = 1.0
            tensors.append(T.to(self.device))
        self._tensors = tensors
        self.is_canonical = True

    def _drain(self):
        """Apply the queued gates (staying in resident mode if active)."""
        if self._pending_1q:
            g1 = self._pending_1q
            self._pending_1q = []
            if self._res is not None:
                resident.single_qubit_entries([(self, q, U) for q, U in g1])
            else:
                apply_single_qubit_entries([(self, q, U) for q, U in g1])
        if self._pending:
            gates = self._pending
            self._pending = []
            self._pending_sites = set()
            if self._res is not None:
                resident.two_site_entries([(self, i, U) for i, U in gates])
            else:
                self._apply_batch(gates)

    def _flush(self):
        """Apply the queued gates and return to host-visible tensors."""
        self._drain()
        if self._res is not None:
            resident.leave(self)

    def promotion_reachable(self) -> bool:
        """Whether the complex128 promotion (adaptive_mps.py:266-274) can fire.

        In complex64 the rank rule's cumulative sum is float32 (each partial
        rounded), so a kept sigma_{k-1} either changed that sum (sigma_{k-1}^2
        >= 2^-25 sigma_0^2) or, when the cap cut first, heads a tail of at most
        n = 2 chi_cap values whose sum the float32 sum still resolves (>= 2^-26
        of the total, or eps^2 of it when 1 - eps^2 is representable):
        sigma_0 / sigma_{k-1} <= sqrt(n 2^26) (1.9e5 at chi_cap 256), so a
        threshold at or above that bound is out of reach.  The one exception is
        a rounding tie: a tail too small to change the partial sums that still
        moves the float32 total up by one ulp lets the cap cut at a value below
        that bound; a resident gate of that kind is counted in ``unpromoted``.
        complex128 never promotes."""
        if self.dtype_policy.default == _C128:
            return False
        n = 2 * max(self.chi_max_per_bond + [1])
        return self.dtype_policy.default != torch.complex64 or \
            self.dtype_policy.promote_if_cond_gt < math.sqrt(n * 2.0 ** 26)

    def _maybe_enter_resident(self):
        # resident mode has no host step between gates, so it is entered only
        # where the host path's per-gate decisions cannot fire: no predictor,
        # budget or logs, and no reachable precision promotion
        if (self.device_resident and self._res is None and self.rank_predictor is None
                and self.budget_global_mb is None and self.feature_log is None and self.svd_logger is None
                and self.spectrum_log is None and not self.promotion_reachable()):
            self._drain()
            resident.enter(self)

    def flush(self):
        """Apply all queued two-site gates now."""
        self._flush()

    @property
    def tensors(self) -> List[torch.Tensor]:
        self._flush()
        return self._tensors

    @tensors.setter
    def tensors(self, value):
        self._flush()
        self._tensors = list(value)

    @property
    def bond_dims(self) -> List[int]:
        self._flush()
        return self._bond_dims

    @bond_dims.setter
    def bond_dims(self, value):
        self._flush()
        self._bond_dims = list(value)

    @property
    def statistics(self) -> MPSStatistics:
        self._flush()
        if self._log_queue:
            q, self._log_queue = self._log_queue, []
            for step, kw in q:
                self._statistics.record(step=step, **kw)
        return self._statistics

    # ------------------------------------------------------------ stats API
    def _log_operation(self, **kwargs):
        # recorded when the statistics are read, off the gate path
        self._log_queue.append((self._operation_counter, kwargs))
        self._operation_counter += 1

    def stats_summary(self) -> Dict[str, float]:
        return self.statistics.summary()

    def global_error_bound(self) -> float:
        return self.statistics.global_error_bound()

    def reset_stats(self):
        self.statistics.reset()
        self._log_queue = []
        self._operation_counter = 0

    # ------------------------------------------------------------ gates
    @torch.no_grad()
    def apply_single_qubit_gate(self, q: int, U2: torch.Tensor):
        """adaptive_mps.py:159-180; applies U^T like the reference.  Queued: all
        queued single-qubit gates run in one launch at the next flush, before the
        queued two-site gates (a single-qubit gate on a site with a queued
        two-site gate flushes first, so the order of operations is kept)."""
        assert 0 <= q < self.num_qubits, f"Qubit index {q} out of range"
        assert U2.shape == (2, 2), "U2 must be 2x2"
        self._maybe_enter_resident()
        if q in self._pending_sites:
            self._drain()
        self._pending_1q.append((q, U2))
        self.is_canonical = False

    @torch.no_grad()
    def apply_two_site_gate(self, i: int, U4: torch.Tensor):
        """adaptive_mps.py:182-308 (queued; see the module docstring)."""
        assert 0 <= i < self.num_qubits - 1, f"Bond index {i} out of range"
        if U4.shape == (2, 2, 2, 2):
            U = U4.reshape(4, 4)
        elif U4.shape == (4, 4):
            U = U4
        else:
            raise ValueError(f"U4 must be (2,2,2,2) or (4,4), got {U4.shape}")
        self._maybe_enter_resident()
        if i in self._pending_sites or (i + 1) in self._pending_sites:
            self._drain()
        self._pending.append((i, U))
        self._pending_sites.update((i, i + 1))
        self.is_canonical = False

    def _eps_bits(self) -> int:
        c = getattr(self, "_eps_cache", None)
        if c is None or c[0] != self.eps_bond:
            c = (self.eps_bond, _dbits(self.eps_bond))
            self._eps_cache = c
        return c[1]

    def _budget_ok_fn(self, chiL, chiM, chiR, dt):
        if self.budget_global_mb is None:
            return None
        bpe = torch.finfo(dt).bits // 8

        def ok(k):
            before = (chiL * chiM + chiM * chiR) * 2 * bpe
            after = (chiL * k + k * chiR) * 2 * bpe
            delta = max(0, after - before)
            cur = sum(t.element_size() * t.nelement() for t in self._tensors) / (1024 ** 2)
            return (cur + delta / (1024 ** 2)) < self.budget_global_mb
        return ok

    def _apply_batch(self, gates):
        apply_gate_entries([(self, i, U) for i, U in gates])

    # ------------------------------------------------------------ canonical forms
    def _common(self, T):
        return T if T.dtype == self.dtype and T.is_contiguous() else T.to(self.dtype).contiguous()

    @torch.no_grad()
    def to_left_canonical(self):
        """adaptive_mps.py:310-339."""
        self._flush()
        T = self._tensors
        for i in range(self.num_qubits - 1):
            A = self._common(T[i])
            l, p, r = A.shape
            Q, R = ops.qr(A.reshape(l * p, r))
            m = Q.shape[1]
            T[i] = Q.reshape(l, p, m)
            B = self._common(T[i + 1])
            T[i + 1] = ops.cgemm(R, B.reshape(B.shape[0], -1)).reshape(m, 2, B.shape[2])
            if i < len(self._bond_dims):
                self._bond_dims[i] = m
        self.is_canonical = True

    def canonicalize_left_to_right(self):
        self.to_left_canonical()

    @torch.no_grad()
    def _right_sweep(self, tensors, stop=0):
        """mps_pytorch.py:123-152 on a list, sites n-1 .. stop+1."""
        for i in range(len(tensors) - 1, stop, -1):
            Tm = self._common(tensors[i])
            l, p, r = Tm.shape
            Q, R = ops.qr(Tm.reshape(l, p * r), transA=True, trans_out=True)
            kk = Q.shape[0]
            tensors[i] = Q.reshape(kk, p, r)
            prev = self._common(tensors[i - 1])
            pl, pp, pr = prev.shape
            tensors[i - 1] = ops.cgemm(prev.reshape(pl * pp, pr), R).reshape(pl, pp, kk)
            if i - 1 < len(self._bond_dims):
                self._bond_dims[i - 1] = kk
        return tensors

    @torch.no_grad()
    def canonicalize_right_to_left(self):
        self._flush()
        self._right_sweep(self._tensors)

    @torch.no_grad()
    def to_mixed_canonical(self, center: int):
        """adaptive_mps.py:346-385."""
        assert 0 <= center < self.num_qubits, "Center out of range"
        self._flush()
        T = self._tensors
        for i in range(center):
            A = self._common(T[i])
            l, p, r = A.shape
            Q, R = ops.qr(A.reshape(l * p, r))
            T[i] = Q.reshape(l, p, Q.shape[1])
            B = self._common(T[i + 1])
            T[i + 1] = ops.cgemm(R, B.reshape(B.shape[0], -1)).reshape(Q.shape[1], 2, B.shape[2])
            self._bond_dims[i] = Q.shape[1]
        self._right_sweep(T, stop=center)

    def _normalize(self):
        """mps_pytorch.py:595-604."""
        self.to_left_canonical()
        last = self._tensors[-1]
        nrm = float(torch.linalg.vector_norm(last).item())
        if nrm > 0:
            self._tensors[-1] = last / nrm

    # ------------------------------------------------------------ sampling
    def sample(self, num_shots: int = 1, seed: Optional[int] = None) -> List[int]:
        return self.measure(num_shots, seed=seed)

    def measure(self, num_shots: int = 1, seed: Optional[int] = None) -> List[int]:
        """mps_pytorch.py:373-385 -> right-canonical Philox sweep sampler."""
        return self.sweep_sample(num_shots, seed=seed)

    def sweep_sample(self, num_shots: int = 1, seed: Optional[int] = None) -> List[int]:
        from .sampling import sample_mps
        self._flush()
        bits = sample_mps(self, num_shots, seed=self._seed if seed is None else seed)
        return bits.cpu().tolist()

    # ------------------------------------------------------------ dense / amplitudes
    @torch.no_grad()
    def to_statevector(self) -> torch.Tensor:
        """adaptive_mps.py:444-481 (n <= 20)."""
        if self.num_qubits > 20:
            raise ValueError(f"Converting {self.num_qubits} qubits to statevector would require "
                             f"{2**self.num_qubits} amplitudes. Use get_amplitude() for large systems.")
        T = self.tensors
        res = self._common(T[0]).reshape(2, -1)  # [2, chi1]
        for t in T[1:]:
            t = self._common(t)
            res = ops.cgemm(res.contiguous(), t.reshape(t.shape[0], -1)).reshape(-1, t.shape[2])
        return res.reshape(-1)

    @torch.no_grad()
    def get_amplitude(self, basis_state: int) -> complex:
        """mps_pytorch.py:606-627 (qubit 0 = most significant bit)."""
        T = self.tensors
        n = self.num_qubits
        bits = [(basis_state >> (n - 1 - i)) & 1 for i in range(n)]
        res = self._common(T[0])[:, bits[0], :].contiguous()
        for i in range(1, n):
            res = ops.cgemm(res, self._common(T[i])[:, bits[i], :].contiguous())
        amp = res[0, 0].item()
        return complex(amp)

    def get_probability(self, basis_state: int) -> float:
        return abs(self.get_amplitude(basis_state)) ** 2

    def memory_usage(self) -> int:
        return sum(t.element_size() * t.nelement() for t in self.tensors)

    def get_memory_usage(self) -> int:
        return self.memory_usage()

    # ------------------------------------------------------------ snapshots
    def snapshot(self, path: str):
        """adaptive_mps.py:387-404 (same dict keys)."""
        torch.save({"tensors": [t.cpu() for t in self.tensors], "bond_dims": self.bond_dims,
                    "num_qubits": self.num_qubits, "eps_bond": self.eps_bond,
                    "chi_max_per_bond": self.chi_max_per_bond, "statistics": self.statistics.logs}, path)

    @staticmethod
    def load_snapshot(path: str, device: str = "cuda") -> "AdaptiveMPS":
        """adaptive_mps.py:406-433."""
        data = torch.load(path, weights_only=False)
        mps = AdaptiveMPS(num_qubits=data["num_qubits"], bond_dim=max(data["bond_dims"]) if data["bond_dims"] else 1,
                          eps_bond=data["eps_bond"], chi_max_per_bond=data["chi_max_per_bond"], device=device)
        mps.tensors = [t.to(device) for t in data["tensors"]]
        mps.bond_dims = data["bond_dims"]
        if "statistics" in data:
            mps.statistics.logs = data["statistics"]
        return mps

    def to_numpy_mps(self):
        return {"tensors": [t.cpu().numpy() for t in self.tensors], "num_qubits": self.num_qubits,
                "bond_dim": self.bond_dim, "is_canonical": self.is_canonical}

    # ------------------------------------------------------------ named gates (:489-619)
    def _g1(self, rows):
        return torch.tensor(rows, dtype=self.dtype)

    def h(self, qubit):
        self.apply_single_qubit_gate(qubit, self._g1([[1, 1], [1, -1]]) / math.sqrt(2.0))

    def x(self, qubit):
        self.apply_single_qubit_gate(qubit, self._g1([[0, 1], [1, 0]]))

    def y(self, qubit):
        self.apply_single_qubit_gate(qubit, self._g1([[0, -1j], [1j, 0]]))

    def z(self, qubit):
        self.apply_single_qubit_gate(qubit, self._g1([[1, 0], [0, -1]]))

    def s(self, qubit):
        self.apply_single_qubit_gate(qubit, self._g1([[1, 0], [0, 1j]]))

    def sdg(self, qubit):
        self.apply_single_qubit_gate(qubit, self._g1([[1, 0], [0, -1j]]))

    def t(self, qubit):
        self.apply_single_qubit_gate(qubit, self._g1([[1, 0], [0, complex(math.cos(math.pi / 4), math.sin(math.pi / 4))]]))

    def tdg(self, qubit):
        self.apply_single_qubit_gate(qubit, self._g1([[1, 0], [0, complex(math.cos(math.pi / 4), -math.sin(math.pi / 4))]]))

    def rx(self, qubit, theta):
        th = float(theta)
        c, s = math.cos(th / 2), math.sin(th / 2)
        self.apply_single_qubit_gate(qubit, self._g1([[c, -1j * s], [-1j * s, c]]))

    def ry(self, qubit, theta):
        th = float(theta)
        c, s = math.cos(th / 2), math.sin(th / 2)
        self.apply_single_qubit_gate(qubit, self._g1([[c, -s], [s, c]]))

    def rz(self, qubit, theta):
        th = float(theta)
        self.apply_single_qubit_gate(qubit, self._g1([[complex(math.cos(th / 2), -math.sin(th / 2)), 0],
                                                      [0, complex(math.cos(th / 2), math.sin(th / 2))]]))

    def _two(self, q0, q1, rows, ordered):
        if abs(q0 - q1) != 1:
            raise NotImplementedError("Only adjacent qubit gates supported in MPS")
        if ordered and q0 > q1:
            raise NotImplementedError("Reversed control/target not yet supported")
        self.apply_two_site_gate(min(q0, q1), torch.tensor(rows, dtype=self.dtype))

    def cnot(self, control, target):
        self._two(control, target, [[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 0, 1], [0, 0, 1, 0]], True)

    def cx(self, control, target):
        self.cnot(control, target)

    def cz(self, q0, q1):
        self._two(q0, q1, [[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 1, 0], [0, 0, 0, -1]], False)

    def cy(self, control, target):
        self._two(control, target, [[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 0, -1j], [0, 0, 1j, 0]], True)

    def swap(self, q0, q1):
        self._two(q0, q1, [[1, 0, 0, 0], [0, 0, 1, 0], [0, 1, 0, 0], [0, 0, 0, 1]], False)


# ---------------------------------------------------------------- batched single-qubit gates
def apply_single_qubit_entries(entries):
    """Apply queued single-qubit gates ``[(mps, site, U2), ...]`` (any number of
    instances, in order per site) with one launch of agb_single_qubit_batch."""
    if not entries:
        return
    lib = _lib.load()
    device = entries[0][0].device
    groups = {}
    for m, q, U in entries:
        if m.device != device:
            raise ValueError("batched entries must share the device")
        groups.setdefault((id(m), q), (m, q, []))[2].append(U)
    dts = {m._tensors[q].dtype for m, q, _ in groups.values()}
    if len(dts) != 1:
        for dt in dts:  # one launch per tensor dtype
            apply_single_qubit_entries([e for e in entries if e[0]._tensors[e[1]].dtype == dt])
        return
    dt = dts.pop()
    if len(groups) > 65535:
        keys = list(groups)
        for c in range(0, len(keys), 65535):
            part = set(keys[c:c + 65535])
            apply_single_qubit_entries([e for e in entries if (id(e[0]), e[1]) in part])
        return
    ng = len(groups)
    nu = len(entries)
    desc = np.zeros(ng * 5 + nu, dtype=np.int64)
    keep = []
    host_U, host_slot = [], []
    first = 0
    max_elems = 1
    for g, (m, q, Us) in enumerate(groups.values()):
        T = m._tensors[q]
        if not T.is_contiguous():
            T = T.contiguous()
            m._tensors[q] = T
        keep.append(T)
        desc[5 * g:5 * g + 5] = (T.data_ptr(), T.shape[0], T.shape[2], first, len(Us))
        max_elems = max(max_elems, T.shape[0] * T.shape[2])
        for j, U in enumerate(Us):
            if U.device == device:
                if U.dtype != dt or not U.is_contiguous():
                    U = U.to(dtype=dt).contiguous()  # device-side copy
                keep.append(U)
                desc[ng * 5 + first + j] = U.data_ptr()
            else:
                host_U.append(U.detach().to("cpu", dt))
                host_slot.append(ng * 5 + first + j)
        first += len(Us)
    if host_U:
        Ud = torch.stack(host_U).to(device)
        keep.append(Ud)
        es = 4 * Ud.element_size()
        for j, slot in enumerate(host_slot):
            desc[slot] = Ud.data_ptr() + j * es
    desc_dev = torch.from_numpy(desc).to(device, non_blocking=False)
    check(lib.agb_single_qubit_batch(dtype_code(dt), ng, ptr(desc_dev), max_elems, stream_ptr(device)),
          "single_qubit_batch")
    # buffers released here return to the stream-ordered caching allocator, so
    # they are not reused before this launch has consumed them
    del keep


# ---------------------------------------------------------------- batched two-site updates
def apply_gate_entries(entries):
    """Apply queued two-site gates ``[(mps, bond, U4), ...]`` as one batched
    launch sequence.  Entries may come from many AdaptiveMPS instances (of any
    sizes); within one instance their bonds must be disjoint.  Per instance the
    result, the statistics and the rank-fallback / precision-promotion rules
    are exactly those of applying its gates alone (adaptive_mps.py:182-308)."""
    if not entries:
        return
    t0 = time.perf_counter()
    mps0 = entries[0][0]
    dt = mps0.dtype_policy.default
    device = mps0.device
    for m, _, _ in entries:
        if m.dtype_policy.default != dt or m.device != device:
            raise ValueError("batched entries must share the dtype policy and the device")
    # group positions per instance (predictor and feature hooks see one instance at a time)
    groups = {}
    for g, (m, i, U) in enumerate(entries):
        groups.setdefault(id(m), (m, []))[1].append(g)
    ells = None
    feats = {}
    for m, idx in groups.values():
        if m.feature_log is not None:
            from .rank_predictor import gate_features
            feats[id(m)] = (idx, gate_features(m, [(entries[g][1], entries[g][2]) for g in idx]))
        if m.rank_predictor is not None:
            if ells is None:
                ells = [0] * len(entries)
            pe = m.rank_predictor(m, [(entries[g][1], entries[g][2]) for g in idx])
            for g, e in zip(idx, pe):
                ells[g] = int(e)
    spectra = any(m.svd_logger is not None or m.spectrum_log is not None for m, _ in groups.values())
    res = _run_pipeline(entries, dt, ells, spectra=spectra)
    for m, idx in groups.values():
        m.ell_total += sum(res[g]["ell"] for g in idx)
    # rank fallback: predicted size too small -> rerun those gates at full size
    redo = [g for g, r in enumerate(res) if r["status"] == _lib.AGB_ERR_RANK]
    if redo:
        full = _run_pipeline([entries[g] for g in redo], dt, None, all_vectors=True, spectra=spectra)
        for g, r in zip(redo, full):
            r["driver"] = "gb300_gram_heevd_full"
            res[g] = r
            entries[g][0].rank_fallbacks += 1
            entries[g][0].ell_total += r["ell"]
    # precision promotion (adaptive_mps.py:268-274), and the robust-SVD
    # fallback (linalg_robust.py:17-52 retries a failed factorisation at
    # higher precision): a complex64 gate whose eigenvectors still failed the
    # orthogonality guard after the device repair is re-run in complex128
    promote = [g for g, r in enumerate(res)
               if dt != _C128 and (r["status"] == _lib.AGB_ERR_NOCONV or (
                   math.isfinite(r["condS"]) and r["condS"] > entries[g][0].dtype_policy.promote_if_cond_gt))]
    if promote:
        r2 = _run_pipeline([entries[g] for g in promote], _C128, None, all_vectors=True, spectra=spectra)
        for g, r in zip(promote, r2):
            r["driver"] = ("gb300_gram_heevd_c128_robust" if res[g]["status"] == _lib.AGB_ERR_NOCONV
                           else "gb300_gram_heevd_c128")
            res[g] = r
    elapsed = (time.perf_counter() - t0) * 1000.0 / len(entries)
    for m, idx in groups.values():
        m.batch_log.append((len(idx), elapsed * len(idx) / 1000.0))
        fi = feats.get(id(m))
        for j, g in enumerate(idx):
            _, i, _ = entries[g]
            r = res[g]
            m._tensors[i] = r["A"]
            m._tensors[i + 1] = r["B"]
            m._bond_dims[i] = r["k"]
            m._last_entropy[i] = r["entropy"]
            if fi is not None:
                m.feature_log.append((fi[1][0][j], r["k"], int(fi[1][1][j])))
            if "sigma" in r:
                if m.spectrum_log is not None:
                    m.spectrum_log.append((m._operation_counter, i, r["sigma"]))
                if m.svd_logger is not None:
                    m.svd_logger.spectrum(bond=i, pre_rank=r["chiM"], chi_max=m.chi_max_per_bond[i], tol=m.eps_bond,
                                          total_weight=r["total"], sigma=r["sigma"].tolist(), keep=r["k"],
                                          step=m._operation_counter, chi_left=r["chiL"], chi_right=r["chiR"],
                                          features=None if fi is None else list(fi[1][0][j]),
                                          full=None if fi is None else int(fi[1][1][j]))
            if not check_entropy_sanity(r["entropy"], r["chiL"], r["chiR"]):
                print(f"Warning: Entropy {r['entropy']:.3f} exceeds physical bound at bond {i}")
            m._log_operation(bond=i, k_star=r["k"], chi_before=r["chiM"], chi_after=r["k"],
                             eps_local=r["eps_local"], entropy=r["entropy"], svd_driver=r["driver"],
                             dtype=str(r["dtype"]), ms_elapsed=elapsed, condS=r["condS"])


def _run_pipeline(entries, dt, ells, all_vectors=False, cluster_tol=None, spectra=False, guard=True):
    """One batched launch sequence: plan -> run -> read ranks -> finalize.
    By default the device computes eigenvectors only for the eigenvalues the
    rank rule can keep (AGB_D_NVEC = 0); ``all_vectors`` computes every one
    (the re-run of a gate that reported AGB_ERR_RANK).  ``cluster_tol``
    overrides the eigensolver's relative cluster tolerance (AGB_D_CTOL; the
    library default is 1e-5).  ``spectra`` also reads back each gate's
    computed singular values (result key ``sigma``, descending).
    ``guard=False`` only measures the eigenvector orthogonality guard (result
    keys ``orth`` / ``orth_w``: the largest overlap before the polish, and the
    same weighted by the smaller eigenvalue over the largest) instead of
    repairing or rejecting on it.
    Descriptor rows are built and read with NumPy; the two small copies per
    batch (descriptors up, results down) are the only host synchronisation."""
    lib = _lib.load()
    code = dtype_code(dt)
    device = entries[0][0].device
    G = len(entries)
    desc = np.zeros((G, _lib.D_NFIELDS), dtype=np.int64)
    keep = []
    if all(U.device == device for _, _, U in entries):
        Us = torch.stack([U.to(dtype=dt) for _, _, U in entries]).contiguous()
    else:
        Us = torch.stack([U.to(dtype=dt, device="cpu") for _, _, U in entries]).contiguous()
        Us = Us.to(device, non_blocking=True)
    keep.append(Us)
    u_base, u_stride = Us.data_ptr(), 16 * Us.element_size()
    meta = []
    seeds = {}
    cols = {k: [0] * G for k in ("A", "B", "L", "M", "R", "cap", "eps", "seed")}
    for g, (m, i, _) in enumerate(entries):
        A = m._tensors[i]
        B = m._tensors[i + 1]
        if A.dtype != dt or not A.is_contiguous():
            A = A.to(dt).contiguous()
        if B.dtype != dt or not B.is_contiguous():
            B = B.to(dt).contiguous()
        keep += [A, B]
        chiL, chiM, chiR = A.shape[0], A.shape[2], B.shape[2]
        # per-instance seed: (instance seed, operation counter, position in its batch)
        j = seeds.get(id(m), 0)
        seeds[id(m)] = j + 1
        cols["A"][g] = A.data_ptr()
        cols["B"][g] = B.data_ptr()
        cols["L"][g], cols["M"][g], cols["R"][g] = chiL, chiM, chiR
        cols["cap"][g] = m.chi_max_per_bond[i]
        cols["eps"][g] = m._eps_bits()
        cols["seed"][g] = ((m._seed * 1000003 + m._operation_counter) & 0x3FFFFFFFFFFFFFFF) + j
        meta.append((m, i, chiL, chiM, chiR))
    desc[:, _lib.D_A] = cols["A"]
    desc[:, _lib.D_B] = cols["B"]
    desc[:, _lib.D_U] = u_base + np.arange(G, dtype=np.int64) * u_stride
    desc[:, _lib.D_CHIL] = cols["L"]
    desc[:, _lib.D_CHIM] = cols["M"]
    desc[:, _lib.D_CHIR] = cols["R"]
    desc[:, _lib.D_CAP] = cols["cap"]
    desc[:, _lib.D_EPS] = cols["eps"]
    if ells is not None:
        desc[:, _lib.D_ELL] = [int(e) for e in ells]
    desc[:, _lib.D_SEED] = cols["seed"]
    desc[:, _lib.D_NVEC] = -1 if all_vectors else 0
    if cluster_tol is not None:
        desc[:, _lib.D_CTOL] = _dbits(float(cluster_tol))
    maxL, maxM, maxR = max(cols["L"]), max(cols["M"]), max(cols["R"])
    wsz = _lib.SZ(0)
    check(lib.agb_two_site_plan(code, G, desc.ctypes.data_as(ctypes.c_void_p), ctypes.byref(wsz)),
          "two_site_plan")
    maxell = int(desc[:, _lib.D_ELL].max())
    ws = ops.workspace(wsz.value, device, "two_site")
    desc_dev = torch.from_numpy(desc).to(device)
    stream = stream_ptr(device)
    # a gate whose eigenvalue-guided eigenvector count fell short is re-run with
    # every vector on the device; AGB_ERR_RANK then only means a predicted ell
    # below the rank, which the caller re-runs at full size
    check(lib.agb_two_site_run(code, G, ptr(desc_dev), ptr(desc_dev), maxL, maxM, maxR, maxell,
                               ptr(ws), wsz.value, stream,
                               _lib.AGB_RUN_REPAIR | (0 if guard else _lib.AGB_RUN_NO_GUARD)), "two_site_run")
    sig = None
    if spectra:
        cnt = max(1, maxell)
        sig_dev = torch.empty(G, cnt, dtype=torch.float64, device=device)
        check(lib.agb_two_site_spectra(code, G, ptr(desc_dev), ptr(ws), cnt, ptr(sig_dev), stream),
              "two_site_spectra")
        sig = sig_dev.cpu().numpy()
    out = desc_dev.cpu().numpy()
    res = []
    maxk = 1
    sts = out[:, _lib.D_STATUS].tolist()
    ks = out[:, _lib.D_K].tolist()
    reals = np.ascontiguousarray(out[:, [_lib.D_EPSLOC, _lib.D_ENTROPY, _lib.D_CONDS, _lib.D_TOTAL, _lib.D_ORTH,
                                         _lib.D_ORTHW]]).view(np.float64).tolist()
    modes = out[:, _lib.D_MODE].tolist()
    ellv = out[:, _lib.D_ELL].tolist()
    repv = out[:, _lib.D_REPAIR].tolist()
    for g, (m, i, chiL, chiM, chiR) in enumerate(meta):
        row = out[g]
        st = sts[g]
        k = ks[g]
        r = {"status": st, "k": k, "eps_local": reals[g][0], "entropy": reals[g][1], "condS": reals[g][2],
             "chiL": chiL, "chiM": chiM, "chiR": chiR, "driver": "gb300_gram_heevd", "dtype": dt,
             "mode": modes[g], "ell": ellv[g], "repair": repv[g], "total": reals[g][3],
             "orth": math.sqrt(max(reals[g][4], 0.0)), "orth_w": reals[g][5]}
        if sig is not None:
            row_s = sig[g]
            r["sigma"] = row_s[:int(np.count_nonzero(row_s))].copy()
        if st not in (_lib.AGB_OK, _lib.AGB_ERR_RANK) and not (st == _lib.AGB_ERR_NOCONV and dt != _C128):
            check(st, f"two-site update on bond {i}")
        ok = m._budget_ok_fn(chiL, chiM, chiR, dt)
        if ok is not None and st == _lib.AGB_OK:
            kk = k
            while kk > 1 and not ok(kk):
                kk -= 1
            if kk != k:
                r["k"] = k = kk
                row[_lib.D_K] = kk
        if st == _lib.AGB_OK:
            A_new = torch.empty(chiL, 2, k, dtype=dt, device=device)
            B_new = torch.empty(k, 2, chiR, dtype=dt, device=device)
            row[_lib.D_ANEW] = A_new.data_ptr()
            row[_lib.D_BNEW] = B_new.data_ptr()
            r["A"], r["B"] = A_new, B_new
            maxk = max(maxk, k)
        else:
            row[_lib.D_K] = 0
            row[_lib.D_ANEW] = 0
            row[_lib.D_BNEW] = 0
        res.append(r)
    desc_dev.copy_(torch.from_numpy(out))
    check(lib.agb_two_site_finalize(code, G, ptr(desc_dev), maxL, maxR, maxk, ptr(ws), stream),
          "two_site_finalize")
    return res
