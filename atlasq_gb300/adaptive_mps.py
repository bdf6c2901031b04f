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

from . import _lib, ops
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
                 device: str = "cuda", dtype: Optional[torch.dtype] = None, seed: int = 0):
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
        self._operation_counter = 0
        self._seed = int(seed)
        self._pending = []
        self._pending_sites = set()
        self.rank_predictor = None  # optional callable(mps, list_of_bonds) -> list of ell
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

    def _flush(self):
        if self._pending:
            gates = self._pending
            self._pending = []
            self._pending_sites = set()
            self._apply_batch(gates)

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
        return self._statistics

    # ------------------------------------------------------------ stats API
    def _log_operation(self, **kwargs):
        self._statistics.record(step=self._operation_counter, **kwargs)
        self._operation_counter += 1

    def stats_summary(self) -> Dict[str, float]:
        return self.statistics.summary()

    def global_error_bound(self) -> float:
        return self.statistics.global_error_bound()

    def reset_stats(self):
        self.statistics.reset()
        self._operation_counter = 0

    # ------------------------------------------------------------ gates
    @torch.no_grad()
    def apply_single_qubit_gate(self, q: int, U2: torch.Tensor):
        """adaptive_mps.py:159-180; applies U^T like the reference."""
        assert 0 <= q < self.num_qubits, f"Qubit index {q} out of range"
        assert U2.shape == (2, 2), "U2 must be 2x2"
        if q in self._pending_sites:
            self._flush()
        T = self._tensors[q]
        if not T.is_contiguous():
            T = T.contiguous()
        ops.single_qubit_gate_(T, U2)
        self._tensors[q] = T
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
        if i in self._pending_sites or (i + 1) in self._pending_sites:
            self._flush()
        self._pending.append((i, U))
        self._pending_sites.update((i, i + 1))
        self.is_canonical = False

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
        t0 = time.perf_counter()
        dt = self.dtype_policy.default
        ells = None
        if self.rank_predictor is not None:
            ells = self.rank_predictor(self, [i for i, _ in gates])
        res = self._run_pipeline(gates, dt, ells)
        # rank fallback: predicted sketch too small -> rerun those gates at full size
        redo = [g for g, r in enumerate(res) if r["status"] == _lib.AGB_ERR_RANK]
        if redo:
            full = self._run_pipeline([gates[g] for g in redo], dt, None)
            for g, r in zip(redo, full):
                r["driver"] = "gb300_gram_heevd_full"
                res[g] = r
        # precision promotion (adaptive_mps.py:268-274)
        thr = self.dtype_policy.promote_if_cond_gt
        for g, r in enumerate(res):
            if math.isfinite(r["condS"]) and r["condS"] > thr and dt != _C128:
                r2 = self._run_pipeline([gates[g]], _C128, None)[0]
                r2["driver"] = "gb300_gram_heevd_c128"
                res[g] = r2
        elapsed = (time.perf_counter() - t0) * 1000.0 / max(1, len(gates))
        self.batch_log.append((len(gates), elapsed * len(gates) / 1000.0))
        for (i, _), r in zip(gates, res):
            self._tensors[i] = r["A"]
            self._tensors[i + 1] = r["B"]
            self._bond_dims[i] = r["k"]
            if not check_entropy_sanity(r["entropy"], r["chiL"], r["chiR"]):
                print(f"Warning: Entropy {r['entropy']:.3f} exceeds physical bound at bond {i}")
            self._log_operation(bond=i, k_star=r["k"], chi_before=r["chiM"], chi_after=r["k"],
                                eps_local=r["eps_local"], entropy=r["entropy"], svd_driver=r["driver"],
                                dtype=str(r["dtype"]), ms_elapsed=elapsed, condS=r["condS"])

    def _run_pipeline(self, gates, dt, ells):
        """One batched launch sequence: plan -> run -> read ranks -> finalize.
        Descriptor rows are built and read with NumPy; the two small copies per
        batch (descriptors up, results down) are the only host synchronisation."""
        lib = _lib.load()
        code = dtype_code(dt)
        G = len(gates)
        desc = np.zeros((G, _lib.D_NFIELDS), dtype=np.int64)
        keep = []
        if all(U.device == self.device for _, U in gates):
            Us = torch.stack([U.to(dtype=dt) for _, U in gates]).contiguous()
        else:
            Us = torch.stack([U.to(dtype=dt, device="cpu") for _, U in gates]).contiguous()
            Us = Us.to(self.device, non_blocking=True)
        keep.append(Us)
        u_base, u_stride = Us.data_ptr(), 16 * Us.element_size()
        maxL = maxM = maxR = 1
        meta = []
        eps_bits = _dbits(self.eps_bond)
        seed0 = (self._seed * 1000003 + self._operation_counter) & 0x3FFFFFFFFFFFFFFF
        for g, (i, _) in enumerate(gates):
            A = self._tensors[i]
            B = self._tensors[i + 1]
            if A.dtype != dt or not A.is_contiguous():
                A = A.to(dt).contiguous()
            if B.dtype != dt or not B.is_contiguous():
                B = B.to(dt).contiguous()
            keep += [A, B]
            chiL, chiM, chiR = A.shape[0], A.shape[2], B.shape[2]
            maxL, maxM, maxR = max(maxL, chiL), max(maxM, chiM), max(maxR, chiR)
            row = desc[g]
            row[_lib.D_A] = A.data_ptr()
            row[_lib.D_B] = B.data_ptr()
            row[_lib.D_U] = u_base + g * u_stride
            row[_lib.D_CHIL] = chiL
            row[_lib.D_CHIM] = chiM
            row[_lib.D_CHIR] = chiR
            row[_lib.D_CAP] = self.chi_max_per_bond[i]
            row[_lib.D_EPS] = eps_bits
            row[_lib.D_ELL] = int(ells[g]) if ells is not None else 0
            row[_lib.D_SEED] = seed0 + g
            meta.append((i, chiL, chiM, chiR))
        wsz = _lib.SZ(0)
        check(lib.agb_two_site_plan(code, G, desc.ctypes.data_as(ctypes.c_void_p), ctypes.byref(wsz)),
              "two_site_plan")
        maxell = int(desc[:, _lib.D_ELL].max())
        ws = ops.workspace(wsz.value, self.device, "two_site")
        desc_dev = torch.from_numpy(desc).to(self.device)
        stream = stream_ptr(self.device)
        check(lib.agb_two_site_run(code, G, ptr(desc_dev), ptr(desc_dev), maxL, maxM, maxR, maxell,
                                   ptr(ws), wsz.value, stream), "two_site_run")
        out = desc_dev.cpu().numpy()
        res = []
        maxk = 1
        for g, (i, chiL, chiM, chiR) in enumerate(meta):
            row = out[g]
            st = int(row[_lib.D_STATUS])
            k = int(row[_lib.D_K])
            r = {"status": st, "k": k, "eps_local": _bitsd(int(row[_lib.D_EPSLOC])),
                 "entropy": _bitsd(int(row[_lib.D_ENTROPY])), "condS": _bitsd(int(row[_lib.D_CONDS])),
                 "chiL": chiL, "chiM": chiM, "chiR": chiR, "driver": "gb300_gram_heevd", "dtype": dt,
                 "mode": int(row[_lib.D_MODE]), "ell": int(row[_lib.D_ELL])}
            if st not in (_lib.AGB_OK, _lib.AGB_ERR_RANK):
                check(st, f"two-site update on bond {i}")
            ok = self._budget_ok_fn(chiL, chiM, chiR, dt)
            if ok is not None and st == _lib.AGB_OK:
                kk = k
                while kk > 1 and not ok(kk):
                    kk -= 1
                if kk != k:
                    r["k"] = k = kk
                    row[_lib.D_K] = kk
            if st == _lib.AGB_OK:
                A_new = torch.empty(chiL, 2, k, dtype=dt, device=self.device)
                B_new = torch.empty(k, 2, chiR, dtype=dt, device=self.device)
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
