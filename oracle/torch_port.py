"""PyTorch-CPU restatement of the reference two-site update, for TIMING ONLY.

Test / benchmark infrastructure: the CPU baseline of ``bench.py`` (its
``cpu_baseline`` leg and ``--impl reference``) times this port on the host
cores.  It issues the same library calls, in the same order, as the
reference's complex64 ``AdaptiveMPS.apply_two_site_gate``
(src/atlas_q/adaptive_mps.py:182-308) on the CPU:

* contraction: ``torch.einsum`` + permute + the 4x4 gate matmul, the
  fused_two_qubit_gate_pytorch formulation (src/triton_kernels/mps_complex.py:343-368);
* SVD: ``torch.linalg.svd(X, full_matrices=False)``, the first try of
  robust_svd (src/atlas_q/linalg_robust.py:37);
* rank rule: float32 ``cumsum`` / ``searchsorted`` with the reference's
  scalar reads (src/atlas_q/truncation.py:52-81);
* condition-number promotion to complex128 (adaptive_mps.py:266-274);
* split U_k S_k | Vh_k (adaptive_mps.py:281-289) and the per-gate log record.

The NumPy restatement (``mps_oracle``) is slower than the reference on the
same cores (``np.einsum`` without BLAS and a slower LAPACK SVD), so it is not
used as the timing baseline.  Parity is checked against ``mps_oracle`` and the
committed reference fixtures, never against this module.
"""
import math
import time

import torch


def _contract(A, B, U):
    li, rj = A.shape[0], B.shape[2]
    psi = torch.einsum("lpr,rqj->lpqj", A, B).permute(1, 2, 0, 3).reshape(4, li * rj)
    return (U @ psi).reshape(2, 2, li, rj).permute(2, 0, 1, 3).reshape(2 * li, 2 * rj)


def _rank(S, eps, cap):
    E = (S * S).cumsum(0)
    total = E[-1]
    if total < 1e-30:
        return 1, 0.0, 0.0, float("inf")
    k = min(int(torch.searchsorted(E, (1.0 - eps ** 2) * total).item()) + 1, S.numel(), cap)
    eps_local = float(torch.sqrt(torch.clamp(total - E[k - 1], min=0.0)).item())
    w = S[:k] * S[:k]
    p = w / w.sum()
    entropy = float(-(p * torch.log(torch.clamp(p, min=1e-30))).sum().item())
    cond = float((S[0] / S[k - 1]).item()) if k > 1 and S[k - 1] > 0 else float("inf")
    return k, eps_local, entropy, cond


class TorchPortMPS:
    """Product state |0...0> (bond dimension 1) with the reference's two-site update."""

    def __init__(self, num_qubits, eps_bond=1e-8, chi_max=256, dtype=torch.complex64, promote_if_cond_gt=1e6):
        self.n = num_qubits
        self.eps = eps_bond
        self.cap = chi_max
        self.dtype = dtype
        self.promote = promote_if_cond_gt
        self.tensors = []
        for _ in range(num_qubits):
            t = torch.zeros(1, 2, 1, dtype=dtype)
            t[0, 0, 0] = 1
            self.tensors.append(t)
        self.log = []

    @torch.no_grad()
    def apply_two_site_gate(self, i, U):
        t0 = time.time()
        A, B = self.tensors[i], self.tensors[i + 1]
        li, chiM, rj = A.shape[0], A.shape[2], B.shape[2]
        X = _contract(A, B, U.to(self.dtype))
        Uu, S, Vh = torch.linalg.svd(X, full_matrices=False)
        k, el, ent, cond = _rank(S, self.eps, self.cap)
        dt = self.dtype
        if math.isfinite(cond) and cond > self.promote:
            Uu, S, Vh = torch.linalg.svd(X.to(torch.complex128), full_matrices=False)
            k, el, ent, cond = _rank(S, self.eps, self.cap)
            dt = torch.complex128
        self.tensors[i] = (Uu[:, :k] * S[:k]).reshape(li, 2, k)
        self.tensors[i + 1] = Vh[:k].reshape(k, 2, rj)
        self.log.append((i, k, chiM, el, ent, str(dt), (time.time() - t0) * 1e3, cond))
        return k
