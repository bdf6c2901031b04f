"""robust_svd / robust_qr with the reference signatures (src/atlas_q/linalg_robust.py),
computed by this package's CUDA kernels.

robust_svd(X): Gram G = X^H X (GEMM), Hermitian eigensolver (heevd), then
U S = X V with S = column norms (Rayleigh quotients).  There is no jitter or CPU
cascade: a failure raises.  The driver tag is "gb300_gram_heevd"."""
from typing import Tuple

import torch

from . import ops


def robust_svd(X: torch.Tensor) -> Tuple[torch.Tensor, torch.Tensor, torch.Tensor, str]:
    m, n = X.shape
    X = X.contiguous()
    G = ops.cgemm(X, X, opA="C", opB="N")
    r = min(m, n)
    _, V = ops.heevd(G, ell=r)
    AV = ops.cgemm(X, V)
    S = torch.linalg.vector_norm(AV, dim=0)
    order = torch.argsort(S, descending=True)
    S = S[order]
    AV = AV[:, order]
    V = V[:, order]
    U = AV / torch.where(S > 0, S, torch.ones_like(S)).to(AV.dtype)
    return U, S, V.conj().transpose(0, 1).contiguous(), "gb300_gram_heevd"


def robust_qr(X: torch.Tensor) -> Tuple[torch.Tensor, torch.Tensor, str]:
    Q, R = ops.qr(X.contiguous())
    return Q, R, "gb300_householder"


def condition_number(S: torch.Tensor) -> float:
    """linalg_robust.py:79-91."""
    if len(S) == 0 or S[-1] == 0:
        return float("inf")
    return float((S[0] / S[-1]).item())
