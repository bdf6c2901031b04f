"""Truncation policy, API-compatible with src/atlas_q/truncation.py.

``choose_rank_from_sigma`` is host logic over an already-computed spectrum (the
GPU two-site update evaluates the same rule inside its rank kernel); it follows
truncation.py:21-83 with torch-CPU float32 semantics (double-accumulated
cumsum rounded to float32)."""
import math
from typing import Callable, Tuple

import numpy as np
import torch


def choose_rank_from_sigma(S: torch.Tensor, eps_bond: float, chi_cap: int,
                           budget_ok: Callable[[int], bool] = lambda k: True) -> Tuple[int, float, float, float]:
    s = S.detach().cpu().numpy() if isinstance(S, torch.Tensor) else np.asarray(S)
    if s.size == 0:
        return 0, 0.0, 0.0, float("inf")
    if s.dtype == np.float32:
        E = np.cumsum((s * s).astype(np.float32).astype(np.float64)).astype(np.float32)
        total = E[-1]
        if total < 1e-30:
            return 1, 0.0, 0.0, float("inf")
        thresh = np.float32(np.float32(1.0 - eps_bond ** 2) * total)
    else:
        s = s.astype(np.float64)
        E = np.cumsum(s * s)
        total = E[-1]
        if total < 1e-30:
            return 1, 0.0, 0.0, float("inf")
        thresh = (1.0 - eps_bond ** 2) * total
    k_tol = min(int(np.searchsorted(E, thresh, side="left")) + 1, s.size)
    k = min(k_tol, chi_cap)
    while k > 1 and not budget_ok(k):
        k -= 1
    eps_local = float(np.sqrt(max(total - E[k - 1], 0.0)))
    kept = s[:k].astype(np.float64)
    p = kept * kept / np.sum(kept * kept)
    entropy = float(-(p * np.log(np.clip(p, 1e-30, None))).sum())
    condS = float(s[0] / s[k - 1]) if (k > 1 and s[k - 1] > 0) else float("inf")
    return k, eps_local, entropy, condS


def compute_global_error_bound(local_errors: list) -> float:
    """truncation.py:86-101: sqrt(sum eps_local^2)."""
    return math.sqrt(sum(e ** 2 for e in local_errors))


def check_entropy_sanity(entropy: float, chi_left: int, chi_right: int) -> bool:
    """truncation.py:104-122 (log2 bound compared with the natural-log entropy, as in the reference)."""
    return entropy <= math.log2(min(chi_left * 2, 2 * chi_right)) + 1e-6
