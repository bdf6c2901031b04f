"""Diagnostics, API-compatible with src/atlas_q/diagnostics.py (host-side logs)."""
import math
from typing import Dict, List

import numpy as np
import torch


def bond_entropy_from_S(S: torch.Tensor) -> float:
    """diagnostics.py:17-35 (bits)."""
    s = S.detach().double().cpu() if isinstance(S, torch.Tensor) else torch.as_tensor(S, dtype=torch.float64)
    if s.numel() == 0:
        return 0.0
    p = s * s / (s * s).sum()
    return float(-(p * torch.log2(torch.clamp(p, min=1e-30))).sum())


def effective_rank(S: torch.Tensor, threshold: float = 0.99) -> int:
    """diagnostics.py:38-55."""
    s = S.detach().cpu() if isinstance(S, torch.Tensor) else torch.as_tensor(S)
    if s.numel() == 0:
        return 0
    E = (s * s).cumsum(0)
    k = int(torch.searchsorted(E, threshold * E[-1]).item()) + 1
    return min(k, s.numel())


def spectral_gap(S: torch.Tensor, k: int) -> float:
    """diagnostics.py:58-75."""
    if k >= len(S) or k < 1 or S[k] == 0:
        return float("inf")
    return float((S[k - 1] / S[k]).item())


GPU_DRIVERS = ("gb300_gram_heevd", "gb300_gram_heevd_full", "gb300_gram_heevd_c128", "gb300_gram_heevd_resident",
               "gb300_gram_heevd_unpromoted")


class MPSStatistics:
    """diagnostics.py:78-152: per-operation logs with the same 11 columns."""

    def __init__(self):
        self.logs: Dict[str, List] = {k: [] for k in (
            "step", "bond", "k_star", "chi_before", "chi_after", "eps_local", "entropy",
            "svd_driver", "dtype", "ms_elapsed", "condS")}

    def record(self, **kwargs):
        for key, value in kwargs.items():
            if key in self.logs:
                self.logs[key].append(value)

    def summary(self) -> Dict[str, float]:
        def safe_agg(key, fn):
            if not self.logs[key]:
                return 0.0
            try:
                return float(fn(np.array(self.logs[key])))
            except Exception:
                return 0.0

        return {
            "total_operations": len(self.logs["step"]),
            "max_chi": safe_agg("chi_after", np.max),
            "mean_chi": safe_agg("chi_after", np.mean),
            "sum_eps2": safe_agg("eps_local", lambda x: (x ** 2).sum()),
            "max_eps": safe_agg("eps_local", np.max),
            "mean_entropy": safe_agg("entropy", np.mean),
            "p95_entropy": safe_agg("entropy", lambda x: np.percentile(x, 95)),
            "total_time_ms": safe_agg("ms_elapsed", np.sum),
            # GPU drivers of this build count as the CUDA SVD path
            "cuda_svd_pct": self._driver_percentage(("torch_cuda",) + GPU_DRIVERS),
            "cpu_fallback_pct": self._driver_percentage(("torch_cpu",)),
        }

    def _driver_percentage(self, names) -> float:
        if isinstance(names, str):
            names = (names,)
        d = self.logs["svd_driver"]
        if not d:
            return 0.0
        return 100.0 * sum(1 for x in d if x in names) / len(d)

    def global_error_bound(self) -> float:
        if not self.logs["eps_local"]:
            return 0.0
        return math.sqrt(sum(e ** 2 for e in self.logs["eps_local"]))

    def reset(self):
        for key in self.logs:
            self.logs[key].clear()
