"""atlasq_gb300: GB300-native (sm_103a) MPS circuit-simulation hot path with the
ATLAS-Q AdaptiveMPS API (followthesapper/ATLAS-Q 0.7.0).

Public names mirror the reference: AdaptiveMPS, DTypePolicy, robust_svd,
robust_qr, choose_rank_from_sigma, MPO, MPOBuilder, expectation_value,
correlation_function, MPSStatistics, get_adaptive_mps(), apply_mpo_to_mps,
apply_pauli_exp_to_mps and the TDVP environment steps.  Additions for the
GB300 path: MPSBatch (many instances per launch sequence),
rank_predictor.RankPredictor (learned kept-rank sizing) and svd_log (the
SVD-event log).  A Qiskit circuit runs through adapters.run_circuit."""

__version__ = "0.1.0"

from .adaptive_mps import AdaptiveMPS, DTypePolicy, apply_gate_entries  # noqa: E402
from .batched import CapturedCircuit, MPSBatch  # noqa: E402
from . import autotune  # noqa: E402
from .diagnostics import MPSStatistics, bond_entropy_from_S, effective_rank, spectral_gap  # noqa: E402
from .linalg_robust import condition_number, robust_qr, robust_svd  # noqa: E402
from .mpo_ops import (MPO, MPOBuilder, apply_mpo_to_mps, apply_pauli_exp_to_mps,  # noqa: E402
                      correlation_function, expectation_value, local_expectations, pauli_exp_mpo,
                      pauli_string_to_mpo, tdvp_apply_local_H, tdvp_left_environment, tdvp_right_environment)
from . import svd_log  # noqa: E402
from .truncation import check_entropy_sanity, choose_rank_from_sigma, compute_global_error_bound  # noqa: E402


def get_adaptive_mps():
    """Lazy getter with the same keys as atlas_q.get_adaptive_mps() (src/atlas_q/__init__.py:47-66)."""
    return {
        "AdaptiveMPS": AdaptiveMPS,
        "DTypePolicy": DTypePolicy,
        "robust_svd": robust_svd,
        "robust_qr": robust_qr,
        "condition_number": condition_number,
        "choose_rank_from_sigma": choose_rank_from_sigma,
        "compute_global_error_bound": compute_global_error_bound,
        "check_entropy_sanity": check_entropy_sanity,
        "MPSStatistics": MPSStatistics,
        "bond_entropy_from_S": bond_entropy_from_S,
        "effective_rank": effective_rank,
        "spectral_gap": spectral_gap,
    }
