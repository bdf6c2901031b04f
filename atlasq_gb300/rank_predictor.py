"""Learned kept-rank predictor for the two-site update.

A small MLP (5 -> 64 -> 64 -> 64 -> 1, FP32) predicts, before any SVD work, the
fraction k / min(2 chi_L, 2 chi_R, cap) of singular values the reference rank
rule will keep.  Its prediction sizes the number of eigenpairs each gate
computes (``ell``); if the prediction is too small the pipeline reports
``AGB_ERR_RANK`` and the gate is re-run with the plain full size (the plain
form is both the fallback and the arbiter of the predictor's error).

Features (all O(1) on the host, per gate):
  0  log2(chi_L) / 10
  1  log2(chi_R) / 10
  2  entangling power of the 4x4 gate (Zanardi, Zalka, Faoro 2000), scaled by 9/2 to [0, 1]
  3  mean entropy of the neighbouring bonds at their last update (nats) / 5
  4  previous rank of this bond / min(2 chi_L, 2 chi_R, cap)
Training, inference and the optimiser run on the GPU through the library's own
kernels (agb_mlp_forward / agb_mlp_backward / agb_mlp_adam).

The reference's learned predictor (src/atlas_q/tools_qih/ai_rank_predictor.py:14-89)
consumes singular values after a full SVD; this one replaces it on the hot path
with a pre-SVD estimate, trained on (features, kept rank) pairs logged from
plain runs of this simulator.
"""
import ctypes
import math

import numpy as np
import torch

from . import _lib, ops
from ._lib import check, ptr, stream_ptr

NPARAM = _lib.MLP_NPARAM
_SWAP = np.eye(4)[[0, 2, 1, 3]]


def _op_entanglement(U):
    """Linear operator entanglement E(U) = 1 - sum lambda_i^2 of the operator
    Schmidt decomposition of a batch of 4x4 gates (rows 2p+q, cols 2p'+q')."""
    G = U.shape[0]
    M = U.reshape(G, 2, 2, 2, 2).transpose(0, 1, 3, 2, 4).reshape(G, 4, 4)
    R = M @ np.conj(np.swapaxes(M, -1, -2))
    n = np.real(np.trace(R, axis1=-2, axis2=-1))
    n2 = np.real(np.trace(R @ R, axis1=-2, axis2=-1))
    return 1.0 - n2 / np.maximum(n * n, 1e-300)


def entangling_power(U):
    """e_p(U) = (4/9) [E(U) + E(U S) - E(S)], E(S) = 3/4, for d = 2."""
    U = np.asarray(U, dtype=np.complex128).reshape(-1, 4, 4)
    return (4.0 / 9.0) * (_op_entanglement(U) + _op_entanglement(U @ _SWAP) - 0.75)


def gate_features(mps, gates):
    """Feature rows [G, 5] (float32) and the full size min(2chiL, 2chiR, cap) per gate."""
    G = len(gates)
    X = np.zeros((G, 5), dtype=np.float32)
    full = np.zeros(G, dtype=np.int64)
    Us = np.stack([U.detach().cpu().numpy().reshape(4, 4) for _, U in gates])
    ep = entangling_power(Us)
    ent = mps._last_entropy
    for g, (i, _) in enumerate(gates):
        chiL = mps._tensors[i].shape[0]
        chiM = mps._tensors[i].shape[2]
        chiR = mps._tensors[i + 1].shape[2]
        nb = [ent[b] for b in (i - 1, i + 1) if b in ent]
        full[g] = min(2 * chiL, 2 * chiR, mps.chi_max_per_bond[i])
        X[g] = (math.log2(chiL) / 10.0, math.log2(chiR) / 10.0, ep[g] * 4.5,
                (sum(nb) / len(nb) if nb else 0.0) / 5.0, min(1.0, chiM / full[g]))
    return X, full


class RankPredictor:
    """MLP on the GPU.  Call it as ``mps.rank_predictor = RankPredictor(...)``."""

    def __init__(self, device="cuda", params=None, seed=0, margin=0.1, pad=4):
        self.device = _lib.require_cuda(device)
        _lib.load()
        if params is None:
            from_init = _init_params(seed)
            params = torch.from_numpy(from_init)
        self.params = params.to(device=self.device, dtype=torch.float32).contiguous()
        assert self.params.numel() == NPARAM
        self.margin = margin
        self.pad = pad
        self.calls = 0
        self.predicted_ell = 0
        self.full_ell = 0

    # ---------------------------------------------------------------- inference
    def predict_fraction(self, X):
        lib = _lib.load()
        Xd = torch.as_tensor(np.ascontiguousarray(X, dtype=np.float32)).to(self.device)
        Y = torch.empty(Xd.shape[0], dtype=torch.float32, device=self.device)
        check(lib.agb_mlp_forward(ptr(self.params), ptr(Xd), Xd.shape[0], ptr(Y), stream_ptr(self.device)),
              "mlp_forward")
        return Y

    def __call__(self, mps, gates):
        X, full = gate_features(mps, gates)
        frac = self.predict_fraction(X).cpu().numpy()
        ell = np.minimum(full, np.ceil(frac * (1.0 + self.margin) * full).astype(np.int64) + self.pad)
        ell = np.maximum(ell, 1)
        self.calls += 1
        self.predicted_ell += int(ell.sum())
        self.full_ell += int(full.sum())
        return [int(e) for e in ell]

    # ---------------------------------------------------------------- training
    def loss_and_grad(self, X, T):
        """Mean-squared error and its gradient (device tensors) for one batch."""
        lib = _lib.load()
        Xd = torch.as_tensor(np.ascontiguousarray(X, dtype=np.float32)).to(self.device)
        Td = torch.as_tensor(np.ascontiguousarray(T, dtype=np.float32)).to(self.device)
        grads = torch.empty(NPARAM, dtype=torch.float32, device=self.device)
        loss = torch.empty(1, dtype=torch.float32, device=self.device)
        need = lib.agb_mlp_backward_workspace(Xd.shape[0])
        ws = ops.workspace(need, self.device, "mlp")
        check(lib.agb_mlp_backward(ptr(self.params), ptr(Xd), ptr(Td), Xd.shape[0], ptr(grads), ptr(loss),
                                   ptr(ws), ws.numel(), stream_ptr(self.device)), "mlp_backward")
        return loss / Xd.shape[0], grads

    def train(self, X, T, steps=400, batch=512, lr=3e-3, weight_decay=1e-5, seed=0):
        """AdamW on minibatches; returns the loss history (host floats)."""
        lib = _lib.load()
        rng = np.random.default_rng(seed)
        X = np.asarray(X, dtype=np.float32)
        T = np.asarray(T, dtype=np.float32)
        m = torch.zeros(NPARAM, dtype=torch.float32, device=self.device)
        v = torch.zeros(NPARAM, dtype=torch.float32, device=self.device)
        hist = []
        for step in range(1, steps + 1):
            idx = rng.integers(0, len(T), size=min(batch, len(T)))
            loss, grads = self.loss_and_grad(X[idx], T[idx])
            check(lib.agb_mlp_adam(ptr(self.params), ptr(grads), ptr(m), ptr(v), step, ctypes.c_float(lr),
                                   ctypes.c_float(0.9), ctypes.c_float(0.999), ctypes.c_float(1e-8),
                                   ctypes.c_float(weight_decay), stream_ptr(self.device)), "mlp_adam")
            if step % 20 == 0 or step == 1:
                hist.append(float(loss.item()))
        return hist

    def state_dict(self):
        return {"params": self.params.detach().cpu(), "margin": self.margin, "pad": self.pad}

    @classmethod
    def from_state_dict(cls, d, device="cuda"):
        return cls(device=device, params=d["params"], margin=d.get("margin", 0.1), pad=d.get("pad", 4))


def _init_params(seed):
    """He initialisation in the kernels' flat layout."""
    rng = np.random.default_rng(seed)
    parts = [rng.standard_normal((64, 5)) * math.sqrt(2.0 / 5), np.zeros(64),
             rng.standard_normal((64, 64)) * math.sqrt(2.0 / 64), np.zeros(64),
             rng.standard_normal((64, 64)) * math.sqrt(2.0 / 64), np.zeros(64),
             rng.standard_normal(64) * math.sqrt(1.0 / 64), np.zeros(1)]
    return np.concatenate([p.reshape(-1) for p in parts]).astype(np.float32)


def collect_training_data(circuit_fn, seeds, n, chi, eps, device="cuda"):
    """Run plain (full-size) simulations and log (features, kept-rank fraction)."""
    from .adaptive_mps import AdaptiveMPS
    Xs, Ts = [], []
    for sd in seeds:
        m = AdaptiveMPS(n, bond_dim=1, eps_bond=eps, chi_max_per_bond=chi, device=device)
        m.feature_log = []
        for kind, q, U in circuit_fn(sd):
            if kind == "2q":
                m.apply_two_site_gate(q, U)
            else:
                m.apply_single_qubit_gate(q, U)
        m.flush()
        for feat, k, full in m.feature_log:
            Xs.append(feat)
            Ts.append(k / max(full, 1))
    return np.asarray(Xs, dtype=np.float32), np.asarray(Ts, dtype=np.float32)


# ---------------------------------------------------------------------- training pipeline
# Plain runs log one SVD event per gate (svd_log.py, the reference's record with
# the predictor's features added); training reads the events back, so the
# pipeline is: log_plain_runs -> training_data_from_events -> RankPredictor.train
# -> save_predictor.  The reference trains its predictor from the same event
# stream (scripts/ai_tools/finetune_rank_predictor.py over svd_logger files).

def log_plain_runs(circuit_fn, seeds, n, chi, eps, log_dir, device="cuda"):
    """Run the plain simulator (no predictor) on ``circuit_fn(seed)`` for every
    seed with the SVD-event log on; returns the log file's path.  The number of
    gates per SVD driver tag over all runs is left in ``log_plain_runs.drivers``."""
    from . import svd_log
    from .adaptive_mps import AdaptiveMPS
    logger = svd_log.SVDEventLogger(log_dir)
    log_plain_runs.drivers = {}
    try:
        for sd in seeds:
            m = AdaptiveMPS(n, bond_dim=1, eps_bond=eps, chi_max_per_bond=chi, device=device)
            m.feature_log = []   # features computed per gate -> written into the events
            m.svd_logger = logger
            for kind, q, U in circuit_fn(sd):
                if kind == "2q":
                    m.apply_two_site_gate(q, U)
                else:
                    m.apply_single_qubit_gate(q, U)
            m.flush()
            for d in m.statistics.logs["svd_driver"]:
                log_plain_runs.drivers[d] = log_plain_runs.drivers.get(d, 0) + 1
    finally:
        logger.close()
    return str(logger.path)


def training_data_from_events(events):
    """(features [N, 5] float32, kept-rank fraction [N] float32) from SVD events
    that carry ``features`` and ``full`` (records without them are skipped)."""
    Xs, Ts = [], []
    for rec in events:
        if "features" not in rec or "full" not in rec:
            continue
        Xs.append(rec["features"])
        Ts.append(rec["adaptive_keep"] / max(int(rec["full"]), 1))
    return np.asarray(Xs, dtype=np.float32).reshape(-1, 5), np.asarray(Ts, dtype=np.float32)


def default_predictor_path(name="hea64"):
    """Weights shipped with the package: ``hea64`` trained on plain runs of the
    64-qubit hardware-efficient ansatz (12 layers, chi_max 512, eps 1e-8);
    ``brickwork40`` on plain runs of the 40-qubit Haar brickwork (depth 20,
    chi_max 256, eps 1e-8, seeds disjoint from the benchmark's)."""
    import os
    return os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", f"rank_predictor_{name}.npz")


def save_predictor(pred, path, **meta):
    import json
    np.savez(path, params=pred.params.detach().cpu().numpy(), margin=np.float64(pred.margin),
             pad=np.int64(pred.pad), meta=np.array(json.dumps(meta)))


def load_predictor(path=None, device="cuda"):
    """A RankPredictor with saved weights (``default_predictor_path()`` when path is None)."""
    d = np.load(path or default_predictor_path())
    return RankPredictor(device=device, params=torch.from_numpy(d["params"]), margin=float(d["margin"]),
                         pad=int(d["pad"]))


def _main(argv=None):
    """python -m atlasq_gb300.rank_predictor --runs R --log-dir DIR --out FILE [--circuit hea|brickwork]

    Logs R seeded plain runs of the 64-qubit hardware-efficient ansatz (12
    layers of RY RZ on every qubit then a CZ ladder, chi_max 512, eps 1e-8;
    ``--circuit brickwork``: the 40-qubit Haar brickwork, depth 20, chi_max
    256), trains the MLP on the GPU on the logged (features, kept rank) pairs
    and saves the weights.  Prints one JSON summary line."""
    import argparse
    import json
    import time
    from .circuits import haar_brickwork, hea_circuit
    from . import svd_log
    ap = argparse.ArgumentParser()
    ap.add_argument("--circuit", default="hea", choices=["hea", "brickwork"])
    ap.add_argument("--runs", type=int, default=16)
    ap.add_argument("--first-seed", type=int, default=1000)
    ap.add_argument("--qubits", type=int, default=None, help="64 (hea) / 40 (brickwork)")
    ap.add_argument("--layers", type=int, default=None, help="12 (hea) / depth 20 (brickwork)")
    ap.add_argument("--chi", type=int, default=None, help="512 (hea) / 256 (brickwork)")
    ap.add_argument("--eps", type=float, default=1e-8)
    ap.add_argument("--steps", type=int, default=1500)
    ap.add_argument("--log-dir", required=True)
    ap.add_argument("--out", required=True)
    ap.add_argument("--device", default="cuda")
    a = ap.parse_args(argv)
    hea = a.circuit == "hea"
    a.qubits = a.qubits or (64 if hea else 40)
    a.layers = a.layers or (12 if hea else 20)
    a.chi = a.chi or (512 if hea else 256)
    t0 = time.perf_counter()
    seeds = list(range(a.first_seed, a.first_seed + a.runs))
    circ = ((lambda sd: hea_circuit(a.qubits, a.layers, seed=sd)) if hea else
            (lambda sd: haar_brickwork(a.qubits, a.layers, seed=sd)))
    path = log_plain_runs(circ, seeds, a.qubits, a.chi, a.eps, a.log_dir, device=a.device)
    t_log = time.perf_counter() - t0
    X, T = training_data_from_events(svd_log.read_events(path))
    rng = np.random.default_rng(0)
    perm = rng.permutation(len(T))
    nval = max(1, len(T) // 10)
    val, tr = perm[:nval], perm[nval:]
    pred = RankPredictor(device=a.device, seed=0)
    t1 = time.perf_counter()
    hist = pred.train(X[tr], T[tr], steps=a.steps)
    t_train = time.perf_counter() - t1
    fv = pred.predict_fraction(X[val]).cpu().numpy()
    save_predictor(pred, a.out, circuit=a.circuit, runs=a.runs, first_seed=a.first_seed, qubits=a.qubits,
                   layers=a.layers,
                   chi=a.chi, eps=a.eps, samples=int(len(T)))
    print(json.dumps({"samples": int(len(T)), "drivers": log_plain_runs.drivers, "log": path,
                      "log_seconds": t_log, "train_seconds": t_train,
                      "final_loss": hist[-1], "val_mae_fraction": float(np.mean(np.abs(fv - T[val]))),
                      "val_under_predicted": float(np.mean(fv * (1 + pred.margin) < T[val])),
                      "out": a.out}), flush=True)


if __name__ == "__main__":
    _main()
