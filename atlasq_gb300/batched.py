"""Many MPS instances advanced together on one GPU.

``MPSBatch`` holds AdaptiveMPS instances of any qubit counts, bond caps and
cutoffs and runs their circuits in lockstep: each round takes, from every
instance, the longest prefix of its remaining operations that can be queued
without a flush (two-site gates on disjoint bonds, single-qubit gates on sites
with no queued two-site gate), then applies all queued single-qubit gates of
all instances in one launch and all queued two-site gates as ONE batched launch
sequence.  For a hardware-efficient-ansatz layer (a CZ ladder) that is one
gate per instance per round, so a round of 256 instances is one launch sequence
over 256 two-site problems of uneven shapes.

Each instance's result is the one it gets when run alone: the two-site
problems of a batch are independent, and the rank rule, rank fallback and
precision promotion are applied per gate (adaptive_mps.py:182-308).

With device-resident instances (``AdaptiveMPS(..., device_resident=True)``)
nothing synchronises between rounds, and ``capture`` records a whole circuit
(every round of every instance, from a fixed start state) as one CUDA graph:
``CapturedCircuit.replay()`` then re-runs it with one launch, and the gate
matrices can be rewritten in place between replays (same circuit structure,
new angles).
"""
from typing import Iterable, List, Sequence

import numpy as np
import torch

from . import _lib, ops, resident
from ._lib import dtype_code, ptr, stream_ptr
from .adaptive_mps import AdaptiveMPS, apply_gate_entries, apply_single_qubit_entries


def _schedule(instances, circuits):
    """Lockstep rounds [(ones, twos)] without executing anything.  ones: list of
    (instance, site, U) in order; twos: list of (instance, bond, U)."""
    progs = [list(c) for c in circuits]
    cur = [0] * len(progs)
    rounds = []
    while any(c < len(p) for c, p in zip(cur, progs)):
        ones, twos = [], []
        for b, m in enumerate(instances):
            pend = set()
            ops_b = progs[b]
            while cur[b] < len(ops_b):
                kind, q, U = ops_b[cur[b]]
                if kind == "2q":
                    if q in pend or (q + 1) in pend:
                        break
                    assert 0 <= q < m.num_qubits - 1, f"Bond index {q} out of range"
                    if U.shape == (2, 2, 2, 2):
                        U = U.reshape(4, 4)
                    elif U.shape != (4, 4):
                        raise ValueError(f"U4 must be (2,2,2,2) or (4,4), got {U.shape}")
                    twos.append((m, q, U))
                    pend.update((q, q + 1))
                else:
                    if q in pend:
                        break
                    assert 0 <= q < m.num_qubits, f"Qubit index {q} out of range"
                    assert U.shape == (2, 2), "U2 must be 2x2"
                    ones.append((m, q, U))
                cur[b] += 1
        rounds.append((ones, twos))
    return rounds


class MPSBatch:
    def __init__(self, instances: Sequence[AdaptiveMPS]):
        self.instances: List[AdaptiveMPS] = list(instances)
        self.rounds = 0

    def flush(self):
        """Apply every instance's queued single-qubit gates in one launch, then
        every instance's queued two-site gates in one batch."""
        res = [m for m in self.instances if m._res is not None]
        if res and len(res) != len(self.instances):
            raise ValueError("an MPSBatch mixes device-resident and host-visible instances")
        ones = []
        for m in self.instances:
            if m._pending_1q:
                ones += [(m, q, U) for q, U in m._pending_1q]
                m._pending_1q = []
        if ones:
            (resident.single_qubit_entries if res else apply_single_qubit_entries)(ones)
        entries = []
        for m in self.instances:
            if m._pending:
                entries += [(m, i, U) for i, U in m._pending]
                m._pending = []
                m._pending_sites = set()
        if entries:
            (resident.two_site_entries if res else apply_gate_entries)(entries)
            self.rounds += 1

    def run(self, circuits: Sequence[Iterable]):
        """Run ``circuits[b]`` (a list of ("1q"|"2q", site, U) ops) on instance b."""
        if len(circuits) != len(self.instances):
            raise ValueError("one circuit per instance")
        for m in self.instances:
            m._maybe_enter_resident()
        for ones, twos in _schedule(self.instances, circuits):
            for m, q, U in ones:
                m._pending_1q.append((q, U))
            for m, i, U in twos:
                m._pending.append((i, U))
                m._pending_sites.update((i, i + 1))
            self.flush()
        for m in self.instances:
            m.is_canonical = False
        return self

    def synchronize(self):
        """Leave resident mode on every instance (tensors and statistics readable)."""
        for m in self.instances:
            m._flush()

    def capture(self, circuits: Sequence[Iterable]) -> "CapturedCircuit":
        return CapturedCircuit(self, circuits)


class CapturedCircuit:
    """One CUDA graph running ``circuits`` on device-resident instances from
    their current state.  Every launch of every round is recorded; descriptors,
    workspace and the start state stay allocated for the graph's lifetime."""

    def __init__(self, batch: MPSBatch, circuits):
        self.batch = batch
        insts = batch.instances
        for m in insts:
            if not m.device_resident:
                raise ValueError("capture needs device_resident instances")
            m._flush()
            m._maybe_enter_resident()
            if m._res is None:
                raise ValueError("capture needs instances that can run device-resident: no rank predictor, "
                                 "budget or SVD logs, and a promotion threshold the rank rule cannot reach "
                                 "(AdaptiveMPS.promotion_reachable)")
        device = insts[0].device
        self.device = device
        self.rounds = _schedule(insts, circuits)
        self.ngates = sum(len(t) for _, t in self.rounds)
        # start state (restored at the head of every replay)
        self.start = [(m._res, [b.clone() for b in m._res.bufs], m._res.dims.clone()) for m in insts]
        lib = _lib.load()
        dt = insts[0]._res.dtype
        self.code = dtype_code(dt)
        self.keep = []
        self.plan = []
        self._ones_staged = []
        wsmax = 1
        for ones, twos in self.rounds:
            step = {}
            if ones:
                step["ones"] = self._stage_ones(ones, dt)
            if twos:
                # the gate matrices are staged in buffers owned by the graph, so they
                # can be rewritten between replays (update_gates)
                U2 = torch.stack([U.to(device=device, dtype=dt).reshape(4, 4) for _, _, U in twos]).contiguous()
                staged = [(m, i, U2[g]) for g, (m, i, _) in enumerate(twos)]
                desc, wsz, dims, keep = resident.build_two_site(staged)
                self.keep.append(keep)
                step["twos"] = (torch.from_numpy(desc).to(device), wsz, dims, len(twos), staged)
                step["U2"] = U2
                wsmax = max(wsmax, wsz)
            self.plan.append(step)
        # autotune the eigensolver's cluster shape for the launches of this circuit
        # (one tuning per size / batch-class, before anything is captured)
        from .autotune import tune_for_batches
        shapes = set()
        for step in self.plan:
            if "twos" in step:
                _, _, dims, G, _ = step["twos"]
                shapes.add((2 * dims[2], G))
        self.tuned = tune_for_batches(sorted(shapes), dt, device)
        self.ws = torch.empty(wsmax, dtype=torch.uint8, device=device)
        self.stream = torch.cuda.Stream(device)
        self.stream.wait_stream(torch.cuda.current_stream(device))  # staged descriptors and gates
        # one eager pass on the capture stream (first-use attributes, module load), then capture
        self._restore_and_launch()
        self.stream.synchronize()
        self.graph = torch.cuda.CUDAGraph()
        n0 = lib.agb_launch_count()
        with torch.cuda.graph(self.graph, stream=self.stream):
            self._restore_and_launch()
        self.kernels_per_replay = lib.agb_launch_count() - n0  # kernel nodes of the library in the graph
        self.replays = 0

    def _stage_ones(self, ones, dt):
        groups = {}
        for m, q, U in ones:
            groups.setdefault((id(m), q), (m, q, []))[2].append(U)
        ng = len(groups)
        desc = np.zeros(ng * 5 + len(ones), dtype=np.int64)
        Us = torch.stack([U.to(device=self.device, dtype=dt).reshape(2, 2) for _, _, U in
                          [(m, q, U) for m, q, Ul in groups.values() for U in Ul]]).contiguous()
        self.keep.append(Us)
        self._ones_staged.append((Us, [(id(m), q) for m, q, Ul in groups.values() for _ in Ul]))
        first, max_elems, j = 0, 1, 0
        for g, (m, q, Ul) in enumerate(groups.values()):
            res = m._res
            desc[5 * g:5 * g + 5] = (res.bufs[q].data_ptr(), -1, res.dims_ptr(q), first, len(Ul))
            max_elems = max(max_elems, res.capL[q] * res.capR[q])
            for _ in Ul:
                desc[ng * 5 + first] = Us.data_ptr() + j * 4 * Us.element_size()
                first += 1
                j += 1
        return torch.from_numpy(desc).to(self.device), ng, max_elems

    def _restore_and_launch(self):
        lib = _lib.load()
        s = self.stream.cuda_stream
        with torch.cuda.stream(self.stream):
            for res, bufs, dims in self.start:
                for b, b0 in zip(res.bufs, bufs):
                    b.copy_(b0, non_blocking=True)
                res.dims.copy_(dims, non_blocking=True)
            for step in self.plan:
                if "ones" in step:
                    d, ng, me = step["ones"]
                    _lib.check(lib.agb_single_qubit_batch(self.code, ng, ptr(d), me, s), "single_qubit_batch")
                if "twos" in step:
                    d, wsz, dims, G, _ = step["twos"]
                    resident.launch_two_site(self.code, G, d, self.ws, wsz, dims, s)

    def update_gates(self, circuits):
        """Write new gate matrices for the same circuit structure (same ops on the
        same sites in the same order, e.g. new rotation angles) into the buffers
        the graph reads; takes effect from the next replay."""
        rounds = _schedule(self.batch.instances, circuits)
        if len(rounds) != len(self.rounds):
            raise ValueError("circuit structure differs from the captured one")
        dt = self.batch.instances[0]._res.dtype
        oi = 0
        with torch.cuda.stream(self.stream):
            for (ones, twos), (o0, t0), step in zip(rounds, self.rounds, self.plan):
                if [(id(m), q) for m, q, _ in twos] != [(id(m), q) for m, q, _ in t0] or len(ones) != len(o0):
                    raise ValueError("circuit structure differs from the captured one")
                if ones:
                    Us, order = self._ones_staged[oi]
                    oi += 1
                    by = {}
                    for m, q, U in ones:
                        by.setdefault((id(m), q), []).append(U)
                    seq = []
                    for key in order:
                        seq.append(by[key].pop(0))
                    Us.copy_(torch.stack([U.to(device=self.device, dtype=dt).reshape(2, 2) for U in seq]))
                if twos:
                    step["U2"].copy_(torch.stack([U.to(device=self.device, dtype=dt).reshape(4, 4)
                                                  for _, _, U in twos]))
        return self

    def replay(self):
        """Run the captured circuit once (asynchronously, ordered on the capture
        stream; ``finish`` or ``stream.synchronize()`` waits for it)."""
        with torch.cuda.stream(self.stream):
            self.graph.replay()
        self.replays += 1
        return self

    def finish(self):
        """Wait for the last replay; record its statistics on the instances and
        leave resident mode (tensors readable; they are views of the buffers the
        next replay overwrites)."""
        self.stream.synchronize()
        import time as _t
        now = _t.perf_counter()
        rows = {}
        for step in self.plan:
            if "twos" in step:
                d, _, _, _, twos = step["twos"]
                per = {}
                for g, (m, i, _) in enumerate(twos):
                    per.setdefault(id(m), []).append((g, i))
                for k, rs in per.items():
                    rows.setdefault(k, []).append((d, rs, now))
        for m, (res, _, _) in zip(self.batch.instances, self.start):
            m._pending, m._pending_1q, m._pending_sites = [], [], set()
            res.batches = rows.get(id(m), [])
            m._res = res
            resident.leave(m)
        return self.batch
