"""Many MPS instances advanced together on one GPU.

``MPSBatch`` holds AdaptiveMPS instances of any qubit counts, bond caps and
cutoffs and runs their circuits in lockstep: each round takes, from every
instance, the longest prefix of its remaining operations that can be queued
without a flush (two-site gates on disjoint bonds, single-qubit gates on sites
with no queued gate), then applies all queued two-site gates of all instances
as ONE batched launch sequence.  For a hardware-efficient-ansatz layer (a CZ
ladder) that is one gate per instance per round, so a round of 256 instances
is one launch sequence over 256 two-site problems of uneven shapes.

Each instance's result is the one it gets when run alone: the two-site
problems of a batch are independent, and the rank rule, rank fallback and
precision promotion are applied per gate (adaptive_mps.py:182-308).
"""
from typing import Iterable, List, Sequence

from .adaptive_mps import AdaptiveMPS, apply_gate_entries, apply_single_qubit_entries


class MPSBatch:
    def __init__(self, instances: Sequence[AdaptiveMPS]):
        self.instances: List[AdaptiveMPS] = list(instances)
        self.rounds = 0

    def flush(self):
        """Apply every instance's queued single-qubit gates in one launch, then
        every instance's queued two-site gates in one batch."""
        ones = []
        for m in self.instances:
            if m._pending_1q:
                ones += [(m, q, U) for q, U in m._pending_1q]
                m._pending_1q = []
        if ones:
            apply_single_qubit_entries(ones)
        entries = []
        for m in self.instances:
            if m._pending:
                entries += [(m, i, U) for i, U in m._pending]
                m._pending = []
                m._pending_sites = set()
        if entries:
            apply_gate_entries(entries)
            self.rounds += 1

    @staticmethod
    def _fits(m: AdaptiveMPS, op) -> bool:
        kind, q = op[0], op[1]
        if kind == "2q":
            return q not in m._pending_sites and (q + 1) not in m._pending_sites
        return q not in m._pending_sites

    @staticmethod
    def _apply(m: AdaptiveMPS, op):
        kind, q, U = op
        if kind == "2q":
            m.apply_two_site_gate(q, U)
        else:
            m.apply_single_qubit_gate(q, U)

    def run(self, circuits: Sequence[Iterable]):
        """Run ``circuits[b]`` (a list of ("1q"|"2q", site, U) ops) on instance b."""
        if len(circuits) != len(self.instances):
            raise ValueError("one circuit per instance")
        progs = [list(c) for c in circuits]
        cur = [0] * len(progs)
        while True:
            moved = False
            for b, m in enumerate(self.instances):
                ops_b = progs[b]
                while cur[b] < len(ops_b) and self._fits(m, ops_b[cur[b]]):
                    self._apply(m, ops_b[cur[b]])
                    cur[b] += 1
                    moved = True
            if not any(m._pending or m._pending_1q for m in self.instances):
                if all(c == len(p) for c, p in zip(cur, progs)):
                    break
                if not moved:
                    raise RuntimeError("batched schedule made no progress")
            self.flush()
        return self
