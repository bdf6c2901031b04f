"""Device-resident MPS state: gates advance without host synchronisation.

In the default mode every batch of two-site gates ends with a device->host read
of the kept ranks, because the host allocates the new site tensors at their
exact shapes.  In resident mode each site has one capacity buffer
``[capL * 2 * capR]`` and the bond dimensions live in an int32 array on the
device: the two-site kernels read the current shapes from it, write the new
site tensors in place and store the new rank back (``AGB_D_DIMS`` /
``AGB_D_BOND`` in the C ABI).  The host only enqueues launches, so a whole
circuit (or a circuit layer of many instances) can be captured into one CUDA
graph and replayed.

What a caller can observe:
* ``tensors``, ``bond_dims``, ``statistics`` and every non-gate method leave
  resident mode first (one synchronisation; the tensors become views of the
  capacity buffers, the per-gate statistics are read back then).
* Kernel-side failures are reported at that point instead of at the gate.
* A gate whose eigenvalue-guided eigenvector count falls short is re-run with
  every vector on the device (the two-site repair pass), as the host path's
  fallback would.
* Precision promotion (adaptive_mps.py:268-274, sigma_0 / sigma_{k-1} above
  the policy's threshold) needs a host decision per gate, so an instance
  enters resident mode only when its threshold is out of the float32 rank
  rule's reach (``AdaptiveMPS.promotion_reachable``: below sqrt(2 chi_cap
  2^26), 1.9e5 at chi_cap 256; the default 1e6 is above it) and otherwise runs
  host-synchronised, where promotion happens.  A gate that nevertheless reports
  a ratio above the threshold (only a float32 rounding tie in the rank rule's
  total allows it) is counted in ``AdaptiveMPS.unpromoted``.
"""
import ctypes
import math
import time
from typing import List

import numpy as np
import torch

from . import _lib, ops
from ._lib import check, dtype_code, ptr, stream_ptr


class _PinnedRing:
    """Host->device uploads without host synchronisation: a ring of pinned
    staging slots allocated once.  A slot is rewritten only after the copy that
    last read it has completed (its event), so a fresh pinned allocation --
    which synchronises the whole device -- never happens on the gate path."""

    def __init__(self, device, nslots=128, slot_bytes=1 << 20):
        self.device = device
        self.slot_bytes = slot_bytes
        self.slots = [torch.empty(slot_bytes, dtype=torch.uint8, pin_memory=True) for _ in range(nslots)]
        self.views = [t.numpy() for t in self.slots]
        self.events = [None] * nslots
        self.next = 0

    def upload(self, arr: np.ndarray) -> torch.Tensor:
        raw = np.ascontiguousarray(arr).view(np.uint8).reshape(-1)
        nb = raw.size
        if nb > self.slot_bytes:  # rare: larger than a slot
            return torch.from_numpy(np.ascontiguousarray(arr)).to(self.device)
        i = self.next
        self.next = (i + 1) % len(self.slots)
        if self.events[i] is not None:
            self.events[i].synchronize()
        self.views[i][:nb] = raw
        dev = torch.empty(nb, dtype=torch.uint8, device=self.device)
        dev.copy_(self.slots[i][:nb], non_blocking=True)
        ev = torch.cuda.Event()
        ev.record(torch.cuda.current_stream(self.device))
        self.events[i] = ev
        return dev


_rings = {}


def upload(arr: np.ndarray, device, dtype=None, shape=None) -> torch.Tensor:
    """Copy a host array to the device asynchronously (stream-ordered)."""
    key = torch.device(device).index or 0
    ring = _rings.get(key)
    if ring is None:
        ring = _rings[key] = _PinnedRing(torch.device(device))
    dev = ring.upload(arr)
    tdt = dtype if dtype is not None else {np.dtype(np.int64): torch.int64, np.dtype(np.complex64): torch.complex64,
                                           np.dtype(np.complex128): torch.complex128}[np.dtype(arr.dtype)]
    out = dev.view(tdt)
    return out.reshape(shape if shape is not None else arr.shape)


def _dbits(x: float) -> int:
    return int(np.array([x], dtype=np.float64).view(np.int64)[0])


def _bitsd(v: int) -> float:
    return float(np.array([v], dtype=np.int64).view(np.float64)[0])


class ResidentState:
    """Capacity buffers, device bond dimensions and pending statistics of one MPS."""

    def __init__(self, mps):
        n = mps.num_qubits
        dev = mps.device
        ts = mps._tensors
        dt = ts[0].dtype
        if any(t.dtype != dt for t in ts):
            ts = [t.to(dt) for t in ts]
        self.dtype = dt
        cur = [t.shape[2] for t in ts[:-1]]
        capb = []
        for b in range(n - 1):
            grow = 1 << min(b + 1, n - 1 - b, 30)
            capb.append(max(cur[b], min(mps.chi_max_per_bond[b], grow)))
        self.capb = capb
        self.capL = [1] + capb
        self.capR = capb + [1]
        self.bufs: List[torch.Tensor] = []
        for s in range(n):
            buf = torch.empty(self.capL[s] * 2 * self.capR[s], dtype=dt, device=dev)
            T = ts[s].contiguous()
            buf[:T.numel()].copy_(T.reshape(-1))
            self.bufs.append(buf)
        self.dims = torch.tensor([1] + cur + [1], dtype=torch.int32, device=dev)
        self.batches = []  # (desc_dev, rows of this instance, enqueue time)
        self.keep = []     # host-side references kept until the next synchronisation

    def dims_ptr(self, site):
        return self.dims.data_ptr() + 4 * site


def enter(mps):
    mps._res = ResidentState(mps)


def leave(mps):
    """Synchronise, turn the capacity buffers into the tensor list, log statistics."""
    res = mps._res
    mps._res = None
    dims = res.dims.cpu().tolist()  # synchronises the stream
    n = mps.num_qubits
    mps._tensors = [res.bufs[s][:dims[s] * 2 * dims[s + 1]].view(dims[s], 2, dims[s + 1]) for s in range(n)]
    mps._bond_dims = dims[1:-1]
    err = None
    ngates = sum(len(rows) for _, rows, _ in res.batches)
    elapsed = (time.perf_counter() - res.batches[0][2]) * 1000.0 / max(ngates, 1) if res.batches else 0.0
    for desc_dev, rows, _ in res.batches:
        out = desc_dev.cpu().numpy()
        for g, bond in rows:
            row = out[g]
            st = int(row[_lib.D_STATUS])
            k = int(row[_lib.D_K])
            cs = _bitsd(int(row[_lib.D_CONDS]))
            drv = "gb300_gram_heevd_resident"
            if math.isfinite(cs) and cs > mps.dtype_policy.promote_if_cond_gt and res.dtype != torch.complex128:
                drv = "gb300_gram_heevd_unpromoted"
                mps.unpromoted += 1
            if st != _lib.AGB_OK and err is None:
                err = (st, bond)
            mps._last_entropy[bond] = _bitsd(int(row[_lib.D_ENTROPY]))
            mps._log_operation(bond=bond, k_star=k, chi_before=int(row[_lib.D_CHIM]), chi_after=k,
                               eps_local=_bitsd(int(row[_lib.D_EPSLOC])),
                               entropy=_bitsd(int(row[_lib.D_ENTROPY])), svd_driver=drv, dtype=str(res.dtype),
                               ms_elapsed=elapsed, condS=cs)
    if err is not None:
        check(err[0], f"two-site update on bond {err[1]} (device-resident batch)")


def single_qubit_entries(entries):
    """Queued single-qubit gates of resident instances, one launch."""
    lib = _lib.load()
    device = entries[0][0].device
    groups = {}
    for m, q, U in entries:
        groups.setdefault((id(m), q), (m, q, []))[2].append(U)
    dt = entries[0][0]._res.dtype
    ng = len(groups)
    nu = len(entries)
    desc = np.zeros(ng * 5 + nu, dtype=np.int64)
    host_U, host_slot, keep = [], [], []
    first, max_elems = 0, 1
    for g, (m, q, Us) in enumerate(groups.values()):
        res = m._res
        desc[5 * g:5 * g + 5] = (res.bufs[q].data_ptr(), -1, res.dims_ptr(q), first, len(Us))
        max_elems = max(max_elems, res.capL[q] * res.capR[q])
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
        Ud = upload(torch.stack(host_U).numpy(), device)
        keep.append(Ud)
        es = 4 * Ud.element_size()
        for j, slot in enumerate(host_slot):
            desc[slot] = Ud.data_ptr() + j * es
    desc_dev = upload(desc, device)
    check(lib.agb_single_qubit_batch(dtype_code(dt), ng, ptr(desc_dev), max_elems, stream_ptr(device)),
          "single_qubit_batch")
    for m, _, _ in groups.values():
        m._res.keep.append((desc_dev, keep))


def build_two_site(entries):
    """Descriptor rows (host, int64) for resident two-site gates; plans them."""
    lib = _lib.load()
    m0 = entries[0][0]
    dt = m0._res.dtype
    code = dtype_code(dt)
    G = len(entries)
    desc = np.zeros((G, _lib.D_NFIELDS), dtype=np.int64)
    device = m0.device
    host_U, host_rows, keep = [], [], []
    seeds = {}
    for g, (m, i, U) in enumerate(entries):
        res = m._res
        if res.dtype != dt:
            raise ValueError("resident batch entries must share the dtype")
        row = desc[g]
        row[_lib.D_A] = row[_lib.D_ANEW] = res.bufs[i].data_ptr()
        row[_lib.D_B] = row[_lib.D_BNEW] = res.bufs[i + 1].data_ptr()
        if U.device == device:
            if U.dtype != dt or not U.is_contiguous():
                U = U.to(dtype=dt).contiguous()  # a device-side copy, no synchronisation
            keep.append(U)
            row[_lib.D_U] = U.data_ptr()
        else:
            host_U.append(U.detach().to("cpu", dt).reshape(4, 4))
            host_rows.append(g)
        row[_lib.D_CHIL] = res.capL[i]
        row[_lib.D_CHIM] = res.capb[i]
        row[_lib.D_CHIR] = res.capR[i + 1]
        row[_lib.D_CAP] = m.chi_max_per_bond[i]
        row[_lib.D_EPS] = _dbits(m.eps_bond)
        j = seeds.get(id(m), 0)
        seeds[id(m)] = j + 1
        row[_lib.D_SEED] = ((m._seed * 1000003 + m._operation_counter + len(res.batches)) & 0x3FFFFFFFFFFFFFFF) + j
        row[_lib.D_DIMS] = res.dims.data_ptr()
        row[_lib.D_BOND] = i
        row[_lib.D_NVEC] = 0  # guided count; a short cut is repaired on the device
    wsz = _lib.SZ(0)
    check(lib.agb_two_site_plan(code, G, desc.ctypes.data_as(ctypes.c_void_p), ctypes.byref(wsz)), "two_site_plan")
    Ud = None
    if host_U:
        Ud = upload(torch.stack(host_U).numpy(), device)
        keep.append(Ud)
        for j, g in enumerate(host_rows):
            desc[g, _lib.D_U] = Ud.data_ptr() + j * 16 * Ud.element_size()
    maxL = int(desc[:, _lib.D_CHIL].max())
    maxM = int(desc[:, _lib.D_CHIM].max())
    maxR = int(desc[:, _lib.D_CHIR].max())
    maxell = int(desc[:, _lib.D_ELL].max())
    maxk = int(desc[:, _lib.D_CAP].max())
    return desc, wsz.value, (maxL, maxM, maxR, maxell, maxk), keep


def launch_two_site(code, G, desc_dev, ws, wsz, dims, stream):
    lib = _lib.load()
    maxL, maxM, maxR, maxell, maxk = dims
    check(lib.agb_two_site_run(code, G, ptr(desc_dev), ptr(desc_dev), maxL, maxM, maxR, maxell, ptr(ws), wsz,
                               stream, _lib.AGB_RUN_REPAIR), "two_site_run")
    check(lib.agb_two_site_finalize(code, G, ptr(desc_dev), maxL, maxR, min(maxk, 2 * max(maxL, maxR)), ptr(ws),
                                    stream), "two_site_finalize")


def two_site_entries(entries):
    """Resident two-site gates of any number of instances, no host synchronisation."""
    m0 = entries[0][0]
    device = m0.device
    desc, wsz, dims, keep = build_two_site(entries)
    ws = ops.workspace(wsz, device, "two_site_resident")
    desc_dev = upload(desc, device)
    launch_two_site(dtype_code(m0._res.dtype), len(entries), desc_dev, ws, wsz, dims, stream_ptr(device))
    t = time.perf_counter()
    rows = {}
    for g, (m, i, _) in enumerate(entries):
        rows.setdefault(id(m), (m, []))[1].append((g, i))
    for m, rs in rows.values():
        m._res.batches.append((desc_dev, rs, t))
        m._res.keep.append(keep)
