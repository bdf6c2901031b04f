"""Batched sequential-conditional sampling on the GPU.

Restates src/atlas_q/mps_pytorch.py:247-355 on a right-canonical copy of the
state (the left-to-right conditional sampler is exact only for a right-canonical
MPS; the reference skips canonicalisation above 10 qubits and canonicalises to
the LEFT below, mps_pytorch.py:166-171).  Randomness is Philox4x32-10 with
counter (shot, site) and key = seed, so results are reproducible and can be
checked decision by decision against the CPU oracle."""
import ctypes

import torch

from . import _lib, ops
from ._lib import check, dtype_code, ptr, stream_ptr


def right_canonical_copy(mps):
    ts = [t.to(mps.dtype).contiguous().clone() for t in mps.tensors]
    saved = list(mps._bond_dims)
    mps._right_sweep(ts)
    mps._bond_dims = saved
    return ts


@torch.no_grad()
def sample_tensors(tensors, num_shots, seed, chunk=16384, return_pz=False):
    """Sample `num_shots` bitstrings (int64, qubit 0 = MSB) from right-canonical tensors."""
    lib = _lib.load()
    dev = tensors[0].device
    dt = tensors[0].dtype
    code = dtype_code(dt)
    n = len(tensors)
    bits = torch.zeros(num_shots, dtype=torch.int64, device=dev)
    pz = torch.empty(num_shots, n, dtype=torch.float64, device=dev) if return_pz else None
    stream = stream_ptr(dev)
    pzcol = torch.empty(min(chunk, max(num_shots, 1)), dtype=torch.float64, device=dev) if return_pz else None
    for c0 in range(0, num_shots, chunk):
        ns = min(chunk, num_shots - c0)
        L = torch.ones(ns, 1, dtype=dt, device=dev)
        for i, T in enumerate(tensors):
            T = T.contiguous()
            l, _, r = T.shape
            Tm = T.reshape(l, 2 * r)
            use_tc = dt == torch.complex64 and ns >= 64 and 2 * r >= 64 and l >= 32
            temp = ops.cgemm_tc(L, Tm, sync=False) if use_tc else ops.cgemm(L, Tm)
            Lnew = torch.empty(ns, r, dtype=dt, device=dev) if i < n - 1 else None
            check(lib.agb_sample_site(code, ptr(temp), ns, r, i, ctypes.c_uint64(seed & 0xFFFFFFFFFFFFFFFF),
                                      ctypes.c_uint64(c0), ctypes.c_void_p(bits.data_ptr() + 8 * c0),
                                      ptr(Lnew) if Lnew is not None else None,
                                      ptr(pzcol) if return_pz else None, stream), "sample_site")
            if return_pz:
                pz[c0:c0 + ns, i] = pzcol[:ns]
            L = Lnew
    if dt == torch.complex64:
        ops.check_tc_status(dev)
    return (bits, pz) if return_pz else bits


def sample_mps(mps, num_shots, seed=0, chunk=16384, return_pz=False):
    ts = right_canonical_copy(mps)
    return sample_tensors(ts, num_shots, seed, chunk=chunk, return_pz=return_pz)
