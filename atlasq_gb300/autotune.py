"""Autotuning of the launch shapes the two-site pipeline uses.

The Householder tridiagonalisation (the eigensolver's first and longest stage)
runs one thread-block cluster per Gram matrix, keeping the packed matrix in the
cluster's distributed shared memory.  How many CTAs a cluster should have
depends on the matrix size and on how many problems share the GPU in one
launch (a 512 x 512 problem alone wants every SM it can get; twenty of them
want the cluster that just fits).  ``tune_tridiag`` times each admissible
cluster size on synthetic problems of that shape, inside the library, and the
library keeps the fastest for every later launch of that shape.

``tune_for_batches`` derives the shapes from the two-site problems a batch
will launch (n = 2 chi_R, count = gates per launch) and tunes each once.
"""
import ctypes
from typing import Dict, Iterable, Tuple

import torch

from . import _lib
from ._lib import check, dtype_code, ptr, stream_ptr

_done: Dict[Tuple[int, int, int], Tuple[int, float]] = {}


def _bucket(n: int) -> int:
    return (n + 31) // 32


def _count_class(count: int) -> int:
    return 0 if count <= 8 else (1 if count <= 32 else 2)


def tune_tridiag(n: int, count: int, dtype=torch.complex64, device="cuda"):
    """Tune the cluster size for `count` problems of size n; returns (C, ms)."""
    dev = _lib.require_cuda(device)
    lib = _lib.load()
    code = dtype_code(dtype)
    key = (code, _bucket(n), _count_class(count))
    if key in _done:
        return _done[key]
    n_t = min(1024, _bucket(n) * 32)  # tune at the top of the bucket
    count_t = {0: min(count, 8), 1: min(max(count, 9), 32), 2: max(count, 33)}[key[2]]
    need = lib.agb_tune_tridiag_workspace(code, n_t, count_t)
    ws = torch.empty(need, dtype=torch.uint8, device=dev)
    bc = ctypes.c_int(0)
    bms = ctypes.c_float(0)
    # (the library also tries 256 and 512 threads per CTA and keeps the faster)
    check(lib.agb_tune_tridiag(code, n_t, count_t, ptr(ws), need, stream_ptr(dev), ctypes.byref(bc),
                               ctypes.byref(bms)), "tune_tridiag")
    _done[key] = (bc.value, bms.value)
    return _done[key]


def tuned_cluster(n: int, count: int, dtype=torch.complex64) -> int:
    lib = _lib.load()
    return lib.agb_tuned_tridiag_cluster(dtype_code(dtype), n, count)


def tune_for_batches(batches: Iterable[Tuple[int, int]], dtype=torch.complex64, device="cuda"):
    """batches: (max n, problem count) of the launches to come."""
    out = {}
    for n, count in batches:
        if n >= 64:  # small problems finish in microseconds whatever the shape
            out[(n, count)] = tune_tridiag(n, count, dtype, device)
    return out
