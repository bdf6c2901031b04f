"""ctypes binding of the C ABI (``include/atlasq_gb300.h``).

The library is loaded from the package's ``lib/`` directory.  There is no CPU
or PyTorch fallback: if the library is missing or no CUDA device is present,
every operation raises.
"""
import ctypes
import os

import torch

from . import _build

AGB_OK = 0
AGB_ERR_ARG = 1
AGB_ERR_WORKSPACE = 2
AGB_ERR_NOCONV = 3
AGB_ERR_TIMEOUT = 4
AGB_ERR_CUDA = 5
AGB_ERR_UNSUPPORTED = 6
AGB_ERR_RANK = 7
AGB_ERR_TOO_LARGE = 8

AGB_C64 = 0
AGB_C128 = 1
AGB_RUN_REPAIR = 1
AGB_RUN_NO_GUARD = 2

# descriptor fields (enum agb_desc_field)
D_A, D_B, D_U, D_CHIL, D_CHIM, D_CHIR, D_CAP, D_EPS = 0, 1, 2, 3, 4, 5, 6, 7
D_ANEW, D_BNEW, D_ELL, D_SEED, D_WS, D_CTOL, D_ORTH, D_ORTHW = 8, 9, 10, 11, 12, 13, 14, 15
D_K, D_EPSLOC, D_ENTROPY, D_CONDS, D_STATUS, D_TOTAL, D_NEEDED, D_MODE = 16, 17, 18, 19, 20, 21, 22, 23
D_DIMS, D_BOND, D_CAPL, D_CAPM, D_CAPR, D_ELLPLAN, D_NVEC, D_REPAIR = 24, 25, 26, 27, 28, 29, 30, 31
D_NFIELDS = 32

MLP_NPARAM = 8769

STAGES = ["host_gap", "setup", "contract", "gram", "tridiag", "bisect", "invit", "cluster",
          "backtransform", "polish", "xv", "rank", "scatter"]

_ERRS = {
    AGB_ERR_ARG: (ValueError, "invalid argument or shape"),
    AGB_ERR_WORKSPACE: (RuntimeError, "workspace too small"),
    AGB_ERR_NOCONV: (RuntimeError, "eigensolver did not converge"),
    AGB_ERR_TIMEOUT: (RuntimeError, "device-side wait timed out"),
    AGB_ERR_CUDA: (RuntimeError, "CUDA launch failed"),
    AGB_ERR_UNSUPPORTED: (NotImplementedError, "size or mode not supported"),
    AGB_ERR_RANK: (RuntimeError, "eigenpairs computed below the required rank"),
    AGB_ERR_TOO_LARGE: (ValueError, "problem exceeds the fixed scratch of the allocation-free entry point"),
}

_lib = None

P = ctypes.c_void_p
I = ctypes.c_int
I64 = ctypes.c_int64
SZ = ctypes.c_size_t
D = ctypes.c_double
U64 = ctypes.c_uint64

_SIGS = {
    "agb_version": (I, []),
    "agb_contract_gate": (I, [I, P, P, P, P, I, I, I, P]),
    "agb_two_site_plan": (I, [I, I, P, ctypes.POINTER(SZ)]),
    "agb_two_site_run": (I, [I, I, P, P, I, I, I, I, P, SZ, P, I]),
    "agb_two_site_finalize": (I, [I, I, P, I, I, I, P, P]),
    "agb_two_site_spectra": (I, [I, I, P, P, I, P, P]),
    "agb_single_qubit_gate": (I, [I, P, P, I, I, P]),
    "agb_single_qubit_batch": (I, [I, I, P, I, P]),
    "agb_tune_tridiag_workspace": (SZ, [I, I, I]),
    "agb_tune_tridiag": (I, [I, I, I, P, SZ, P, P, P]),
    "agb_tuned_tridiag_cluster": (I, [I, I, I]),
    "agb_set_tridiag_cluster": (I, [I, I, I, I, I]),
    "agb_set_tridiag_stages": (I, [I]),
    "agb_heevd_workspace": (SZ, [I, I, I]),
    "agb_heevd": (I, [I, I, I, I, P, P, P, P, SZ, U64, P]),
    "agb_qr_workspace": (SZ, [I, I, I]),
    "agb_qr": (I, [I, P, I, I, I, P, P, I, P, SZ, P]),
    "agb_qr_noalloc": (I, [I, P, I, I, I, P, P, I, P]),
    "agb_sample_site": (I, [I, P, I, I, I, U64, U64, P, P, P, P]),
    "agb_mpo_mix": (I, [I, P, P, P, I, I, I, I, P]),
    "agb_trace_prod": (I, [I, P, P, I, P, P]),
    "agb_mpo_apply_site": (I, [I, P, P, P, I, I, I, I, P]),
    "agb_tdvp_local_h_workspace": (SZ, [I, I, I, I, I]),
    "agb_tdvp_local_h": (I, [I, P, P, P, P, P, I, I, I, I, I, I, P, SZ, P]),
    "agb_site_mix": (I, [I, P, P, P, I, I, I, P]),
    "agb_prof_begin": (I, [I]),
    "agb_launch_count": (ctypes.c_longlong, []),
    "agb_last_error": (ctypes.c_char_p, []),
    "agb_prof_end": (I, [P, P, I]),
    "agb_mlp_forward": (I, [P, P, I, P, P]),
    "agb_mlp_backward_workspace": (SZ, [I]),
    "agb_mlp_backward": (I, [P, P, P, I, P, P, P, SZ, P]),
    "agb_mlp_adam": (I, [P, P, P, P, I, ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                         ctypes.c_float, P]),
    "agb_cgemm_tc_workspace": (SZ, [I, I, I, I]),
    "agb_set_gemm_wait_limit": (I, [ctypes.c_longlong]),
    "agb_cgemm_tc": (I, [ctypes.c_char, ctypes.c_char, I, I, I, I, P, I64, I64, P, I64, I64, P, I64, I64,
                         ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_float, P, SZ, P, P]),
    "agb_cgemm_tc_async": (I, [ctypes.c_char, ctypes.c_char, I, I, I, I, P, I64, I64, P, I64, I64, P, I64, I64,
                               ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_float, P, SZ, P, P]),
    "agb_cgemm_batched": (I, [I, ctypes.c_char, ctypes.c_char, I, I, I, I, P, I64, I64, P, I64, I64,
                              P, I64, I64, D, D, D, D, P]),
}


def exported_symbols():
    return sorted(_SIGS)


def load(build_if_missing=True):
    """Load (building first if needed) the CUDA library; raise if impossible."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.lib_path()
    if not os.path.exists(path):
        if not build_if_missing:
            raise RuntimeError(f"atlasq_gb300 CUDA library not built: {path}")
        _build.build()
    lib = ctypes.CDLL(path)
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(rc, what=""):
    if rc != AGB_OK:
        exc, msg = _ERRS.get(rc, (RuntimeError, f"error {rc}"))
        where = ""
        if rc == AGB_ERR_CUDA and _lib is not None:
            site = _lib.agb_last_error()
            if site:
                where = f" at {site.decode(errors='replace')}"
        raise exc(f"atlasq_gb300: {what}: {msg} (status {rc}){where}")


def require_cuda(device):
    dev = torch.device(device)
    if dev.type != "cuda" or not torch.cuda.is_available():
        raise RuntimeError("atlasq_gb300 runs on a CUDA device only (GB300, sm_103a); "
                           f"got device={device!r}, cuda available={torch.cuda.is_available()}")
    if dev.index is None:  # "cuda" -> "cuda:<current>", so device comparisons with tensors hold
        dev = torch.device("cuda", torch.cuda.current_device())
    return dev


def dtype_code(dtype):
    if dtype == torch.complex64:
        return AGB_C64
    if dtype == torch.complex128:
        return AGB_C128
    raise ValueError(f"unsupported dtype {dtype}")


def stream_ptr(device=None):
    return ctypes.c_void_p(torch.cuda.current_stream(device).cuda_stream)


def ptr(t):
    return ctypes.c_void_p(t.data_ptr())
