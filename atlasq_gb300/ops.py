"""Torch-facing wrappers of the C ABI.  PyTorch supplies device memory and the
current stream; every computation is a kernel of ``libatlasq_gb300.so``."""
import ctypes

import torch

from . import _lib
from ._lib import check, dtype_code, ptr, stream_ptr

_WS = {}


def workspace(nbytes, device, tag="default"):
    """Grow-only per-device scratch buffer (uint8)."""
    key = (tag, torch.device(device).index or 0)
    buf = _WS.get(key)
    if buf is None or buf.numel() < nbytes:
        buf = torch.empty(max(int(nbytes), 256), dtype=torch.uint8, device=device)
        _WS[key] = buf
    return buf


def _c(t):
    if not t.is_contiguous():
        raise ValueError("atlasq_gb300 kernels take contiguous tensors")
    return t


def contract_gate(A, B, U):
    """X[2chiL, 2chiR] = gate U applied to contract(A, B) (mps_complex.py:343-368 layout)."""
    lib = _lib.load()
    A, B = _c(A), _c(B)
    U = U.reshape(4, 4).to(device=A.device, dtype=A.dtype).contiguous()
    chiL, _, chiM = A.shape
    chiR = B.shape[2]
    if B.shape[0] != chiM or A.shape[1] != 2 or B.shape[1] != 2:
        raise ValueError("shape mismatch in contract_gate")
    X = torch.empty(2 * chiL, 2 * chiR, dtype=A.dtype, device=A.device)
    check(lib.agb_contract_gate(dtype_code(A.dtype), ptr(A), ptr(B), ptr(U), ptr(X), chiL, chiM, chiR,
                                stream_ptr(A.device)), "contract_gate")
    return X


def cgemm(A, B, opA="N", opB="N", alpha=1.0, beta=0.0, C=None):
    """C = alpha op(A) op(B) + beta C for 2-D or batched 3-D contiguous tensors."""
    lib = _lib.load()
    A, B = _c(A), _c(B)
    batched = A.dim() == 3
    if not batched:
        A2, B2 = A.unsqueeze(0), B.unsqueeze(0)
    else:
        A2, B2 = A, B
    bat = A2.shape[0]
    ra, ca = A2.shape[1], A2.shape[2]
    rb, cb = B2.shape[1], B2.shape[2]
    M, K = (ra, ca) if opA in ("N", "R") else (ca, ra)
    K2, N = (rb, cb) if opB in ("N", "R") else (cb, rb)
    if K != K2:
        raise ValueError(f"inner dimension mismatch {K} vs {K2}")
    if C is None:
        C = torch.empty(bat, M, N, dtype=A.dtype, device=A.device)
        beta = 0.0
    else:
        C = C if batched else C.unsqueeze(0)
    al = complex(alpha)
    be = complex(beta)
    check(lib.agb_cgemm_batched(dtype_code(A.dtype), opA.encode(), opB.encode(), bat, M, N, K,
                                ptr(A2), ca, ra * ca, ptr(B2), cb, rb * cb, ptr(C), N, M * N,
                                al.real, al.imag, be.real, be.imag, stream_ptr(A.device)), "cgemm")
    return C if batched else C[0]


def cgemm_strided(batch, M, N, K, A, a_off, lda, sA, B, b_off, ldb, sB, C, c_off, ldc, sC, opA="N", opB="N",
                  alpha=1.0, beta=0.0):
    """Strided-batch GEMM on raw layouts: batch entry z uses A from element
    a_off + z * sA with row stride lda (likewise B, C); op(A) is M x K, op(B)
    K x N.  Lets a contraction read and write a permuted index order in place."""
    lib = _lib.load()
    for t in (A, B, C):
        _c(t)
    es = A.element_size()
    al, be = complex(alpha), complex(beta)
    check(lib.agb_cgemm_batched(dtype_code(A.dtype), opA.encode(), opB.encode(), batch, M, N, K,
                                ctypes.c_void_p(A.data_ptr() + a_off * es), lda, sA,
                                ctypes.c_void_p(B.data_ptr() + b_off * es), ldb, sB,
                                ctypes.c_void_p(C.data_ptr() + c_off * es), ldc, sC,
                                al.real, al.imag, be.real, be.imag, stream_ptr(A.device)), "cgemm_strided")
    return C


def heevd(H, ell=None, seed=0):
    """Top-`ell` eigenpairs of Hermitian H ([n,n] or [batch,n,n]); descending.
    H is not modified (a copy is reduced)."""
    lib = _lib.load()
    batched = H.dim() == 3
    Hb = (H if batched else H.unsqueeze(0)).contiguous().clone()
    bat, n, _ = Hb.shape
    ell = n if ell is None else int(ell)
    rdt = torch.float32 if H.dtype == torch.complex64 else torch.float64
    evals = torch.empty(bat, ell, dtype=rdt, device=H.device)
    evecs = torch.empty(bat, n, ell, dtype=H.dtype, device=H.device)
    per = lib.agb_heevd_workspace(dtype_code(H.dtype), n, ell)
    ws = workspace(per * bat, H.device, "heevd")
    check(lib.agb_heevd(dtype_code(H.dtype), bat, n, ell, ptr(Hb), ptr(evals), ptr(evecs), ptr(ws),
                        ws.numel(), ctypes.c_uint64(seed), stream_ptr(H.device)), "heevd")
    return (evals, evecs) if batched else (evals[0], evecs[0])


def qr(A, transA=False, trans_out=False):
    """Thin Householder QR of op(A); returns (Q, R) (or (Q^T, R^T) with trans_out)."""
    lib = _lib.load()
    A = _c(A)
    M, N = (A.shape[1], A.shape[0]) if transA else (A.shape[0], A.shape[1])
    kk = min(M, N)
    if trans_out:
        Q = torch.empty(kk, M, dtype=A.dtype, device=A.device)
        R = torch.empty(N, kk, dtype=A.dtype, device=A.device)
    else:
        Q = torch.empty(M, kk, dtype=A.dtype, device=A.device)
        R = torch.empty(kk, N, dtype=A.dtype, device=A.device)
    need = lib.agb_qr_workspace(dtype_code(A.dtype), M, N)
    ws = workspace(need, A.device, "qr")
    check(lib.agb_qr(dtype_code(A.dtype), ptr(A), M, N, int(transA), ptr(Q), ptr(R), int(trans_out),
                     ptr(ws), ws.numel(), stream_ptr(A.device)), "qr")
    return Q, R


def single_qubit_gate_(T, U):
    """In place: T[a,t,b] <- sum_s U[s,t] T[a,s,b]."""
    lib = _lib.load()
    T = _c(T)
    U = U.to(device=T.device, dtype=T.dtype).contiguous()
    check(lib.agb_single_qubit_gate(dtype_code(T.dtype), ptr(T), ptr(U), T.shape[0], T.shape[2],
                                    stream_ptr(T.device)), "single_qubit_gate")
    return T


_TC_STATUS = {}


def _tc_status_word(device):
    dev = torch.device(device)
    key = dev.index or 0
    w = _TC_STATUS.get(key)
    if w is None:
        w = torch.zeros(1, dtype=torch.int32, device=dev)
        _TC_STATUS[key] = w
    return w


def check_tc_status(device):
    """Raise if a tensor-core GEMM issued with sync=False on `device` had a
    bounded wait expire since the last check (reads one device word)."""
    w = _tc_status_word(device)
    v = int(w.item())
    if v:
        w.zero_()
        check(v, "cgemm_tc")


def cgemm_tc(A, B, opA="N", opB="N", alpha=1.0, beta=0.0, C=None, sync=True):
    """complex64 GEMM on the tcgen05 tensor cores (3xTF32); same contract as cgemm.
    sync=False issues it without synchronising the stream; check_tc_status()
    reports a timeout of any such call."""
    lib = _lib.load()
    A, B = _c(A), _c(B)
    if A.dtype != torch.complex64:
        raise ValueError("cgemm_tc takes complex64")
    batched = A.dim() == 3
    A2, B2 = (A, B) if batched else (A.unsqueeze(0), B.unsqueeze(0))
    bat = A2.shape[0]
    ra, ca = A2.shape[1], A2.shape[2]
    rb, cb = B2.shape[1], B2.shape[2]
    M, K = (ra, ca) if opA in ("N", "R") else (ca, ra)
    K2, N = (rb, cb) if opB in ("N", "R") else (cb, rb)
    if K != K2:
        raise ValueError(f"inner dimension mismatch {K} vs {K2}")
    if C is None:
        C = torch.empty(bat, M, N, dtype=A.dtype, device=A.device)
        beta = 0.0
    else:
        C = C if batched else C.unsqueeze(0)
    need = lib.agb_cgemm_tc_workspace(bat, M, N, K)
    ws = workspace(need, A.device, "gemm_tc")
    al, be = complex(alpha), complex(beta)
    if sync:
        st = ctypes.c_int(0)
        check(lib.agb_cgemm_tc(opA.encode(), opB.encode(), bat, M, N, K, ptr(A2), ca, ra * ca, ptr(B2), cb,
                               rb * cb, ptr(C), N, M * N, al.real, al.imag, be.real, be.imag, ptr(ws), ws.numel(),
                               ctypes.byref(st), stream_ptr(A.device)), "cgemm_tc")
    else:
        check(lib.agb_cgemm_tc_async(opA.encode(), opB.encode(), bat, M, N, K, ptr(A2), ca, ra * ca, ptr(B2), cb,
                                     rb * cb, ptr(C), N, M * N, al.real, al.imag, be.real, be.imag, ptr(ws),
                                     ws.numel(), ptr(_tc_status_word(A.device)), stream_ptr(A.device)),
              "cgemm_tc")
    return C if batched else C[0]
