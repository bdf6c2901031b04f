"""The allocation-free QR entry point (agb_qr_noalloc) against the regular one.

agb_qr_noalloc exists for callers that cannot allocate device memory (e.g. a
host runtime that only receives device pointers through the C ABI): its scratch
is a fixed device array inside the library instead of a caller workspace.  This
file is collected last so that a failure here leaves every other test already
run; it must pass alone in a fresh process and after the rest of the suite."""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

from atlasq_gb300 import _lib  # noqa: E402

DEV = "cuda:0"
TOL = {torch.complex64: 1e-5, torch.complex128: 1e-12}


def _rand(shape, dtype, seed):
    g = torch.Generator().manual_seed(seed)
    x = torch.complex(torch.randn(*shape, generator=g, dtype=torch.float64),
                      torch.randn(*shape, generator=g, dtype=torch.float64))
    return x.to(dtype).to(DEV)


def _qr(lib, fn, A, M, N, trans, dtype):
    kk = min(M, N)
    if trans:
        Q = torch.empty(kk, M, dtype=dtype, device=DEV)
        R = torch.empty(N, kk, dtype=dtype, device=DEV)
    else:
        Q = torch.empty(M, kk, dtype=dtype, device=DEV)
        R = torch.empty(kk, N, dtype=dtype, device=DEV)
    code = _lib.dtype_code(dtype)
    stream = _lib.stream_ptr(DEV)
    if fn == "noalloc":
        rc = lib.agb_qr_noalloc(code, _lib.ptr(A), M, N, int(trans), _lib.ptr(Q), _lib.ptr(R), int(trans), stream)
    else:
        need = lib.agb_qr_workspace(code, M, N)
        ws = torch.empty(need, dtype=torch.uint8, device=DEV)
        rc = lib.agb_qr(code, _lib.ptr(A), M, N, int(trans), _lib.ptr(Q), _lib.ptr(R), int(trans),
                        _lib.ptr(ws), need, stream)
    _lib.check(rc, fn)
    torch.cuda.synchronize()
    return Q.cpu(), R.cpu()


@pytest.mark.parametrize("dtype", [torch.complex64, torch.complex128])
def test_noalloc_qr_matches_regular_entry_point_twice(dtype):
    lib = _lib.load()
    # two calls in a row with different inputs, then a size where agb_qr takes its
    # blocked cluster kernels (M*N >= 4096) while noalloc stays single-CTA
    cases = [((96, 40), False, 1), ((33, 70), True, 2), ((256, 128), False, 3)]
    for (rows, cols), trans, seed in cases:
        A = _rand((rows, cols), dtype, seed)
        M, N = (cols, rows) if trans else (rows, cols)
        Qa, Ra = _qr(lib, "noalloc", A, M, N, trans, dtype)
        Qb, Rb = _qr(lib, "regular", A, M, N, trans, dtype)
        tol = TOL[dtype]
        assert torch.allclose(Qa, Qb, atol=tol, rtol=tol)
        assert torch.allclose(Ra, Rb, atol=tol * float(Rb.abs().max()), rtol=tol)
        Aop = (A.T if trans else A).cpu().to(torch.complex128)
        Qm, Rm = (Qa.T, Ra.T) if trans else (Qa, Ra)
        assert float((Qm.to(torch.complex128) @ Rm.to(torch.complex128) - Aop).abs().max()) < 10 * tol * float(Aop.abs().max())


def test_noalloc_rejects_problems_beyond_the_fixed_scratch():
    lib = _lib.load()
    M, N = 2048, 1024  # complex64 working copy alone is 16 MiB > 8 MiB
    dummy = torch.empty(1, dtype=torch.complex64, device=DEV)
    rc = lib.agb_qr_noalloc(_lib.AGB_C64, _lib.ptr(dummy), M, N, 0, _lib.ptr(dummy), _lib.ptr(dummy), 0,
                            _lib.stream_ptr(DEV))
    assert rc == _lib.AGB_ERR_TOO_LARGE
    with pytest.raises(ValueError):
        _lib.check(rc, "qr_noalloc")
