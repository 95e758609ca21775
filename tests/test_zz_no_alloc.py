"""GPU: the allocation-free GEMV entry point (mpdok_gemv_noalloc).

It exists for callers that cannot allocate device memory where they need a
product: their GPU memory is already committed to another pool, or they must
not cause the device synchronisation an allocation can bring.  Its scratch is a
fixed built-in device array, so the test checks that it gives the same result
as the allocating entry point (mpdok_gemv, caller-owned workspace) on two
calls in a row (the array keeps the previous call's contents) and that a
product too large for the array is refused with a clear error.

Collected last (file name) so that a run stopping at the first failure has
already run every other test; it also passes alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


@pytest.mark.parametrize("dt,m,n,nrhs,trans", [("f32", 4099, 3001, 1, 0), ("f32", 2000, 2500, 4, 0),
                                                ("f64", 3000, 2048, 1, 0), ("f32", 1500, 1700, 1, 1),
                                                ("bf16", 4096, 4096, 2, 0)])
def test_noalloc_gemv_matches_allocating_entry_point(dt, m, n, nrhs, trans):
    from mpdok_gb300 import _native as N
    lib = N.load()
    code = {"f32": N.F32, "f64": N.F64, "bf16": N.BF16}[dt]
    tdt = {"f32": torch.float32, "f64": torch.float64, "bf16": torch.bfloat16}[dt]
    xdt = torch.float64 if dt == "f64" else torch.float32
    g = torch.Generator(device="cuda").manual_seed(m + n + nrhs)
    A = torch.randn(n, m, device="cuda", generator=g).to(tdt).t()  # column-major (m, n)
    k_in, k_out = (m, n) if trans else (n, m)
    ws = torch.empty(lib.mpdok_gemv_workspace_size(code, m, n, nrhs, trans), dtype=torch.uint8, device="cuda")
    for call in range(2):
        X = torch.randn(nrhs, k_in, device="cuda", generator=g, dtype=xdt).t()
        Y0 = torch.randn(nrhs, k_out, device="cuda", generator=g, dtype=xdt).t()
        Y_ref, Y_na = Y0.clone().t().contiguous().t(), Y0.clone().t().contiguous().t()
        assert lib.mpdok_gemv(code, trans, _ptr(A), m, m, n, _ptr(X), k_in, nrhs, _ptr(Y_ref), k_out, 1.5, -0.5,
                              _ptr(ws), ws.numel(), None) == 0, N.last_error()
        assert lib.mpdok_gemv_noalloc(code, trans, _ptr(A), m, m, n, _ptr(X), k_in, nrhs, _ptr(Y_na), k_out, 1.5,
                                      -0.5, None) == 0, N.last_error()
        torch.cuda.synchronize()
        tol = 1e-12 if dt == "f64" else 1e-5
        scale = Y_ref.abs().max().item() + 1e-30
        assert torch.allclose(Y_na, Y_ref, rtol=0, atol=tol * scale), f"call {call}"


def test_noalloc_gemv_rejects_products_beyond_its_scratch():
    from mpdok_gb300 import _native as N
    lib = N.load()
    m = n = 1 << 20  # partial sums of this product need far more than the built-in array
    assert lib.mpdok_gemv_workspace_size(N.F64, m, n, 8, 0) > N.NOALLOC_SCRATCH_BYTES
    st = lib.mpdok_gemv_noalloc(N.F64, 0, ctypes.c_void_p(256), m, m, n, ctypes.c_void_p(256), n, 8,
                                ctypes.c_void_p(256), m, 1.0, 0.0, None)
    assert st == N.ERR_INVALID_ARG
    assert "built-in scratch" in N.last_error()
