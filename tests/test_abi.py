"""CPU: the C-ABI library loads and exports every symbol include/*.h declares.

No compute calls are made (there is no GPU here); only host-side entry points
that validate arguments or report sizes are exercised.
"""
import ctypes
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def header_symbols():
    syms = []
    for h in sorted((ROOT / "include").glob("*.h")):
        txt = h.read_text()
        syms += re.findall(r"MPDOK_API\s+[A-Za-z_][A-Za-z0-9_\s\*]*?\b([a-z_][a-z0-9_]*)\s*\(", txt)
    return sorted(set(syms))


def test_header_declares_reference_abi():
    syms = header_symbols()
    for name in ("py_gmres_ir", "py_alloc_managed", "py_free_managed"):
        assert name in syms


def test_library_exports_every_declared_symbol(native_lib):
    missing = [s for s in header_symbols() if not hasattr(native_lib, s)]
    assert not missing, f"declared but not exported: {missing}"


def test_ctypes_signatures_cover_exports(native_lib):
    from mpdok_gb300 import _native
    for name in _native.declared_symbols():
        assert hasattr(native_lib, name), name
    assert set(header_symbols()) >= set(_native.declared_symbols())


def test_host_only_entry_points(native_lib):
    assert native_lib.mpdok_version() >= 10000
    assert native_lib.mpdok_status_string(0) == b"ok"
    assert b"invalid" in native_lib.mpdok_status_string(-1)
    assert native_lib.mpdok_krylov_workspace_size(1000, 50) > 1000 * 51 * 4
    assert native_lib.mpdok_krylov_workspace_size(-1, 50) == 0
    assert native_lib.mpdok_gemv_workspace_size(1, 4096, 4096, 1, 0) > 0


def test_argument_validation_without_gpu(native_lib):
    from mpdok_gb300 import _native as N
    # bad dim / null pointers are rejected before any device work
    s = native_lib.mpdok_rbf_assemble(None, 10, None, 10, 5, 0, 1.0, 0.0, 0, N.F64, None, 10, 1, None)
    assert s == N.ERR_INVALID_ARG
    assert b"dim" in native_lib.mpdok_last_error() or b"null" in native_lib.mpdok_last_error()
    s = native_lib.mpdok_gemv(9, 0, ctypes.c_void_p(16), 4, 4, 4, None, 4, 1, None, 4, 1.0, 0.0, None, 0, None)
    assert s == N.ERR_INVALID_ARG
    info = N.SolveInfo()
    s = native_lib.mpdok_gmres_ir(None, 4, None, 4, 0, 4, None, None, 1e-10, 3, 0, 1e-6, None, 0,
                                  ctypes.byref(info), None)
    assert s == N.ERR_INVALID_ARG
    # empty systems are trivially converged
    s = native_lib.mpdok_gmres_ir(None, 1, None, 1, 0, 0, None, None, 1e-10, 3, 5, 1e-6, None, 0,
                                  ctypes.byref(info), None)
    assert s == 0 and info.converged == 1


def test_reference_abi_tolerates_empty_system(native_lib):
    conv = ctypes.c_int(-7)
    native_lib.py_gmres_ir(None, None, None, None, 0, 1e-11, 5, 50, ctypes.byref(conv))
    assert conv.value == 1
