"""CPU: the reference's own mpdok_ops.py binds libmpdok_gb300.so unmodified.

The reference module is copied byte for byte into a temporary directory and
imported under the NumPy stand-in for CuPy (tests/golden/cupy_shim).  Its two
solver classes load a library with ctypes.CDLL(lib_path) and set the argtypes
and restype of every py_* symbol they call; a symbol the library did not
export would raise AttributeError there.  The test then compares the
reference's argument lists with the signatures this package binds, so the
drop-in claim is checked against the reference's own binding code.

No compute call is made: that needs a GPU, and the reference checkout is not
present where the GPU tests run.  The checkout is looked up in the
MPDOK_REFERENCE environment variable, then next to this repository; the test
is skipped when neither exists.
"""
import importlib
import os
import shutil
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _reference_root():
    for cand in (os.environ.get("MPDOK_REFERENCE"), ROOT.parent / "reference"):
        if cand and (Path(cand) / "mpdok_ops.py").exists():
            return Path(cand)
    return None


@pytest.fixture(scope="module")
def ref_ops(tmp_path_factory):
    ref = _reference_root()
    if ref is None:
        pytest.skip("reference checkout not available")
    tmp = tmp_path_factory.mktemp("mpdok_ref_ops")
    shutil.copy(ref / "mpdok_ops.py", tmp / "mpdok_ops.py")
    assert (tmp / "mpdok_ops.py").read_bytes() == (ref / "mpdok_ops.py").read_bytes()
    old_path, old_dwb = list(sys.path), sys.dont_write_bytecode
    sys.dont_write_bytecode = True
    sys.path.insert(0, str(tmp))
    sys.path.insert(0, str(ROOT / "tests" / "golden" / "cupy_shim"))
    try:
        for m in ("mpdok_ops", "cupy"):
            sys.modules.pop(m, None)
        yield importlib.import_module("mpdok_ops")
    finally:
        for m in ("mpdok_ops", "cupy"):
            sys.modules.pop(m, None)
        sys.path[:] = old_path
        sys.dont_write_bytecode = old_dwb


def test_reference_solvers_bind_every_symbol(ref_ops, native_lib):
    from mpdok_gb300 import _native
    lib_path = str(_native.LIB_PATH)
    lu = ref_ops.LUIRSolver(lib_path=lib_path)
    gm = ref_ops.MPDOKSolver(lib_path=lib_path)
    bound = {
        "py_lu_ir": lu._lib.py_lu_ir, "py_lu_factor": lu._lib.py_lu_factor,
        "py_lu_solve_factored": lu._lib.py_lu_solve_factored, "py_lu_free_factored": lu._lib.py_lu_free_factored,
        "py_lu_alloc_managed": lu._lib.py_lu_alloc_managed, "py_lu_free_managed": lu._lib.py_lu_free_managed,
        "py_gmres_ir": gm._lib.py_gmres_ir, "py_alloc_managed": gm._lib.py_alloc_managed,
        "py_free_managed": gm._lib.py_free_managed,
    }
    for name, fn in bound.items():
        res, args = _native._SIGS[name]
        assert fn.restype is None and res is None, name
        ref_args = list(fn.argtypes or [])
        assert len(ref_args) == len(args), (name, ref_args, args)
        for a, b in zip(ref_args, args):
            # the reference passes device pointers as c_void_p and sizes as c_int / c_double
            assert a == b, (name, a, b)


def test_reference_empty_system_through_its_own_wrapper(ref_ops, native_lib):
    """py_gmres_ir with N = 0 needs no device: the reference's bound function
    returns converged = 1 through the int out-parameter, as it documents."""
    import ctypes
    from mpdok_gb300 import _native
    gm = ref_ops.MPDOKSolver(lib_path=str(_native.LIB_PATH))
    conv = ctypes.c_int(-3)
    gm._lib.py_gmres_ir(None, None, None, None, 0, 1e-11, 5, 50, ctypes.byref(conv))
    assert conv.value == 1
