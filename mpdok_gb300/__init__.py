"""mpdok_gb300 — GB300-native (sm_103a) dense-operator Krylov solvers for RBF systems.

Drop-in for MPDOK's Python solver API, backed by hand-written CUDA in
libmpdok_gb300.so (C ABI, ctypes):

* ``rbf_kernel``:   synthetic_coords, _estimate_gamma, build_rbf_kernel, weather_front
* ``dense_krylov``: DenseLinearOperator, cg, gmres, gmres_ir
* ``mpdok_ops``:    MPDOKSolver (py_gmres_ir), LUIRSolver (py_lu_*)
* ``mpdok_ooc``:    MPDOKOOCSolver (pinned-host streamed tiles)
"""
from . import _native  # noqa: F401

__version__ = "1.0.0"


def build(verbose: bool = False):
    """Compile libmpdok_gb300.so for sm_103a (in-tree)."""
    from . import _build
    return _build.build(verbose=verbose)
