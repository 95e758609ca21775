"""Generate golden vectors by running the reference's own Python modules on CPU.

Usage (in a container that has the reference checkout):
    python tests/golden/make_golden.py /path/to/MPDOK

The reference modules import CuPy; tests/golden/cupy_shim provides a NumPy
stand-in so they run unchanged on the CPU.  The modules are copied to a
temporary directory first so that nothing is written into the reference
checkout.  Outputs: tests/golden/*.npz (small; committed).
"""
from __future__ import annotations

import io
import os
import shutil
import sys
import tempfile
from contextlib import redirect_stdout
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent


def load_reference(ref_root: Path):
    tmp = Path(tempfile.mkdtemp(prefix="mpdok_ref_"))
    for name in ("dense_krylov.py", "mpdok_ooc.py", "rbf_kernel.py"):
        shutil.copy(ref_root / name, tmp / name)
    sys.dont_write_bytecode = True
    sys.path.insert(0, str(tmp))
    sys.path.insert(0, str(HERE / "cupy_shim"))
    import dense_krylov, mpdok_ooc, rbf_kernel  # noqa: E401
    return dense_krylov, mpdok_ooc, rbf_kernel, tmp


def hist_arr(h):
    return np.array([[float(i), float(r)] for i, r in h], dtype=np.float64).reshape(-1, 2)


def main(ref_root: str):
    dk, ooc, rk, tmp = load_reference(Path(ref_root))
    quiet = io.StringIO()

    # 1. assembly: rbf_kernel.synthetic_coords / _estimate_gamma / build_rbf_kernel / _build_rbf_cpu_into
    coords = rk.synthetic_coords(128, D=2, seed=5, scale=1.0)
    gamma_est = rk._estimate_gamma(coords)
    A_g, _ = rk.build_rbf_kernel(coords, gamma=9.0, reg=1e-6)
    A_auto, g_auto = rk.build_rbf_kernel(coords, reg=1e-3)
    A_cpu = np.empty((128, 128), order="F")
    rk._build_rbf_cpu_into(coords, 9.0, 1e-6, A_cpu, chunk=50)
    coords3 = rk.synthetic_coords(96, D=3, seed=6, scale=1.0)
    sq3 = np.sum(coords3 ** 2, axis=1)
    tile = ooc._build_fp32_tile(coords3, sq3, 16, 40, 25.0)
    np.savez_compressed(HERE / "rbf_assembly.npz", coords=coords, gamma_est=gamma_est, A_gauss=A_g,
                        A_auto=A_auto, gamma_auto=g_auto, A_cpu=A_cpu, coords3=coords3, tile3=tile)

    # 2. dense_krylov: cg / gmres / gmres_ir on the reference's own test matrices
    rng = np.random.default_rng(7)
    n = 96
    X = rng.standard_normal((n, n))
    A_spd = X.T @ X + n * np.eye(n)
    A_ns = X + n * np.eye(n)
    b = rng.standard_normal(n)
    with redirect_stdout(quiet):
        op_spd = dk.DenseLinearOperator(A_spd)
        op_ns = dk.DenseLinearOperator(A_ns)
        x_cg, h_cg, c_cg = dk.cg(op_spd, b, tol=1e-6)
        x_gm, h_gm, c_gm = dk.gmres(op_ns, b, tol=1e-6, restart=20)
        x_ir, h_ir, c_ir = dk.gmres_ir(op_ns, b, tol=1e-11, restart=20)
        x_ir2, h_ir2, c_ir2 = dk.gmres_ir(op_spd, b, tol=1e-11, restart=20)
        y32 = op_ns.matvec(b.astype(np.float32))
        rn = op_ns.residual_norm(x_ir, b)
    np.savez_compressed(HERE / "dense_krylov.npz", A_spd=A_spd, A_ns=A_ns, b=b,
                        x_cg=x_cg, h_cg=hist_arr(h_cg), c_cg=c_cg,
                        x_gm=x_gm, h_gm=hist_arr(h_gm), c_gm=c_gm,
                        x_ir=x_ir, h_ir=hist_arr(h_ir), c_ir=c_ir,
                        x_ir_spd=x_ir2, h_ir_spd=hist_arr(h_ir2), c_ir_spd=c_ir2,
                        y32=y32, rn=rn)

    # 3. mpdok_ooc: build (RAM and SSD stores), tiled GEMVs, inner GMRES, solve
    rng = np.random.default_rng(11)
    pts = rng.uniform(0.0, 1.0, size=(150, 2))
    bo = rng.standard_normal(150)
    with redirect_stdout(quiet):
        s = ooc.MPDOKOOCSolver(tile_rows=40)
        g = s.build(pts, gamma=9.0, reg=1e-2, store="ram", verbose=False)
        A32_ram = s._ram_buf.copy()
        y_sg = s._tiled_sgemv(bo.astype(np.float32))
        y_dg = s._tiled_dgemv_fp64(bo)
        e_in = s._inner_gmres(bo, 20)
        import warnings
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            x_ooc = s.solve(bo, tol=1e-10, maxiter_outer=8, restart=20, verbose=False)
        fd, path = tempfile.mkstemp(suffix=".bin")
        os.close(fd)
        s2 = ooc.MPDOKOOCSolver(tile_rows=40)
        s2.build(pts, gamma=9.0, reg=1e-2, store="ssd", path=path, verbose=False)
        raw = np.fromfile(path, dtype=np.float32)
        y_ssd = s2._tiled_sgemv(bo.astype(np.float32))
        os.remove(path)
    np.savez_compressed(HERE / "mpdok_ooc.npz", pts=pts, b=bo, gamma=g, A32=A32_ram, y_sgemv=y_sg,
                        y_dgemv=y_dg, e_inner=e_in, x=x_ooc, ssd_raw=raw, y_ssd=y_ssd)
    shutil.rmtree(tmp, ignore_errors=True)
    print("golden vectors written to", HERE)


if __name__ == "__main__":
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("MPDOK_REFERENCE")
    if not ref:
        sys.exit("usage: python tests/golden/make_golden.py <path to the MPDOK reference checkout> "
                 "(or set MPDOK_REFERENCE)")
    main(ref)
