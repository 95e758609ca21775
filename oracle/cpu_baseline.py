"""CPU baseline: the reference's SciPy FP64 direct path on the host cores.

TEST / BENCH INFRASTRUCTURE: run by bench.py (cpu_baseline leg and the
``--impl reference`` arm) in a child process, so that the BLAS thread count
can be set before NumPy loads.  It times scipy.linalg.lu_factor + lu_solve
(FP64, partial pivoting) plus FP64 refinement steps until the relative
residual meets the tolerance, on the same seeded RBF family as the GPU run.

    python -m oracle.cpu_baseline --n 8192 --repeats 1 --config HEADLINE
prints one JSON line: {"seconds": [...], "n": ..., "threads": ..., "relres": ...}
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=8192)
    ap.add_argument("--repeats", type=int, default=1)
    ap.add_argument("--config", default="HEADLINE")
    ap.add_argument("--tol", type=float, default=1e-12)
    args = ap.parse_args(argv)

    import numpy as np
    import scipy.linalg as sla

    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    from mpdok_gb300 import configs
    from oracle.krylov_ref import rbf_matrix

    gen = {"HEADLINE": configs.headline, "C3": configs.c3}[args.config.upper()]
    sysm = gen(n=args.n)
    A = np.asfortranarray(rbf_matrix(sysm.coords, gamma=sysm.gamma, reg=sysm.reg, kernel=sysm.kernel))
    b = np.asarray(sysm.b, dtype=np.float64)
    bn = float(np.linalg.norm(b))
    times, rel = [], float("nan")
    for _ in range(args.repeats):
        t0 = time.perf_counter()
        lu = sla.lu_factor(A, check_finite=False)
        x = sla.lu_solve(lu, b, check_finite=False)
        for _ in range(3):
            r = b - A @ x
            rel = float(np.linalg.norm(r)) / bn
            if rel <= args.tol:
                break
            x = x + sla.lu_solve(lu, r, check_finite=False)
        times.append(time.perf_counter() - t0)
    print(json.dumps({"seconds": times, "n": args.n, "threads": int(os.environ.get("OPENBLAS_NUM_THREADS", "0")),
                      "relres": rel, "config": args.config}))


if __name__ == "__main__":
    main()
