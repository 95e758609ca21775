"""CPU baseline: the reference's SciPy FP64 direct path on the host cores.

TEST / BENCH INFRASTRUCTURE: run by bench.py (cpu_baseline leg and the
``--impl reference`` arm) in a child process, so that the BLAS thread count
can be set before NumPy loads.  It times scipy.linalg.lu_factor + lu_solve
(FP64, partial pivoting) plus FP64 refinement steps until the relative
residual meets the tolerance, on the same seeded RBF family as the GPU run.

    python -m oracle.cpu_baseline --n 32768 --repeats 2 --warmup-n 2048 --config HEADLINE
prints one JSON line: {"seconds": [...], "n": ..., "threads": ..., "relres": ..., "assembly_seconds": ...}.
Each repeat is one full solve of the N-point system (no sampling, no
scaling); --warmup-n runs one untimed solve of a small system of the same
family first, so that the BLAS threads are up before the timed solves.

    python -m oracle.cpu_baseline --config C4 --systems 0,37,101
times SciPy FP64 cho_factor + cho_solve (8 RHS) on the listed C4 systems and
prints {"seconds": ..., "flops": sum n^3/3, "relres_max": ..., "threads": ...}.
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
    ap.add_argument("--systems", default="")
    ap.add_argument("--warmup-n", type=int, default=0)
    args = ap.parse_args(argv)

    import numpy as np
    import scipy.linalg as sla

    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    from mpdok_gb300 import configs
    from oracle.krylov_ref import rbf_matrix

    if args.config.upper() == "C4":
        systems = configs.c4()
        pick = [int(t) for t in args.systems.split(",") if t.strip()] or [0]
        total, flops, worst = 0.0, 0.0, 0.0
        for i in pick:
            sysm = systems[i]
            A = rbf_matrix(sysm.coords, gamma=sysm.gamma, reg=sysm.reg)
            B = np.asarray(sysm.b, dtype=np.float64)
            t0 = time.perf_counter()
            x = sla.cho_solve(sla.cho_factor(A, lower=True, check_finite=False), B, check_finite=False)
            total += time.perf_counter() - t0
            flops += sysm.n ** 3 / 3.0
            worst = max(worst, float(np.max(np.linalg.norm(B - A @ x, axis=0) / np.linalg.norm(B, axis=0))))
        print(json.dumps({"seconds": total, "flops": flops, "systems": pick, "relres_max": worst,
                          "threads": int(os.environ.get("OPENBLAS_NUM_THREADS", "0")), "config": "C4"}))
        return

    gen = {"HEADLINE": configs.headline, "HARD": configs.hard_headline, "C3": configs.c3}[args.config.upper()]

    def system(n):
        sysm = gen(n=n)
        # the kernel matrix is symmetric, so the transposed view of the C-order
        # result is the column-major A of the reference ABI without a copy
        A = rbf_matrix(sysm.coords, gamma=sysm.gamma, reg=sysm.reg, kernel=sysm.kernel).T
        return A, np.asarray(sysm.b, dtype=np.float64)

    def solve(A, b):
        bn = float(np.linalg.norm(b))
        lu = sla.lu_factor(A, check_finite=False)
        x = sla.lu_solve(lu, b, check_finite=False)
        rel = float("nan")
        for _ in range(3):
            r = b - A @ x
            rel = float(np.linalg.norm(r)) / bn
            if rel <= args.tol:
                break
            x = x + sla.lu_solve(lu, r, check_finite=False)
        return rel

    if args.warmup_n > 0:
        solve(*system(args.warmup_n))
    t0 = time.perf_counter()
    A, b = system(args.n)
    t_asm = time.perf_counter() - t0
    times, rel = [], float("nan")
    for _ in range(args.repeats):
        t0 = time.perf_counter()
        rel = solve(A, b)
        times.append(time.perf_counter() - t0)
    print(json.dumps({"seconds": times, "n": args.n, "threads": int(os.environ.get("OPENBLAS_NUM_THREADS", "0")),
                      "relres": rel, "config": args.config, "assembly_seconds": t_asm,
                      "warmup_n": args.warmup_n}))


if __name__ == "__main__":
    main()
