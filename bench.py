#!/usr/bin/env python
"""Headline benchmark: time to FP64 relres <= 1e-12 on the N=32768 Gaussian RBF system.

One step = one complete solve of the headline system from x = 0 to the FP64
relative residual tolerance (factorization / FP32 copy included, assembly
excluded), with A already resident in HBM.  Prints ONE JSON line.

Extra keys:
  fp64_gpu_baseline  the plain FP64 GPU solve of the same system (FP64 LU of
                     the vendor library + FP64 refinement), timed once
  roofline           the dominant kernel class, timed live with CUDA events
  cpu_baseline       SciPy FP64 LU + refinement on all host cores, on the
                     same full-size system (one timed solve)
  e2e                the same solve through the public API with host inputs
                     (pinned host -> device copy and x back to the host timed)

--impl reference runs the reference's CPU path (SciPy FP64 LU, the oracle)
instead, on rank 0 only.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

HEADLINE_METRIC = "time to FP64 relres<=1e-12, mixed-precision GMRES-IR vs plain FP64 GPU solve (N=32768 Gaussian RBF)"
UNIT = "s"
FALLBACK_HBM = 6800.0
FALLBACK_BF16 = 1900.0


def _peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d.get("hbm_gbs", FALLBACK_HBM)), float(d.get("bf16_tflops", FALLBACK_BF16)), \
            float(d.get("bf16_tflops_sustained", FALLBACK_BF16)), "measured"
    return FALLBACK_HBM, FALLBACK_BF16, 1700.0, "fallback"


# the kernels behind the profiled classes
KERNEL_NAMES = {
    "lu_gemm_deep": "tc::ws::tc_gemm_update_ws (the 16-bit factorization's tcgen05 trailing updates, K >= 128)",
    "lu_gemm": "k_gemm_update_f32 (FP32 factors) and tc::tc_gemm_update (K = 64)",
    "lu_panel": "k_lu_diag + k_trsm_pair (the chain and below-panel windows)",
    "trsv": "k_trsv + k_scale_out",
    "gemv_f32": "gemv_n_stage1 (FP32 and 16-bit stored operator)",
    "gemv_f64": "gemv_n_stage1 (FP64 stored operator)",
}


def _traffic_model():
    """DRAM bytes per unit of algorithmic work, from the committed ncu summary
    (profiles/traffic.json); empty when no capture has been summarised."""
    p = ROOT / "profiles" / "traffic.json"
    if p.exists():
        try:
            return json.loads(p.read_text())
        except Exception:
            return {}
    return {}


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.idx = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sms, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sms.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        sms.sort()
        med = sms[len(sms) // 2] if sms else None
        return {"sm_mhz": med, "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sms)}


def cpu_lu_sample(n_sample: int, repeats: int, config: str = "HEADLINE", warmup_n: int = 0):
    """SciPy FP64 LU solve timed in a child process with all host threads."""
    try:
        threads = len(os.sched_getaffinity(0))
    except AttributeError:
        threads = os.cpu_count() or 1
    env = dict(os.environ, OPENBLAS_NUM_THREADS=str(threads), OMP_NUM_THREADS=str(threads),
               MKL_NUM_THREADS=str(threads))
    out = subprocess.run([sys.executable, "-m", "oracle.cpu_baseline", "--n", str(n_sample), "--repeats",
                          str(repeats), "--config", config, "--warmup-n", str(warmup_n)], cwd=str(ROOT), env=env,
                         capture_output=True, text=True, timeout=1800)
    if out.returncode != 0:
        raise RuntimeError(out.stderr[-2000:])
    d = json.loads(out.stdout.strip().splitlines()[-1])
    d["threads"] = threads
    return d


def update_standalone(n: int, warmup: int, reps: int) -> dict:
    """The factorization's first far update alone: C ((n - w) x (n - w), FP32,
    larger than L2) -= A B^T with K = w, the super-panel width, FP16
    operands, through the library's tensor-core update; CUDA events on the
    launching stream."""
    import torch
    from mpdok_gb300 import _native as NV
    from mpdok_gb300.lu import gemm_update
    s = NV.lu_schedule(16384, NV.F16)
    w = sorted({int(j) for j in s[s[:, 0] == 0][:, 2]})[1]
    m = n - w
    C = torch.zeros((m, m), dtype=torch.float32, device="cuda").t()
    A = (torch.randn((m, w), device="cuda") * 1e-2).half()
    B = (torch.randn((m, w), device="cuda") * 1e-2).half()
    for _ in range(warmup):
        gemm_update(C, A, B)
    st = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(st)
    for _ in range(reps):
        gemm_update(C, A, B)
    e1.record(st)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    hbm, bf16, bf16s, kind = _peaks()
    flops = 2.0 * m * m * w
    byts = 8.0 * m * m + 2.0 * w * 2 * m
    # timed alone: the burst bf16 peak is its denominator (the sustained one beside it)
    out = {"shape": f"{m}x{m}x{w}", "ms": ms, "TFLOPs": flops / ms / 1e9, "frac_of_burst_bf16": flops / ms / 1e9 / bf16,
           "frac_of_sustained_bf16": flops / ms / 1e9 / bf16s, "GBs": byts / ms / 1e6,
           "frac_of_hbm": byts / ms / 1e6 / hbm, "arithmetic_intensity_flop_per_byte": flops / byts,
           "peak_source": f"{kind}"}
    del C, A, B
    torch.cuda.empty_cache()
    return out


def gemv_standalone(n: int, warmup: int, reps: int) -> dict:
    """Stored-matrix GEMV y = A x on (n x n) column-major FP32 / FP64 / BF16
    operands larger than L2, timed with CUDA events on the launching stream."""
    import ctypes
    import torch
    from mpdok_gb300 import _native as NV
    lib = NV.load()
    hbm = _peaks()[0]
    out = {}
    for name, code, tdt in (("f32", NV.F32, torch.float32), ("f64", NV.F64, torch.float64),
                            ("bf16", NV.BF16, torch.bfloat16)):
        A = torch.empty((n, n), dtype=tdt, device="cuda").normal_().t()
        xdt = torch.float64 if name == "f64" else torch.float32
        x = torch.randn(n, device="cuda", dtype=xdt)
        y = torch.empty(n, device="cuda", dtype=xdt)
        ws = torch.empty(lib.mpdok_gemv_workspace_size(code, n, n, 1, 0), dtype=torch.uint8, device="cuda")
        args = (code, 0, ctypes.c_void_p(A.data_ptr()), n, n, n, ctypes.c_void_p(x.data_ptr()), n, 1,
                ctypes.c_void_p(y.data_ptr()), n, 1.0, 0.0, ctypes.c_void_p(ws.data_ptr()), ws.numel(), None)
        for _ in range(warmup):
            NV.check(lib.mpdok_gemv(*args), "gemv")
        st = torch.cuda.current_stream()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(st)
        for _ in range(reps):
            lib.mpdok_gemv(*args)
        e1.record(st)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / reps
        byts = A.element_size() * n * n + 2 * x.element_size() * n
        out[name] = {"ms": ms, "GBs": byts / ms / 1e6, "frac_of_hbm": byts / ms / 1e6 / hbm,
                     "bytes_per_launch": byts}
        del A
        torch.cuda.empty_cache()
    # matrix-free evaluate-and-multiply on the headline centres (no stored A)
    from mpdok_gb300 import configs
    sysm = configs.headline(n=n)
    coords = torch.from_numpy(sysm.coords).cuda()
    x = torch.randn(n, device="cuda")
    y = torch.empty(n, device="cuda")
    ws = torch.empty(lib.mpdok_matfree_workspace_size(n, n, 1, NV.F32), dtype=torch.uint8, device="cuda")
    args = (ctypes.c_void_p(coords.data_ptr()), n, ctypes.c_void_p(coords.data_ptr()), n, 2, NV.KERNEL_GAUSSIAN,
            sysm.gamma, sysm.reg, 0, NV.F32, ctypes.c_void_p(x.data_ptr()), n, 1, ctypes.c_void_p(y.data_ptr()), n,
            ctypes.c_void_p(ws.data_ptr()), ws.numel(), None)
    for _ in range(warmup):
        NV.check(lib.mpdok_matfree_apply(*args), "matfree")
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record()
    for _ in range(reps):
        lib.mpdok_matfree_apply(*args)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    sfu = 16 * 152 * 2.07e9  # nominal MUFU ops/s (16 per SM per clock)
    out["matfree_f32"] = {"ms": ms, "entries_per_s": n * n / ms * 1e3, "frac_of_nominal_sfu": n * n / ms * 1e3 / sfu,
                          "note": "Gaussian, 2-D headline centres, entries recomputed (A never stored)"}
    out["n"] = n
    out["note"] = "A larger than L2 (129 MB) for n >= 8192; FP64 is bound by GB300's FP64 pipe, not HBM"
    return out


DF_FMA_OPS = 13  # FP32 instructions per double-float multiply-add in the trailing update


def bench_batch(args, emit: bool = True) -> dict:
    """C4: 256 Gaussian RBF systems, N ~ U{500..8000}, eps ~ U(2, 8), nugget 1e-8,
    8 RHS each.  One step = factor + solve + 2 FP64 refinement steps (one CUDA
    graph launch) + the adjoint of L = ||X - X*||^2 (one more solve on the
    stored factors + the fused gradient contraction), inputs resident in HBM."""
    import numpy as np
    import torch
    from mpdok_gb300 import configs
    from mpdok_gb300.batch import BatchedRBFSolver, pack_coords, pack_rhs
    from mpdok_gb300.replicas import max_over_ranks, shard_imbalance, shard_systems
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    all_systems = configs.c4(n_systems=args.systems)
    # the systems are independent: each rank solves its share (by N^3 cost), no data-path collective
    parts = shard_systems([q.n for q in all_systems], world)
    systems = [all_systems[i] for i in parts[rank]]
    sizes = [q.n for q in systems]
    eps = np.array([np.sqrt(q.gamma) for q in systems])
    C = pack_coords([q.coords for q in systems])
    B = pack_rhs([q.b for q in systems], 8)
    rng = np.random.default_rng(30)
    T = torch.from_numpy(rng.standard_normal(B.numel())).cuda()
    solver = BatchedRBFSolver(sizes, dim=2, nrhs=8, arith="df32")
    solver.load(C, eps, 1e-8)
    tune = solver.autotune()
    Bbuf, Xbuf = solver.build_graph(B, refine=2)
    flops = sum(n ** 3 / 3.0 for n in sizes)

    def step():
        solver.run_graph()
        G = 2.0 * (Xbuf - T)
        lam = solver.solve(G, refine=1)
        return solver.adjoint(Xbuf, lam)

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    for _ in range(max(3, args.warmup)):
        step()
    torch.cuda.synchronize()
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    clocks.start()
    from mpdok_gb300 import _native as NV
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    torch.cuda.synchronize()
    l0 = NV.launch_count()
    e0.record()
    for _ in range(args.steps):
        grads = step()
    e1.record()
    torch.cuda.synchronize()
    launches = NV.launch_count() - l0
    barrier()
    ck = clocks.stop()
    if solver.schedule == "dag":
        solver.dag_status()
    per = max_over_ranks(e0.elapsed_time(e1) / 1e3 / args.steps, device="cuda")
    # the graph step alone (assembly + factor + solve + 2 refinements), and the
    # level-scheduled factor alone for the roofline of the trailing update
    g0, g1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    g0.record()
    solver.run_graph()
    g1.record()
    torch.cuda.synchronize()
    t_graph = g0.elapsed_time(g1) / 1e3
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    f0.record()
    solver.factor()
    f1.record()
    torch.cuda.synchronize()
    t_factor = f0.elapsed_time(f1) / 1e3
    relres = solver.relres(B, Xbuf).cpu().numpy()
    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    fp32_peak = 128 * 2 * sms * 2.07e9 / 1e12        # nominal FP32 FMA rate at the maximum SM clock
    df_peak = fp32_peak / DF_FMA_OPS                  # FP64-equivalent flops of double-float multiply-adds
    ach = flops / t_factor / 1e12                     # Cholesky: sum n^3 / 3 flops
    # plain FP64 GPU solve: the vendor Cholesky per system (torch.linalg) + triangular solves
    base = None
    if not args.no_fp64_baseline and world == 1:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        worst = 0.0
        for q in systems:
            c = torch.from_numpy(q.coords).cuda()
            b = torch.from_numpy(np.asarray(q.b)).cuda()
            d2 = ((c[:, None, :] - c[None, :, :]) ** 2).sum(-1)
            A = torch.exp(-q.gamma * d2)
            A.diagonal().add_(q.reg)
            L = torch.linalg.cholesky(A)
            x = torch.cholesky_solve(b, L)
            worst = max(worst, float((torch.linalg.norm(b - A @ x, dim=0) / torch.linalg.norm(b, dim=0)).max()))
            del A, L
        torch.cuda.synchronize()
        base = {"seconds_factor_solve": time.perf_counter() - t0, "relres_max": worst,
                "method": "torch.linalg.cholesky + cholesky_solve (FP64, vendor library) per system, assembly inside"}
    cpu = None
    if not args.no_cpu and rank == 0 and world == 1:
        pick = list(range(0, len(systems), max(1, len(systems) // 12)))
        try:
            threads = len(os.sched_getaffinity(0))
        except AttributeError:
            threads = os.cpu_count() or 1
        env = dict(os.environ, OPENBLAS_NUM_THREADS=str(threads), OMP_NUM_THREADS=str(threads))
        out = subprocess.run([sys.executable, "-m", "oracle.cpu_baseline", "--config", "C4", "--systems",
                              ",".join(map(str, pick))], cwd=str(ROOT), env=env, capture_output=True, text=True,
                             timeout=1800)
        if out.returncode == 0:
            d = json.loads(out.stdout.strip().splitlines()[-1])
            scale = flops / d["flops"]
            cpu = {"value": d["seconds"] * scale, "unit": "s", "cores": threads, "kind": "port",
                   "sample": f"scipy cho_factor/cho_solve FP64 (8 RHS) on {len(pick)} of the {len(systems)} systems: "
                             f"{d['seconds']:.2f} s, x{scale:.1f} by sum n^3 (factor + solve only, no adjoint); "
                             f"relres max {d['relres_max']:.2e}"}
    h2d = C.numel() * 8 + B.numel() * 8
    line = {
        "metric": "C4 batched solve + adjoint time per step (256 Gaussian RBF systems, 8 RHS)", "value": per,
        "unit": "s", "n_gpus": world, "steps": args.steps, "warmup": max(3, args.warmup), "ms_per_step": per * 1e3,
        "higher_is_better": False, "scaling": "strong", "vs_baseline": None, "dtype": "f64 (double-float update)",
        "data": "synthetic (seeded NumPy, C4)",
        "config": {"workload": f"C4: {len(sizes)} systems, N in [{min(sizes)}, {max(sizes)}], sum N = {sum(sizes)}, "
                               "2-D uniform centres, eps~U(2,8), nugget 1e-8, 8 RHS; step = graph(factor + solve + "
                               "2 FP64 IR) + adjoint (solve + contraction)",
                   "l2": "inputs larger than L2 (A: %.1f GB FP64)" % (sum(n * n for n in sizes) * 8 / 1e9),
                   "schedule": solver.config, "autotune": tune, "graph_nodes": solver.graph_nodes,
                   "parallelism": f"{world} rank(s), systems sharded by N^3 (LPT), imbalance "
                                  f"{shard_imbalance([q.n for q in all_systems], parts):.3f}"},
        "relres_max": float(relres.max()), "relres_median": float(np.median(relres)),
        "factor_seconds": t_factor, "graph_step_seconds": t_graph,
        "roofline": {"bound": "fp32 pipe (double-float trailing update)", "achieved": ach,
                     "peak": df_peak, "unit": "TFLOP/s (FP64-equivalent)", "frac": ach / df_peak, "traffic": None,
                     "kernel": "batched Cholesky factor (k_bsyrk dominant)",
                     "peak_source": f"nominal FP32 FMA rate {fp32_peak:.1f} TFLOP/s / {DF_FMA_OPS} instructions "
                                    "per double-float multiply-add"},
        "fp64_gpu_baseline": base, "cpu_baseline": cpu,
        "e2e": None, "gpu_launches": launches, "clocks": ck,
        "gradient_norms": {"coords": float(grads[0].norm()), "eps": float(grads[1].norm()),
                           "reg": float(grads[2].norm())},
    }
    # end to end: host inputs -> device, graph, adjoint, gradients back to the host
    Ch = C.cpu().pin_memory()
    Bh = B.cpu().pin_memory()
    times = []
    for i in range(3):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        Cd = Ch.cuda(non_blocking=True)
        Bbuf.copy_(Bh, non_blocking=True)
        solver.load(Cd, eps, 1e-8)
        gr = step()
        out = [g.cpu() for g in gr] + [Xbuf.cpu()]
        torch.cuda.synchronize()
        if i > 0:
            times.append(time.perf_counter() - t0)
    line["e2e"] = {"value": max_over_ranks(sum(times) / len(times), device="cuda"), "unit": "s",
                   "h2d_bytes_per_step": h2d,
                   "d2h_bytes_per_step": sum(o.numel() * 8 for o in out),
                   "api": "BatchedRBFSolver.load + run_graph + solve + adjoint from pinned host coords/B"}
    if rank == 0 and emit:
        print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return line


def bench_ooc(args, emit: bool = True) -> dict:
    """C5 layout: FP32 A in pinned host RAM in 16384-row tiles (or a raw file),
    streamed per product; reported against the pinned host->device copy rate
    measured in the same run, next to the matrix-free in-HBM product."""
    import numpy as np
    import torch
    from mpdok_gb300.matfree import MatrixFreeOperator
    from mpdok_gb300.mpdok_ooc import MPDOKOOCSolver
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    n = args.n
    rng = np.random.default_rng(4)
    X = rng.uniform(0.0, 1.0, size=(n, 3))
    # host link: one pinned 1 GiB buffer -> device
    hb = torch.empty(1 << 28, dtype=torch.float32).pin_memory()
    db = torch.empty_like(hb, device="cuda")
    for _ in range(3):
        db.copy_(hb, non_blocking=True)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(5):
        db.copy_(hb, non_blocking=True)
    e1.record()
    torch.cuda.synchronize()
    link = hb.numel() * 4 * 5 / (e0.elapsed_time(e1) / 1e3) / 1e9
    del hb, db
    s = MPDOKOOCSolver(tile_rows=min(16384, n))
    s.build(X, gamma=100.0, reg=1e-6, store="ram", verbose=False)
    v = torch.randn(n, device="cuda")
    for _ in range(max(3, args.warmup)):
        s._tiled_sgemv(v)
    torch.cuda.synchronize()
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    clocks.start()
    e0.record()
    for _ in range(args.steps):
        y = s._tiled_sgemv(v)
    e1.record()
    torch.cuda.synchronize()
    ck = clocks.stop()
    ms = e0.elapsed_time(e1) / args.steps
    gbs = 4.0 * n * n / (ms / 1e3) / 1e9
    s.free()
    op = MatrixFreeOperator(X, gamma=100.0, reg=1e-6)
    for _ in range(3):
        op.matvec(v)
    torch.cuda.synchronize()
    e0.record()
    for _ in range(args.steps):
        op.matvec(v)
    e1.record()
    torch.cuda.synchronize()
    mf_ms = e0.elapsed_time(e1) / args.steps
    import tempfile
    ssd = None
    tmpdir = tempfile.mkdtemp(prefix="mpdok_ooc_")
    path = Path(tmpdir) / "ooc_store.bin"
    try:
        n2 = min(n, 16384)
        s2 = MPDOKOOCSolver(tile_rows=2048)
        s2.build(X[:n2], gamma=100.0, reg=1e-6, store="ssd", path=str(path), verbose=False)
        v2 = torch.randn(n2, device="cuda")
        s2._tiled_sgemv(v2)
        torch.cuda.synchronize()
        e0.record()
        for _ in range(3):
            s2._tiled_sgemv(v2)
        e1.record()
        torch.cuda.synchronize()
        ssd = {"n": n2, "ms": e0.elapsed_time(e1) / 3, "GBs": 4.0 * n2 * n2 / (e0.elapsed_time(e1) / 3e3) / 1e9,
               "note": "raw row-major FP32 file read by 8 pread threads into pinned staging (page cache warm)"}
        s2.free()
    finally:
        if path.exists():
            path.unlink()
        os.rmdir(tmpdir)
    line = {"metric": "OOC streamed FP32 matvec rate (C5 layout, pinned host RAM store)", "value": gbs, "unit": "GB/s",
            "n_gpus": 1, "steps": args.steps, "warmup": max(3, args.warmup), "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded NumPy, C5 centres)",
            "config": {"workload": f"C5 layout at N={n}: Gaussian eps=10 (gamma=100), 3-D uniform seed 4, nugget 1e-6, "
                                   f"FP32 store {4.0 * n * n / 1e9:.1f} GB, 16384-row tiles; step = one streamed "
                                   "product y = A v", "l2": "store far larger than L2"},
            "roofline": {"bound": "host link (pinned H2D)", "achieved": gbs, "peak": link, "unit": "GB/s",
                         "frac": gbs / link, "traffic": 4.0 * n * n,
                         "peak_source": "pinned 1 GiB host->device copy measured in this run"},
            "matrix_free_in_hbm_ms": mf_ms, "streamed_over_matrix_free": ms / mf_ms, "ssd_store": ssd,
            "cpu_baseline": None, "e2e": None, "gpu_launches": None, "clocks": ck}
    if emit:
        print(json.dumps(line))
    return line


def bench_c2(args, emit: bool = True) -> dict:
    """C2 as specified: N=20000 Gaussian, 3-D, eps=5, nugget 1e-6, 4 RHS, through
    the CG path the configuration names.  Its kappa (~1e8) puts every FP32 CG
    body and every 16/32-bit factorization out of reach (kappa * u > 1), so the
    CG-IR runs PCG with FP64 inner vectors, the split (Ozaki-style two-slice
    FP32) operator for every product and the FP64-accurate double-float
    Cholesky as the preconditioner.  One step = assemble A + split it +
    Cholesky (batch plan of one) + CG-IR to the FP64 floor.  Reported with the
    FP64 vendor Cholesky solve and the direct double-float refinement."""
    import numpy as np
    import torch
    from mpdok_gb300 import configs
    from mpdok_gb300.batch import BatchedRBFSolver, CholeskyPreconditioner, pack_rhs, unpack_rhs
    from mpdok_gb300.dense_krylov import DenseLinearOperator, cg_ir
    from mpdok_gb300.rbf_kernel import assemble
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    c2 = configs.c2()
    B = np.asarray(c2.b)
    Bd = torch.from_numpy(np.asfortranarray(B)).cuda()
    n = c2.n
    info = {}

    def step():
        A = assemble(c2.coords, gamma=c2.gamma, reg=c2.reg, dtype=torch.float64)
        op = DenseLinearOperator(A, verbose=False)
        pc = CholeskyPreconditioner(c2.coords, eps=5.0, reg=c2.reg, nrhs=4)
        X, hist, conv = cg_ir(op, Bd, tol=1e-12, maxiter_outer=6, inner_tol=1e-10, inner_maxiter=4, split=True,
                              precond=pc)
        info.update(hist=hist, conv=conv)
        return X, A

    for _ in range(max(1, args.warmup)):
        step()
    torch.cuda.synchronize()
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    clocks.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        Xd, A = step()
    e1.record()
    torch.cuda.synchronize()
    ck = clocks.stop()
    per = e0.elapsed_time(e1) / 1e3 / args.steps
    R = Bd - A @ Xd
    rel = (torch.linalg.norm(R, dim=0) / torch.linalg.norm(Bd, dim=0)).cpu().numpy()
    # the same system by the plan's direct double-float Cholesky + FP64 refinement
    s = BatchedRBFSolver([n], dim=3, nrhs=4, grid_mult=2)
    s.load([c2.coords], [5.0], c2.reg)
    Bp = pack_rhs([B], 4)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    s.factor()
    Xp = s.solve(Bp, refine=3)
    torch.cuda.synchronize()
    t_direct = time.perf_counter() - t0
    rel_direct = float(s.relres(Bp, Xp).max())
    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    df_peak = 128 * 2 * sms * 2.07e9 / 1e12 / DF_FMA_OPS
    base = None
    if not args.no_fp64_baseline:
        c = torch.from_numpy(c2.coords).cuda()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        d2 = ((c[:, None, :] - c[None, :, :]) ** 2).sum(-1)
        Ab = torch.exp(-c2.gamma * d2)
        Ab.diagonal().add_(c2.reg)
        L = torch.linalg.cholesky(Ab)
        x = torch.cholesky_solve(Bd, L)
        torch.cuda.synchronize()
        tb = time.perf_counter() - t0
        relb = float((torch.linalg.norm(Bd - Ab @ x, dim=0) / torch.linalg.norm(Bd, dim=0)).max())
        err = float(torch.linalg.norm(Xd - x) / torch.linalg.norm(x))
        base = {"seconds": tb, "relres_max": relb, "mine_err_vs_fp64": err,
                "method": "torch.linalg.cholesky + cholesky_solve FP64 (assembly inside)"}
        del Ab, L, d2
    line = {"metric": "C2 SPD solve to the FP64 floor through CG-IR, 4 RHS (N=20000, 3-D Gaussian eps=5, nugget 1e-6)",
            "value": per, "unit": "s", "n_gpus": 1, "steps": args.steps, "warmup": max(1, args.warmup),
            "ms_per_step": per * 1e3, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64 vectors, split FP32 products, double-float Cholesky preconditioner",
            "data": "synthetic (seeded NumPy, C2)",
            "config": {"workload": "C2: N=20000 uniform [0,1]^3 seed 1, eps=5, nugget 1e-6, B 20000 x 4 N(0,1); "
                                   "step = assemble + split + Cholesky (preconditioner) + CG-IR (PCG, split "
                                   "operator, FP64 residual / update); tol 1e-12 is below the FP64 floor of this "
                                   "system, the solve stops at the floor", "l2": "A 3.2 GB > L2"},
            "relres_max": float(rel.max()), "relres_by_rhs": [float(v) for v in rel], "converged": info.get("conv"),
            "history": info.get("hist"),
            "direct_refinement": {"seconds": t_direct, "relres_max": rel_direct,
                                  "method": "double-float Cholesky + 3 FP64 refinement steps (no CG)"},
            "roofline": {"bound": "fp32 pipe (double-float Cholesky of the preconditioner)",
                         "achieved": n ** 3 / 3.0 / per / 1e12, "peak": df_peak,
                         "unit": "TFLOP/s (FP64-equivalent)", "frac": n ** 3 / 3.0 / per / 1e12 / df_peak,
                         "traffic": None, "note": "whole step against the Cholesky's flops"},
            "fp64_gpu_baseline": base, "cpu_baseline": None, "e2e": None, "gpu_launches": None, "clocks": ck}
    if emit:
        print(json.dumps(line))
    return line


REF_OOC_SOLVE_32K_S = 45.0  # published: OOC-RAM GMRES-IR N=32768, build + solve, RTX 4060 (rbf_streaming_demo.ipynb)


def bench_ooc_solve(args, emit: bool = True) -> dict:
    """The reference's out-of-core demo at N=32768: 2-D points in [0,100]^2
    (seed 42), moving-front RHS, estimated gamma, nugget 1e-2, tol 1e-5,
    4096-row tiles in pinned host RAM, GMRES(50)-IR with up to 20 outer steps
    (matrix-free FP64 residual).  One step = build the store + solve."""
    import numpy as np
    import torch
    from mpdok_gb300.mpdok_ooc import MPDOKOOCSolver
    from mpdok_gb300.rbf_kernel import _estimate_gamma, synthetic_coords, weather_front
    from oracle import krylov_ref as O
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    n = 32768
    coords = synthetic_coords(n, seed=42)
    b = weather_front(coords, t=0)
    gamma = float(_estimate_gamma(coords))
    s = MPDOKOOCSolver(tile_rows=4096)

    def step():
        t0 = time.perf_counter()
        s.build(coords, gamma=gamma, reg=1e-2, store="ram", verbose=False)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        x = s.solve(b, tol=1e-5, maxiter_outer=20, restart=50, verbose=False)
        torch.cuda.synchronize()
        return x, t1 - t0, time.perf_counter() - t1

    for _ in range(max(1, min(args.warmup, 1))):
        step()
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    clocks.start()
    tb, ts = [], []
    for _ in range(args.steps):
        x, a, c = step()
        tb.append(a)
        ts.append(c)
    ck = clocks.stop()
    info = s.last_info
    moved = s.bytes_moved()
    s.free()
    per = (sum(tb) + sum(ts)) / args.steps
    hist = info.history_list()
    # relres in FP64 against the recomputed operator (matrix-free, on the device)
    from mpdok_gb300.matfree import MatrixFreeOperator
    op = MatrixFreeOperator(coords, gamma=gamma, reg=1e-2)
    rel = op.residual_norm(x, b) / float(torch.linalg.norm(b))
    line = {"metric": "OOC GMRES-IR build + solve to relres 1e-5 (N=32768, FP32 store in pinned host RAM)",
            "value": per, "unit": "s", "n_gpus": 1, "steps": args.steps, "warmup": 1, "ms_per_step": per * 1e3,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": per / REF_OOC_SOLVE_32K_S,
            "dtype": "f32 store + f64 residual", "data": "synthetic (seeded NumPy points, moving-front RHS)",
            "config": {"workload": f"N={n} uniform [0,100]^2 seed 42, Gaussian gamma={gamma:.3e} (estimated), "
                                   "nugget 1e-2, tol 1e-5, GMRES(50)-IR, <= 20 outer, 4096-row tiles (8 tiles, "
                                   "4.3 GB store)", "baseline_hardware": "published 45 s on an RTX 4060 + PCIe 4"},
            "build_seconds": sum(tb) / args.steps, "solve_seconds": sum(ts) / args.steps,
            "relres": rel, "outer_iters": int(info.outer_iters), "history": hist,
            "streamed_GB_per_solve": moved / 1e9,
            "roofline": {"bound": "host link (pinned H2D)", "achieved": moved / max(ts[-1], 1e-9) / 1e9,
                         "peak": None, "unit": "GB/s", "frac": None, "traffic": None,
                         "note": "bytes streamed over the solve time (compare with the --only ooc line's link rate)"},
            "cpu_baseline": None, "e2e": None, "gpu_launches": None, "clocks": ck}
    if emit:
        print(json.dumps(line))
    return line


REF_FACTOR_ONCE_72_S = 0.791  # published: LU-IR factor once + 72 solves, N=8192, RTX 4060 (rbf_demo.ipynb:247)


def bench_multi_rhs(args, emit: bool = True) -> dict:
    """Factor once, solve 72 right-hand sides (3 fields x 24 steps), N=8192,
    nugget 1e-2, tol 1e-5, <= 3 refinement steps: the reference's time-series
    workload.  One step = FP32 LU of A + LU-IR of all 72 columns (8 per
    triangular sweep), A resident in HBM."""
    import numpy as np
    import torch
    from mpdok_gb300 import configs
    from mpdok_gb300.lu import LUFactorization
    from mpdok_gb300.mpdok_ops import LUIRSolver
    from mpdok_gb300.rbf_kernel import _estimate_gamma, assemble
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    n = 8192
    X, Bh = configs.time_series_fields(n=n)
    gamma = float(_estimate_gamma(torch.from_numpy(X).cuda()))
    A = assemble(X, gamma=gamma, reg=1e-2, dtype=torch.float64)
    B = torch.from_numpy(np.asfortranarray(Bh)).cuda()
    tol = 1e-5

    def step():
        lu = LUFactorization(A, dtype="fp32")
        Xs, info = lu.solve_ir_many(A, B, tol=tol, maxiter_outer=3)
        return Xs, info, lu

    for _ in range(max(3, args.warmup)):
        step()
    torch.cuda.synchronize()
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    clocks.start()
    l0 = __import__("mpdok_gb300._native", fromlist=["x"]).launch_count()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        Xs, info, lu = step()
    e1.record()
    torch.cuda.synchronize()
    ck = clocks.stop()
    launches = __import__("mpdok_gb300._native", fromlist=["x"]).launch_count() - l0
    per = e0.elapsed_time(e1) / 1e3 / args.steps
    Xh = Xs.cpu().numpy()
    A64 = A.cpu().numpy()
    rel = np.linalg.norm(Bh - A64 @ Xh, axis=0) / np.linalg.norm(Bh, axis=0)
    # the drop-in path: LUIRSolver.factor + 72 x solve_factored (the reference's calls, one RHS each)
    dropin = LUIRSolver()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    dropin.factor(A)
    for j in range(Bh.shape[1]):
        dropin.solve_factored(B[:, j].contiguous(), tol=tol, maxiter_outer=3)
    torch.cuda.synchronize()
    t_dropin = time.perf_counter() - t0
    dropin.free_factored()
    # CPU: SciPy FP64 LU once + 72 lu_solve, all host threads
    cpu = None
    if not args.no_cpu:
        try:
            threads = len(os.sched_getaffinity(0))
        except AttributeError:
            threads = os.cpu_count() or 1
        code = ("import numpy as np, scipy.linalg as sl, time, json, sys; sys.path.insert(0, '.');"
                "from oracle.krylov_ref import rbf_matrix; from mpdok_gb300 import configs;"
                f"X, B = configs.time_series_fields(n={n}); A = rbf_matrix(X, gamma={gamma!r}, reg=1e-2);"
                "t0 = time.perf_counter(); lu = sl.lu_factor(A, check_finite=False);"
                "x = sl.lu_solve(lu, B, check_finite=False); t = time.perf_counter() - t0;"
                "print(json.dumps({'seconds': t}))")
        env = dict(os.environ, OPENBLAS_NUM_THREADS=str(threads), OMP_NUM_THREADS=str(threads))
        out = subprocess.run([sys.executable, "-c", code], cwd=str(ROOT), env=env, capture_output=True, text=True,
                             timeout=1800)
        if out.returncode == 0:
            d = json.loads(out.stdout.strip().splitlines()[-1])
            cpu = {"value": d["seconds"], "unit": "s", "cores": threads, "kind": "port",
                   "sample": f"scipy lu_factor once + lu_solve of all 72 columns, FP64, N={n} (full workload)"}
    line = {
        "metric": "factor once + 72 RHS solves to relres 1e-5 (N=8192 RBF time series)", "value": per, "unit": "s",
        "n_gpus": 1, "steps": args.steps, "warmup": max(3, args.warmup), "ms_per_step": per * 1e3,
        "higher_is_better": False, "scaling": "weak", "vs_baseline": per / REF_FACTOR_ONCE_72_S,
        "dtype": "f32 factors + f64 refinement", "data": "synthetic (seeded NumPy time-series fields)",
        "config": {"workload": f"N={n} sensors uniform in [0,100]^2 (seed 42), Gaussian gamma={gamma:.3e} "
                               "(estimated), nugget 1e-2, 3 fields x 24 steps = 72 RHS, tol 1e-5, <= 3 IR steps; "
                               "step = FP32 LU + multi-RHS LU-IR (8 columns per triangular sweep)",
                   "l2": "A64 537 MB > L2", "baseline_hardware": "published 0.791 s on an RTX 4060"},
        "relres_max": float(rel.max()), "converged": bool(info["converged"]),
        "dropin_per_rhs_seconds": t_dropin,
        "roofline": None, "cpu_baseline": cpu, "e2e": None, "gpu_launches": launches, "clocks": ck,
    }
    if emit:
        print(json.dumps(line))
    return line


REF_FULL_STEPS = 2  # full-size SciPy solves the reference arm times (about 50 s each on 16 Arm cores)


def headline_config(n: int, world: int) -> dict:
    """The workload both arms measure (identical dicts, so the two lines compare like for like)."""
    return {"workload": f"HEADLINE: Gaussian RBF N={n}, 2-D stratified jitter seed 2, eps=40 (gamma=1600), "
                        f"nugget 1e-2, b~N(0,1); tol 1e-12; one step = one full solve from x = 0 "
                        f"(A resident in memory, assembly excluded)",
            "l2": "inputs larger than L2 (A64 8.6 GB, A32 4.3 GB)", "parallelism": f"replicas x{world}"}


def run_reference(args):
    """--impl reference: the reference's CPU path for this workload (SciPy FP64
    lu_factor / lu_solve + FP64 refinement, the path of rbf_demo.ipynb) on all
    host threads, rank 0 only.  Every timed step is one full solve of the
    N=32768 headline system itself: no sample, no scaling.  A full solve takes
    about a minute on the host cores, so the arm times min(steps, 2) of them
    after one small warm-up solve, and reports the count it timed."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    n = args.n
    k = max(1, min(args.steps, REF_FULL_STEPS))
    d = cpu_lu_sample(n, k, warmup_n=2048)
    secs = d["seconds"]
    per = sum(secs) / len(secs)
    world = int(os.environ.get("WORLD_SIZE", "1"))
    line = {
        "impl": "reference", "metric": HEADLINE_METRIC, "value": per, "unit": UNIT, "n_gpus": args.gpus,
        "steps": len(secs), "steps_requested": args.steps, "warmup": 1, "ms_per_step": per * 1e3,
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded NumPy, HEADLINE system)",
        "config": headline_config(n, world),
        "timed_solves_seconds": secs, "relres": d["relres"], "host_assembly_seconds": d.get("assembly_seconds"),
        "cpu_baseline": {"value": per, "unit": UNIT, "cores": d["threads"], "kind": "port",
                         "sample": f"the full N={n} headline system: scipy lu_factor/lu_solve FP64 + refinement, "
                                   f"{len(secs)} timed solve(s) after one N=2048 warm-up solve; relres "
                                   f"{d['relres']:.2e}"},
        "e2e": {"value": per, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def bench_hard(args, emit: bool = True) -> dict:
    """The headline centres with C5's nugget (1e-6, kappa >= 1e6) and a smooth
    right-hand side: each factor type (FP16, BF16, FP32) preconditioning the
    three-precision GMRES-IR, against the plain FP64 GPU solve of the same
    system.  Reports, per factor type, whether it reached relres 1e-12, its
    outer / inner iterations and its time."""
    import numpy as np
    import torch
    from mpdok_gb300 import configs
    from mpdok_gb300.rbf_kernel import assemble
    from mpdok_gb300.solvers import MixedSolver, fp64_gpu_solve
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    sysm = configs.hard_headline(n=args.n)
    n = sysm.n
    A = assemble(sysm.coords, gamma=sysm.gamma, reg=sysm.reg, kernel=sysm.kernel, dtype=torch.float64)
    b = torch.from_numpy(np.asarray(sysm.b)).cuda()
    fp64 = fp64_gpu_solve(A, b, tol=sysm.tol)
    outcomes = {}
    best = None
    for fd in ("fp16", "bf16", "fp32"):
        sv = MixedSolver(factor_dtype=fd, maxiter_outer=20)
        import warnings
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            for _ in range(max(1, args.warmup)):
                sv.solve(A, b, tol=sysm.tol)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(args.steps):
                x, info = sv.solve(A, b, tol=sysm.tol)
            e1.record()
            torch.cuda.synchronize()
        sec = e0.elapsed_time(e1) / 1e3 / args.steps
        err = float(torch.linalg.norm(x - fp64["x"]) / torch.linalg.norm(fp64["x"]))
        outcomes[fd] = {"seconds": sec, "converged": bool(info["converged"]), "relres": info["relres"],
                        "outer_iters": info["outer_iters"], "inner_iters": info["inner_iters"],
                        "perturbed_pivots": info.get("perturbed_pivots"), "err_vs_fp64_lu": err,
                        "factor_ms": info.get("factor_ms"), "refine_ms": info.get("refine_ms"),
                        "speedup_vs_fp64_gpu": fp64["seconds"] / sec}
        if info["converged"] and (best is None or sec < outcomes[best]["seconds"]):
            best = fd
        del sv
        torch.cuda.empty_cache()
    line = {"metric": "time to FP64 relres<=1e-12 on the hard family (N=32768 Gaussian, nugget 1e-6)",
            "value": outcomes[best]["seconds"] if best else None, "unit": "s", "steps": args.steps,
            "warmup": max(1, args.warmup), "higher_is_better": False, "dtype": "f32+f64 (mixed)",
            "config": {"workload": f"HARD: the headline's N={n} stratified-jitter centres, Gaussian eps="
                                   f"{configs.HARD_EPS:g}, nugget 1e-6, b = sin(2 pi x1) cos(2 pi x2); tol 1e-12; "
                                   "one step = one full solve (factor + GMRES(30)-IR), A in HBM"},
            "fastest_converged_factor": best, "by_factor": outcomes,
            "fp64_gpu_baseline": {"seconds": fp64["seconds"], "relres": fp64["relres"], "method": fp64["method"]},
            "speedup_vs_fp64_gpu": (fp64["seconds"] / outcomes[best]["seconds"]) if best else None}
    del A
    if emit:
        print(json.dumps(line))
    return line


def run_extras(args) -> dict:
    """Each secondary configuration once, with short step counts, as dicts for
    the headline line: C2, C4 (batched + adjoint), the hard headline family,
    out-of-core (streamed matvec at N=100000 and the reference's N=32768 OOC
    solve) and factor-once / many-RHS.  A failure is recorded, not raised."""
    import argparse as _ap
    import torch
    out = {}
    plan = (("hard_headline", bench_hard, dict(steps=2, warmup=1)),
            ("c2", bench_c2, dict(steps=2, warmup=1)),
            ("c4_batch_adjoint", bench_batch, dict(steps=2, warmup=1, systems=256)),
            ("ooc_matvec", bench_ooc, dict(steps=3, warmup=1, n=100000)),
            ("ooc_solve", bench_ooc_solve, dict(steps=1, warmup=1)),
            ("multi_rhs", bench_multi_rhs, dict(steps=3, warmup=1)))
    for name, fn, over in plan:
        a = _ap.Namespace(**dict(vars(args), **over))
        t0 = time.perf_counter()
        try:
            line = fn(a, emit=False)
            line = {k: v for k, v in line.items() if k not in ("n_gpus", "scaling", "data")}
            line["wall_seconds"] = time.perf_counter() - t0
            out[name] = line
        except Exception as e:  # noqa: BLE001
            out[name] = {"error": f"{type(e).__name__}: {e}"[:400], "wall_seconds": time.perf_counter() - t0}
        torch.cuda.synchronize()
        torch.cuda.empty_cache()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="mine", choices=["mine", "reference"])
    ap.add_argument("--n", type=int, default=32768)
    ap.add_argument("--no-extras", action="store_true",
                    help="headline only: skip the once-each lines of the other configurations")
    ap.add_argument("--no-fp64-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--only", default="headline",
                    choices=["headline", "gemv", "update", "batch", "ooc", "ooc_solve", "multi_rhs", "c2", "hard"],
                    help="gemv: only the standalone stored-matrix GEMV measurement (used for kernel profiles); "
                         "update: only the standalone first far update of the factorization at --n; "
                         "batch: the batched C4 solve + adjoint line; ooc: the out-of-core C5 streaming line")
    ap.add_argument("--systems", type=int, default=256, help="--only batch: number of C4 systems")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.only == "gemv":
        import torch
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        print(json.dumps(gemv_standalone(args.n, max(3, args.warmup), max(5, args.steps))))
        return 0
    if args.only == "update":
        import torch
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        print(json.dumps(update_standalone(args.n, max(1, args.warmup), max(3, args.steps))))
        return 0
    if args.only == "batch":
        bench_batch(args)
        return 0
    if args.only == "ooc":
        bench_ooc(args)
        return 0
    if args.only == "multi_rhs":
        bench_multi_rhs(args)
        return 0
    if args.only == "c2":
        bench_c2(args)
        return 0
    if args.only == "hard":
        bench_hard(args)
        return 0
    if args.only == "ooc_solve":
        bench_ooc_solve(args)
        return 0

    import numpy as np
    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    from mpdok_gb300 import _native as NV
    from mpdok_gb300 import configs
    from mpdok_gb300.solvers import MixedSolver, fp64_gpu_solve
    from mpdok_gb300.rbf_kernel import assemble

    sysm = configs.headline(n=args.n)
    n = sysm.n
    b = torch.from_numpy(np.asarray(sysm.b)).cuda()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    A = assemble(sysm.coords, gamma=sysm.gamma, reg=sysm.reg, kernel=sysm.kernel, dtype=torch.float64)
    torch.cuda.synchronize()
    t_asm = time.perf_counter() - t0

    solver = MixedSolver()
    solver_desc = solver.describe()
    for _ in range(args.warmup):
        x, info = solver.solve(A, b, tol=sysm.tol)
    torch.cuda.synchronize()
    barrier()

    NV.profile_enable(True)
    l0 = NV.launch_count()
    clocks = ClockSampler(local)
    clocks.start()
    stream = torch.cuda.current_stream()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    torch.cuda.synchronize()
    ev0.record(stream)
    infos = []
    for _ in range(args.steps):
        x, info = solver.solve(A, b, tol=sysm.tol)
        infos.append(info)
    ev1.record(stream)
    torch.cuda.synchronize()
    barrier()
    ck = clocks.stop()
    launches = NV.launch_count() - l0
    total_ms = ev0.elapsed_time(ev1)
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([total_ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    per_s = total_ms / 1e3 / args.steps
    prof, skipped, prof_bytes = {}, {}, {}
    for name, cls in (("gemv_f32", NV.PROF_GEMV_F32), ("gemv_f64", NV.PROF_GEMV_F64), ("lu_gemm", NV.PROF_LU_GEMM),
                      ("lu_gemm_deep", NV.PROF_LU_GEMM_DEEP), ("trsv", NV.PROF_TRSV), ("lu_panel", NV.PROF_LU_PANEL)):
        ms, cnt, work = NV.profile_query(cls)
        prof[name] = (ms, cnt, work)
        skipped[name] = NV.profile_skipped(cls)
        prof_bytes[name] = NV.profile_bytes(cls)
    NV.profile_enable(False)

    hbm, bf16, bf16s, peak_kind = _peaks()
    traffic = _traffic_model()
    share = {k: v[0] / max(1e-9, total_ms) for k, v in prof.items()}
    rooflines = {}
    for name, (ms, cnt, work) in prof.items():
        if cnt == 0 or ms <= 0:
            continue
        if name in ("lu_gemm", "lu_gemm_deep"):
            # K <= 1024 with an FP32 C read and written: 2K / 8 <= 256 flop per byte, at or below
            # the ridge point (sustained bf16 peak / HBM ~ 253), so the binding roofline is
            # normally HBM; the other view is kept beside it
            tflops = work / (ms / 1e3) / 1e12
            byts = prof_bytes[name]
            gbs = byts / (ms / 1e3) / 1e9
            ai = work / max(byts, 1.0)
            tr = None
            if name == "lu_gemm_deep" and traffic.get("lu_gemm_bytes_per_byte"):
                # measured on the warp-specialised kernel; the other class has no capture
                tr = traffic["lu_gemm_bytes_per_byte"] * byts / cnt
            hv = {"bound": "hbm", "achieved": gbs, "peak": hbm, "unit": "GB/s", "frac": gbs / hbm,
                  "peak_source": f"{peak_kind} HBM copy"}
            tv = {"bound": "tensor", "achieved": tflops, "peak": bf16s, "unit": "TFLOP/s", "frac": tflops / bf16s,
                  "peak_source": f"{peak_kind} bf16 dense, sustained"}
            main, other = (tv, hv) if ai * hbm / 1e3 >= bf16s else (hv, tv)
            rooflines[name] = dict(main, traffic=tr, launches=cnt, avg_launch_ms=ms / cnt,
                                   work_per_launch=byts / cnt, flops_per_launch=work / cnt,
                                   arithmetic_intensity_flop_per_byte=ai,
                                   **{("tensor_view" if other is tv else "hbm_view"):
                                      {k: other[k] for k in ("achieved", "peak", "unit", "frac", "peak_source")}})
        elif name in ("gemv_f32", "gemv_f64", "trsv"):
            ach = work / (ms / 1e3) / 1e9
            tr = None
            key = f"{name}_bytes_per_byte"
            if traffic.get(key):
                tr = traffic[key] * work / cnt
            rooflines[name] = {"bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s", "frac": ach / hbm,
                               "traffic": tr, "launches": cnt, "avg_launch_ms": ms / cnt,
                               "work_per_launch": work / cnt, "skipped_launches": skipped[name],
                               "peak_source": f"{peak_kind} HBM copy"}
    dom = max((k for k in rooflines), key=lambda k: prof[k][0]) if rooflines else None
    roof = dict(rooflines[dom], kernel=dom) if dom else None
    if roof and dom in KERNEL_NAMES:
        roof["kernel_name"] = KERNEL_NAMES[dom]
    # both update kernels together: every trailing-update flop of the factorization over the
    # summed per-launch device time (launches on different streams overlap, so this is a
    # per-launch average, not a share of the step)
    up_ms = prof["lu_gemm"][0] + prof["lu_gemm_deep"][0]
    up_work = prof["lu_gemm"][2] + prof["lu_gemm_deep"][2]
    if up_ms > 0:
        tf = up_work / (up_ms / 1e3) / 1e12
        rooflines["lu_update_all"] = {"bound": "tensor", "achieved": tf, "peak": bf16s, "unit": "TFLOP/s",
                                      "frac": tf / bf16s, "launches": prof["lu_gemm"][1] + prof["lu_gemm_deep"][1],
                                      "peak_source": f"{peak_kind} bf16 dense, sustained"}

    # accuracy of the timed solves
    xs = x
    relres = infos[-1]["relres"]

    fp64 = None
    if not args.no_fp64_baseline and rank == 0:
        fp64 = fp64_gpu_solve(A, b, tol=sysm.tol)
        err = float(torch.linalg.norm(xs - fp64["x"]) / torch.linalg.norm(fp64["x"]))
        fp64 = {"seconds": fp64["seconds"], "relres": fp64["relres"], "method": fp64["method"],
                "mixed_err_vs_fp64_lu": err, "speedup_mixed_vs_fp64": fp64["seconds"] / per_s}

    e2e = None
    if not args.no_e2e:
        A_host = torch.empty_strided((n, n), (1, n), dtype=torch.float64, pin_memory=True)
        A_host.copy_(A.cpu())
        b_host = torch.from_numpy(np.asarray(sysm.b)).pin_memory()
        times, parts = [], []
        for i in range(5 + 1):  # one untimed, five timed: the host link is shared, so a median of five
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            xe, _ = solver.solve(A_host, b_host, tol=sysm.tol)
            xh = xe.cpu()
            torch.cuda.synchronize()
            if i > 0:
                times.append(time.perf_counter() - t0)
                parts.append(dict(solver.last_timing))
        # the upload alone (A straight into its device buffer with the FP32
        # copy made per block), against a plain pinned 1 GiB host -> device copy
        from mpdok_gb300._device import fortran_empty, upload_fortran
        a32 = fortran_empty(n, n, torch.float32)
        u0, u1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        u0.record()
        Ad = upload_fortran(A_host, out32=a32)
        u1.record()
        torch.cuda.synchronize()
        up_s = u0.elapsed_time(u1) / 1e3
        del Ad, a32
        hb = torch.empty(1 << 27, dtype=torch.float64).pin_memory()
        db = torch.empty_like(hb, device="cuda")
        db.copy_(hb, non_blocking=True)
        torch.cuda.synchronize()
        u0.record()
        for _ in range(3):
            db.copy_(hb, non_blocking=True)
        u1.record()
        torch.cuda.synchronize()
        link = 3 * hb.numel() * 8 / (u0.elapsed_time(u1) / 1e3) / 1e9
        del hb, db, A_host
        # the median step: the host link is shared with other jobs on the box,
        # and one step in a few meets a busy link (every step is listed)
        e2e = {"value": float(np.median(times)), "unit": UNIT, "h2d_bytes_per_step": 8 * n * n + 8 * n,
               "statistic": "median of the timed steps",
               "d2h_bytes_per_step": 8 * n, "api": "mpdok_gb300.solvers.MixedSolver.solve(host A, host b)",
               "steps_seconds": times, "breakdown_ms": parts,
               "upload_seconds": up_s, "upload_GBs": 8.0 * n * n / up_s / 1e9, "pinned_h2d_GBs": link,
               "upload_frac_of_pinned_copy": 8.0 * n * n / up_s / 1e9 / link}

    gemv_sa = gemv_standalone(n, 3, 10) if rank == 0 else None
    update_sa = update_standalone(n, 1, 3) if rank == 0 else None

    # every other configuration once (not per step), so that the default
    # line carries them; each is a complete measurement of its own workload
    extras = {}
    if not args.no_extras and rank == 0 and world == 1:
        del A
        solver = None
        torch.cuda.empty_cache()
        extras = run_extras(args)

    # the reference's CPU path on the full headline system, after all GPU work
    cpu = None
    if not args.no_cpu and rank == 0 and world == 1:
        try:
            d = cpu_lu_sample(n, 1, warmup_n=2048)
            cpu = {"value": d["seconds"][0], "unit": UNIT, "cores": d["threads"], "kind": "port",
                   "sample": f"the full N={n} headline system: scipy lu_factor/lu_solve FP64 + refinement, one "
                             f"timed solve after an N=2048 warm-up solve; relres {d['relres']:.2e}",
                   "relres": d["relres"]}
        except Exception as e:  # noqa: BLE001
            cpu = {"value": None, "unit": UNIT, "cores": None, "kind": "port", "sample": f"failed: {e}"}

    line = {
        "metric": HEADLINE_METRIC, "value": per_s, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": per_s * 1e3, "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+f64 (mixed)", "data": "synthetic (seeded NumPy, HEADLINE system)",
        "config": headline_config(n, world), "solver": solver_desc, "assembly_s": t_asm,
        "relres": relres, "solve_info": infos[-1], "fp64_gpu_baseline": fp64,
        "roofline": roof, "gemv_roofline": rooflines.get("gemv_f32"), "gemv_standalone": gemv_sa,
        "update_standalone": update_sa,
        "rooflines": rooflines,
        "kernel_time_share": share, "cpu_baseline": cpu, "e2e": e2e,
        "gpu_launches": launches, "clocks": ck, "configs": extras,
    }
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
