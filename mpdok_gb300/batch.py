"""Batched RBF solves with gradients: many systems of uneven N, several RHS each.

``BatchedRBFSolver(sizes, dim, nrhs)`` owns one plan of ``libmpdok_gb300``:
FP64 storage for every A_s = phi(eps_s ||c_i - c_j||) + reg_s I, a batched
Cholesky on 64 x 64 tiles (double-float trailing update), FP64 triangular
solves and FP64 refinement.  Two schedules run the same tile arithmetic:
``levels`` (three launches per block level over every active system, a
persistent trailing-update grid over the level's (system, tile) tasks, then
level-scheduled solves) and ``dag`` (the whole step, assembly to the last
refinement, as ONE persistent launch whose CTAs take tile tasks from a queue
in topological order and start each one when its inputs are final).  The
step is captured into a CUDA graph and replayed with a single launch.
``autotune`` times the schedules and their grid sizes on the real batch and
caches the choice as JSON per device and batch (the tile is 64: two 64 x 65
double-float tiles fill 66.5 KB of shared memory, three CTAs per SM).

``rbf_batch_solve(coords, eps, reg, B, solver)`` is a ``torch.autograd``
function: its backward runs one more solve with A^T = A on the stored factors
(lam = A^{-1} dL/dX) and a fused FP64 contraction that recomputes phi and its
derivatives from the coordinates, giving dL/dB, dL/deps, dL/dreg and
dL/dcoords without forming dA.

Packing: ``coords`` is the concatenation of the (n_s, dim) centre arrays;
``B`` / ``X`` the concatenation of the (n_s, nrhs) blocks, each block stored
column-major (``pack_rhs`` / ``unpack_rhs`` convert from a list of arrays).
"""
from __future__ import annotations

import ctypes
import hashlib
import json
import os
import time
from pathlib import Path

import numpy as np
import torch

from . import _native as N
from ._device import ptr, require_cuda, stream_handle
from .rbf_kernel import KERNELS

ARITH = {"f64": 0, "df32": 1}


def _host_f64(v) -> np.ndarray:
    """Scalar / array / tensor -> FP64 NumPy array (never through a float32 tensor)."""
    if isinstance(v, torch.Tensor):
        return v.detach().to(torch.float64).cpu().numpy()
    return np.asarray(v, dtype=np.float64)


def pack_coords(coords_list) -> torch.Tensor:
    """List of (n_s, dim) arrays -> (sum n_s, dim) FP64 CUDA tensor."""
    dev = require_cuda()
    parts = [torch.as_tensor(np.asarray(c, dtype=np.float64)) if not isinstance(c, torch.Tensor) else c
             for c in coords_list]
    return torch.cat([p.to(device=dev, dtype=torch.float64).reshape(p.shape[0], -1) for p in parts]).contiguous()


def pack_rhs(B_list, nrhs: int) -> torch.Tensor:
    """List of (n_s, nrhs) (or (n_s,)) arrays -> flat FP64 CUDA tensor of column-major blocks."""
    dev = require_cuda()
    out = []
    for b in B_list:
        t = b if isinstance(b, torch.Tensor) else torch.as_tensor(np.asarray(b, dtype=np.float64))
        t = t.to(device=dev, dtype=torch.float64)
        if t.dim() == 1:
            t = t.reshape(-1, 1)
        if t.shape[1] != nrhs:
            raise ValueError(f"each block needs {nrhs} columns, got {t.shape[1]}")
        out.append(t.t().reshape(-1))
    return torch.cat(out).contiguous()


def unpack_rhs(X: torch.Tensor, sizes, nrhs: int):
    """Flat packed blocks -> list of (n_s, nrhs) tensors (views)."""
    res, o = [], 0
    for n in sizes:
        res.append(X[o:o + n * nrhs].reshape(nrhs, n).t())
        o += n * nrhs
    return res


# ---------------------------------------------------------------------------- autotuner

def _cache_path() -> Path:
    p = os.environ.get("MPDOK_GB300_AUTOTUNE")
    if p:
        return Path(p)
    return Path.home() / ".cache" / "mpdok_gb300" / "autotune.json"


def tune_key(device: str, sizes, dim: int, nrhs: int, kernel: str, arith: str) -> str:
    """Cache key: device, problem shape and a digest of the sorted sizes."""
    h = hashlib.sha1(np.sort(np.asarray(sizes, dtype=np.int64)).tobytes()).hexdigest()[:16]
    return f"{device}|batch|d{dim}|k{nrhs}|{kernel}|{arith}|{h}"


def cache_get(key: str):
    p = _cache_path()
    try:
        return json.loads(p.read_text()).get(key)
    except (OSError, ValueError):
        return None


def cache_put(key: str, value) -> None:
    p = _cache_path()
    try:
        data = json.loads(p.read_text())
    except (OSError, ValueError):
        data = {}
    data[key] = value
    p.parent.mkdir(parents=True, exist_ok=True)
    tmp = p.with_suffix(".tmp")
    tmp.write_text(json.dumps(data, indent=1, sort_keys=True))
    tmp.replace(p)


def _config_of(rec):
    """('levels', grid_mult) or ('dag', ctas_per_sm) from a cache record."""
    if "config" in rec:
        kind, v = str(rec["config"]).split(":")
        if kind not in ("levels", "dag"):
            raise ValueError(f"unknown schedule {kind!r}")
        return kind, int(v)
    return "levels", int(rec["grid_mult"])


def choose(candidates, measure, reps: int = 2):
    """Smallest median time over `reps` runs of measure(candidate); returns (best, {cand: seconds})."""
    times = {}
    for c in candidates:
        ts = sorted(measure(c) for _ in range(reps))
        times[c] = ts[len(ts) // 2]
    best = min(times, key=times.get)
    return best, times


# ---------------------------------------------------------------------------- solver

class BatchedRBFSolver:
    """Plan for a fixed list of system sizes; load / factor / solve / adjoint."""

    GRID_CANDIDATES = (1, 2, 4, 8)

    def __init__(self, sizes, dim: int = 2, nrhs: int = 8, kernel: str = "gaussian", arith: str = "df32",
                 grid_mult=None):
        if arith not in ARITH:
            raise ValueError(f"arith must be one of {sorted(ARITH)}")
        self.sizes = [int(n) for n in sizes]
        if not self.sizes or min(self.sizes) < 1:
            raise ValueError("sizes must be a non-empty list of positive integers")
        self.dim, self.nrhs, self.kernel, self.arith = int(dim), int(nrhs), kernel, arith
        self.nsys = len(self.sizes)
        self.total_x = sum(self.sizes) * self.nrhs
        self.total_c = sum(self.sizes) * self.dim
        dev = require_cuda()
        self.device_name = torch.cuda.get_device_name(dev)
        self.key = tune_key(self.device_name, self.sizes, self.dim, self.nrhs, kernel, arith)
        self.tuned = None
        self.schedule, self.dag_ctas = "levels", 3
        cfg = None
        if grid_mult is None:
            hit = cache_get(self.key)
            cfg = _config_of(hit) if hit else None
            self.tuned = hit
        self._plan = None
        self._loaded = None
        if cfg and cfg[0] == "dag":
            self._create(2)
            self._set_schedule("dag", cfg[1])
        else:
            self._create(int(cfg[1]) if cfg else int(grid_mult or 2))

    def _create(self, grid_mult: int):
        self.free()
        lib = N.load()
        h = ctypes.c_void_p()
        n_arr = (ctypes.c_longlong * self.nsys)(*self.sizes)
        N.check(lib.mpdok_batch_create(self.nsys, n_arr, self.dim, self.nrhs, KERNELS[self.kernel],
                                       ARITH[self.arith], grid_mult, ctypes.byref(h)), "batch_create")
        self._plan = h
        self.grid_mult = grid_mult
        self.schedule = "levels"

    def _set_schedule(self, schedule: str, ctas_per_sm: int = 3):
        N.check(N.load().mpdok_batch_schedule(self._plan, 1 if schedule == "dag" else 0, int(ctas_per_sm)),
                "batch_schedule")
        self.schedule, self.dag_ctas = schedule, int(ctas_per_sm)

    def configure(self, config: str):
        """Apply a schedule: 'levels:<grid_mult>' or 'dag:<ctas per SM>'."""
        kind, v = _config_of({"config": config})
        if kind == "dag":
            self._set_schedule("dag", v)
        else:
            if v != self.grid_mult:
                self._create(v)
                if self._loaded is not None:
                    self.load(*self._loaded)
            self._set_schedule("levels")
        return self

    @property
    def config(self) -> str:
        return f"dag:{self.dag_ctas}" if self.schedule == "dag" else f"levels:{self.grid_mult}"

    @property
    def device_bytes(self) -> int:
        return int(N.load().mpdok_batch_bytes(self._plan)) if self._plan else 0

    # -- data -----------------------------------------------------------------
    def load(self, coords, eps, reg):
        """coords: packed (sum n, dim) tensor or list of arrays; eps, reg: scalars or (nsys,)."""
        c = coords if isinstance(coords, torch.Tensor) and coords.dim() == 2 and coords.shape[0] == sum(self.sizes) \
            else pack_coords(coords)
        c = c.detach().to(device=require_cuda(), dtype=torch.float64).contiguous()
        if c.shape != (sum(self.sizes), self.dim):
            raise ValueError(f"coords must be ({sum(self.sizes)}, {self.dim}), got {tuple(c.shape)}")
        e = np.broadcast_to(_host_f64(eps), (self.nsys,)).copy()
        r = np.broadcast_to(_host_f64(reg), (self.nsys,)).copy()
        N.check(N.load().mpdok_batch_load(self._plan, ptr(c), e.ctypes.data, r.ctypes.data, stream_handle()),
                "batch_load")
        self._loaded = (c, e, r)
        return self

    def factor(self):
        self._need_loaded()
        N.check(N.load().mpdok_batch_factor(self._plan, stream_handle()), "batch_factor")
        return self

    def perturbed_pivots(self) -> int:
        st = N.load().mpdok_batch_perturbed(self._plan, stream_handle())
        if st < 0:
            N.check(st, "batch_perturbed")
        return int(st)

    def _rhs(self, B) -> torch.Tensor:
        if isinstance(B, torch.Tensor) and B.dim() == 1:
            t = B.detach().to(device=require_cuda(), dtype=torch.float64).contiguous()
        else:
            t = pack_rhs(B, self.nrhs)
        if t.numel() != self.total_x:
            raise ValueError(f"packed RHS must hold {self.total_x} values, got {t.numel()}")
        return t

    def solve(self, B, refine: int = 2) -> torch.Tensor:
        """X = A^{-1} B (packed), with `refine` FP64 refinement steps."""
        b = self._rhs(B)
        X = torch.empty_like(b)
        N.check(N.load().mpdok_batch_solve(self._plan, ptr(b), ptr(X), int(refine), stream_handle()), "batch_solve")
        return X

    def step(self, B, refine: int = 2) -> torch.Tensor:
        """Assembly + factor + solve + `refine` FP64 refinements under the plan's schedule."""
        self._need_loaded()
        b = self._rhs(B)
        X = torch.empty_like(b)
        N.check(N.load().mpdok_batch_step(self._plan, ptr(b), ptr(X), int(refine), stream_handle()), "batch_step")
        return X

    def dag_status(self):
        """Raise when a task of the last task-graph step gave up waiting on its inputs."""
        N.check(N.load().mpdok_batch_dag_status(self._plan, stream_handle()), "batch_dag_status")

    def relres(self, B, X) -> torch.Tensor:
        b = self._rhs(B)
        x = self._rhs(X)
        out = torch.empty(self.nsys, dtype=torch.float64, device=b.device)
        N.check(N.load().mpdok_batch_relres(self._plan, ptr(b), ptr(x), ptr(out), stream_handle()), "batch_relres")
        return out

    def adjoint(self, X, Lam):
        """(dL/dcoords packed, dL/deps (nsys,), dL/dreg (nsys,)) from Lam = A^{-1} dL/dX."""
        self._need_loaded()
        x = self._rhs(X)
        lam = self._rhs(Lam)
        gc = torch.empty((sum(self.sizes), self.dim), dtype=torch.float64, device=x.device)
        ge = torch.empty(self.nsys, dtype=torch.float64, device=x.device)
        gr = torch.empty(self.nsys, dtype=torch.float64, device=x.device)
        N.check(N.load().mpdok_batch_adjoint(self._plan, ptr(x), ptr(lam), ptr(gc), ptr(ge), ptr(gr),
                                             stream_handle()), "batch_adjoint")
        return gc, ge, gr

    # -- graph ----------------------------------------------------------------
    def build_graph(self, B, refine: int = 2):
        """Capture factor + solve (+ refine) on persistent B / X buffers; returns (B_buf, X_buf)."""
        self._need_loaded()
        self._gB = self._rhs(B).clone()
        self._gX = torch.empty_like(self._gB)
        torch.cuda.synchronize()
        N.check(N.load().mpdok_batch_graph_build(self._plan, ptr(self._gB), ptr(self._gX), int(refine)),
                "batch_graph_build")
        return self._gB, self._gX

    def run_graph(self) -> torch.Tensor:
        N.check(N.load().mpdok_batch_graph_launch(self._plan, stream_handle()), "batch_graph_launch")
        return self._gX

    @property
    def graph_nodes(self) -> int:
        return int(N.load().mpdok_batch_graph_nodes(self._plan))

    # -- tuning ---------------------------------------------------------------
    CANDIDATES = ("levels:2", "levels:4", "dag:2", "dag:3")

    def autotune(self, candidates=None, reps: int = 1, force: bool = False):
        """Time one full step (assembly, factor, solve, two refinements) per
        schedule candidate on the loaded batch, keep the fastest and cache it
        per device and batch.  Candidates: 'levels:<trailing-update grid
        multiplier>' and 'dag:<CTAs per SM of the persistent task graph>'."""
        self._need_loaded()
        if not force:
            hit = cache_get(self.key)
            if hit and "config" in hit:
                self.configure(hit["config"])
                self.tuned = hit
                return hit
        cands = tuple(candidates or self.CANDIDATES)
        Bt = torch.ones(self.total_x, dtype=torch.float64, device=require_cuda())

        def measure(cfg):
            self.configure(cfg)
            self.step(Bt, refine=2)  # warm: allocation of the task-graph tables, first-touch
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            self.step(Bt, refine=2)
            e1.record()
            torch.cuda.synchronize()
            if self.schedule == "dag":
                self.dag_status()
            return e0.elapsed_time(e1) / 1e3

        best, times = choose(cands, measure, reps)
        rec = {"config": best, "seconds": dict(times), "tile": 64, "when": time.time()}
        cache_put(self.key, rec)
        self.configure(best)
        self.tuned = rec
        return rec

    def _need_loaded(self):
        if self._loaded is None:
            raise RuntimeError("call load() first")

    def free(self):
        if getattr(self, "_plan", None):
            N.load().mpdok_batch_destroy(self._plan)
        self._plan = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


# ---------------------------------------------------------------------------- autograd

class CholeskyPreconditioner:
    """FP64-accurate Cholesky factor of one RBF system, for ``cg_ir(..., precond=)``.

    A batch plan of one system (double-float trailing update, FP64 diagonal
    blocks and solves) factored once; the CG-IR's inner CG applies
    z = (L L^T)^-1 r to all ``nrhs`` columns at once.  This makes the FP32 CG
    body converge on systems whose kappa * 6e-8 > 1 (the C2 family), where
    the unpreconditioned CG of the reference (dense_krylov.py:119-205) stalls.
    """

    def __init__(self, coords, eps: float, reg: float, nrhs: int = 1, kernel: str = "gaussian",
                 arith: str = "df32", grid_mult: int = 2):
        c = coords if isinstance(coords, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(coords))
        c = c.detach().to(device=require_cuda(), dtype=torch.float64).contiguous()
        self.n, self.dim = int(c.shape[0]), int(c.shape[1])
        self.nrhs = int(nrhs)
        self.solver = BatchedRBFSolver([self.n], dim=self.dim, nrhs=self.nrhs, kernel=kernel, arith=arith,
                                       grid_mult=grid_mult)
        self.solver.load(c, float(eps), float(reg)).factor()

    @property
    def plan(self):
        return self.solver._plan


class _BatchSolveFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, coords, eps, reg, B, solver, refine):
        solver.load(coords, eps, reg).factor()
        X = solver.solve(B, refine)
        ctx.solver = solver
        ctx.refine = refine
        ctx.save_for_backward(X)
        ctx.eps_shape = eps.shape
        ctx.reg_shape = reg.shape
        return X

    @staticmethod
    def backward(ctx, gX):
        (X,) = ctx.saved_tensors
        solver = ctx.solver
        lam = solver.solve(gX.contiguous(), ctx.refine)  # A^T = A: the same factors
        gc, ge, gr = solver.adjoint(X, lam)
        ge = ge if ctx.eps_shape == ge.shape else ge.sum().reshape(ctx.eps_shape)
        gr = gr if ctx.reg_shape == gr.shape else gr.sum().reshape(ctx.reg_shape)
        return gc, ge, gr, lam, None, None


def rbf_batch_solve(coords: torch.Tensor, eps: torch.Tensor, reg: torch.Tensor, B: torch.Tensor,
                    solver: BatchedRBFSolver, refine: int = 2) -> torch.Tensor:
    """Differentiable X = A(coords, eps, reg)^{-1} B over a batch (packed tensors).

    eps and reg are (nsys,) tensors or 0-d tensors shared by every system.
    The solver's factors must stay untouched between the forward call and
    the backward pass.
    """
    eps = torch.as_tensor(eps, dtype=torch.float64, device=coords.device)
    reg = torch.as_tensor(reg, dtype=torch.float64, device=coords.device)
    return _BatchSolveFn.apply(coords, eps, reg, B, solver, refine)
