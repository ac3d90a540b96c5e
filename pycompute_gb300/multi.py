"""Mixed-model batches: several models and protocol lengths in one persistent launch.

``MultiModelFitter([(Expr, ndata), ...])`` compiles one program holding every
model; ``fit(jobs, iters)`` fits all of them in one launch of the persistent
kernel, whose warps claim chunks of voxels from a device work counter (a warp
always runs a single model). ``capture(jobs, iters)`` records the work-counter
reset and the launch in a CUDA graph for repeated fits of the same buffers.

``autotune(...)`` picks threads per block, a register cap, the chunk size,
the queue order and, per model, the warp lanes that share one voxel (1, or 2
that split the voxel's samples and sum their shares of f, J^T r and the
Hessian with 2 + P + P(P+1)/2 lane shuffles per iteration; the solve then runs
on both lanes) by timing short fits of a sample of every job, and caches the
choice per GPU and model set in ``_build/autotune.json``.
"""
from __future__ import annotations

import ctypes
import hashlib
import json
import os
import time

import torch

from . import _lib, build as _build, codegen
from .lsqnonlin import Expr, _dtype, _stream_ptr

_TD = {torch.float32: 0, torch.float64: 1}


class _Job(ctypes.Structure):
    _fields_ = [("data", ctypes.c_void_p), ("params", ctypes.c_void_p), ("lam", ctypes.c_void_p),
                ("step_type", ctypes.c_void_p), ("f", ctypes.c_void_p), ("first_f", ctypes.c_void_p),
                ("last_f", ctypes.c_void_p), ("iters_done", ctypes.c_void_p), ("nprobs", ctypes.c_int64),
                ("protocol", ctypes.c_void_p), ("lb", ctypes.c_void_p), ("ub", ctypes.c_void_p)]


class MultiJob:
    """Buffers of one model's voxels in a mixed batch (fitter state included)."""

    def __init__(self, pars: torch.Tensor, data: torch.Tensor, protocol, lb, ub):
        N = int(data.shape[1])
        dev = data.device
        self.pars, self.data, self.N = pars, data, N
        self.protocol = [float(x) for x in protocol]
        self.lb = [float(x) for x in lb]
        self.ub = [float(x) for x in ub]
        dt = pars.dtype
        self.lam = torch.full((N,), 5.0, dtype=dt, device=dev)
        self.step_type = torch.ones((N,), dtype=torch.int8, device=dev)
        self.f = torch.zeros((N,), dtype=dt, device=dev)
        self.first_f = torch.empty((N,), dtype=dt, device=dev)
        self.last_f = torch.empty((N,), dtype=dt, device=dev)
        self.iters = torch.zeros((N,), dtype=torch.int32, device=dev)
        self._host = [(ctypes.c_double * max(1, len(v)))(*v) for v in (self.protocol, self.lb, self.ub)]

    def reset(self, init: torch.Tensor | None = None):
        if init is not None:
            self.pars.copy_(init)
        self.lam.fill_(5.0)
        self.step_type.fill_(1)
        self.f.zero_()
        self.iters.zero_()

    def ctype(self) -> _Job:
        p = lambda t: t.data_ptr()  # noqa: E731
        return _Job(p(self.data), p(self.pars), p(self.lam), p(self.step_type), p(self.f), p(self.first_f),
                    p(self.last_f), p(self.iters), self.N, ctypes.cast(self._host[0], ctypes.c_void_p),
                    ctypes.cast(self._host[1], ctypes.c_void_p), ctypes.cast(self._host[2], ctypes.c_void_p))


class MultiModelFitter:
    """One program, one persistent launch, several models (see module docstring)."""

    _programs: dict = {}

    def __init__(self, models: list, dtype=torch.float32, solve_dtype=None, block: int = 128, maxrreg: int = 0,
                 lanes=None):
        self.dtype = _dtype(dtype)
        self.solve_dtype = _dtype(solve_dtype) if solve_dtype is not None else torch.float64
        self.models = []
        for m, ndata in models:
            gm = codegen.generate(m.expr, m.pars_str, m.consts_str)
            self.models.append((gm, int(ndata)))
        self.block, self.maxrreg = int(block), int(maxrreg)
        # warp lanes per voxel, per model (1 or 2: two lanes split a voxel's samples)
        self.lanes = [1] * len(self.models) if lanes is None else [int(x) for x in lanes]
        if len(self.lanes) != len(self.models):
            raise ValueError("one lanes-per-voxel entry per model")
        self._prog = None
        self._counter = None
        self.chunk = 64
        self.grid = 0
        self.order = None  # queue order of the jobs (None = program order)

    def key(self) -> str:
        h = hashlib.sha1()
        for gm, nd in self.models:
            h.update(f"{gm.expr}|{gm.pars}|{gm.consts}|{nd};".encode())
        h.update(f"{self.dtype}{self.solve_dtype}".encode())
        return h.hexdigest()[:16]

    def build(self):
        dev = torch.cuda.current_device()
        key = (self.key(), self.block, self.maxrreg, tuple(self.lanes), dev)
        prog = MultiModelFitter._programs.get(key)
        if prog is None:
            n = len(self.models)
            srcs = (ctypes.c_char_p * n)(*[gm.source.encode() for gm, _ in self.models])
            structs = (ctypes.c_char_p * n)(*[gm.struct_name.encode() for gm, _ in self.models])
            ints = lambda v: (ctypes.c_int * n)(*v)  # noqa: E731
            h = ctypes.c_void_p()
            rc = _lib.lib().pcgb_multi_create(n, srcs, structs, ints([gm.P for gm, _ in self.models]),
                                              ints([gm.C for gm, _ in self.models]),
                                              ints([nd for _, nd in self.models]), _TD[self.dtype],
                                              _TD[self.solve_dtype], self.maxrreg, self.block, ints(self.lanes),
                                              _lib.cache_dir().encode(), ctypes.byref(h))
            _lib.check("pcgb_multi_create", rc)
            prog = h
            MultiModelFitter._programs[key] = prog
        self._prog = prog
        if self._counter is None or self._counter.device.index != dev:
            self._counter = torch.zeros(1, dtype=torch.int32, device=torch.device("cuda", dev))
        return prog

    def persistent_grid(self) -> int:
        return _lib.lib().pcgb_multi_grid(self.build())

    def heaviest_first(self) -> list[int]:
        """Queue order by decreasing work per iteration (samples x parameters^2)."""
        cost = [nd * gm.P * gm.P for gm, nd in self.models]
        return sorted(range(len(cost)), key=lambda k: -cost[k])

    def fit(self, jobs: list[MultiJob], iters: int, tol=1e-8, mu=0.25, eta=0.75, acc=0.2, dec=2.0,
            chunk: int | None = None, grid: int | None = None, order: list[int] | None = None):
        if len(jobs) != len(self.models):
            raise ValueError("one job per model")
        prog = self.build()
        arr = (_Job * len(jobs))(*[j.ctype() for j in jobs])
        order = self.order if order is None else order
        ordc = (ctypes.c_int * len(jobs))(*order) if order is not None else None
        rc = _lib.lib().pcgb_multi_run(prog, arr, len(jobs), ordc, int(iters), float(tol), float(mu), float(eta),
                                       float(acc), float(dec), int(chunk or self.chunk),
                                       int(self.grid if grid is None else grid),
                                       ctypes.c_void_p(self._counter.data_ptr()), ctypes.c_void_p(_stream_ptr()))
        _lib.check("pcgb_multi_run", rc)

    def capture(self, jobs: list[MultiJob], iters: int, **kw) -> torch.cuda.CUDAGraph:
        """CUDA graph of (work-counter reset, persistent launch) for these buffers."""
        self.fit(jobs, 0, **kw)  # loads the program outside the capture
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            with torch.cuda.graph(g, stream=s):
                self.fit(jobs, iters, **kw)
        torch.cuda.current_stream().wait_stream(s)
        return g


def _cache_path() -> str:
    return os.path.join(_build.BUILD, "autotune.json")


def autotune(models: list, make_jobs, iters: int, dtype=torch.float32, solve_dtype=None,
             blocks=(64, 128, 256), maxrregs=(0, 128, 96), chunks=(32, 64, 128, 256), reps: int = 2,
             use_cache: bool = True, lane_options=(1, 2)) -> dict:
    """Pick (block, maxrreg, chunk, order, lanes) for a model set.

    make_jobs() returns fresh MultiJob lists of a representative sample; each
    configuration is timed on it with CUDA events after one warm-up fit. The
    launch shape is searched with one lane per voxel; then, model by model,
    each other lanes-per-voxel option is tried on the best shape and kept if
    the whole fit gets faster. The result is cached per GPU name and model set.
    """
    probe = MultiModelFitter(models, dtype, solve_dtype)
    gpu = torch.cuda.get_device_name()
    key = f"{gpu}|{probe.key()}|{iters}|lanes{','.join(str(x) for x in lane_options)}"
    path = _cache_path()
    cache = {}
    if use_cache and os.path.exists(path):
        try:
            cache = json.load(open(path))
        except (OSError, ValueError):
            cache = {}
        if key in cache:
            return cache[key]
    jobs = make_jobs()
    inits = [j.pars.clone() for j in jobs]
    results = []
    t0 = time.perf_counter()
    for block in blocks:
        for maxrreg in maxrregs:
            fitter = MultiModelFitter(models, dtype, solve_dtype, block=block, maxrreg=maxrreg)
            try:
                fitter.build()
            except _lib.PcgbError:
                continue
            for chunk in chunks:
                for order in (list(range(len(models))), fitter.heaviest_first()):
                    times = []
                    for r in range(reps + 1):
                        for j, i0 in zip(jobs, inits):
                            j.reset(i0)
                        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                        s.record()
                        fitter.fit(jobs, iters, chunk=chunk, order=order)
                        e.record()
                        torch.cuda.synchronize()
                        if r:
                            times.append(s.elapsed_time(e))
                    results.append({"block": block, "maxrreg": maxrreg, "chunk": chunk, "order": order,
                                    "ms": min(times)})
    best = dict(min(results, key=lambda r: r["ms"]), lanes=[1] * len(models))

    def time_lanes(lanes):
        fitter = MultiModelFitter(models, dtype, solve_dtype, block=best["block"], maxrreg=best["maxrreg"],
                                  lanes=lanes)
        try:
            fitter.build()
        except _lib.PcgbError:
            return None
        times = []
        for r in range(reps + 1):
            for j, i0 in zip(jobs, inits):
                j.reset(i0)
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s.record()
            fitter.fit(jobs, iters, chunk=best["chunk"], order=best["order"])
            e.record()
            torch.cuda.synchronize()
            if r:
                times.append(s.elapsed_time(e))
        return min(times)

    lane_trials = []
    for k in range(len(models)):
        for opt in lane_options:
            if opt == best["lanes"][k]:
                continue
            lanes = list(best["lanes"])
            lanes[k] = opt
            ms = time_lanes(lanes)
            lane_trials.append({"lanes": lanes, "ms": ms})
            if ms is not None and ms < best["ms"]:
                best.update(lanes=lanes, ms=ms)
    out = dict(best, gpu=gpu, trials=results, lane_trials=lane_trials, tune_s=round(time.perf_counter() - t0, 2))
    cache[key] = out
    os.makedirs(os.path.dirname(path), exist_ok=True)
    with open(path, "w") as f:
        json.dump(cache, f, indent=1)
    return out
