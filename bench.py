"""Benchmark: IVIM voxel fits/s of the batched LM fitter on GB300.

Workload (default): plain LM at scale - IVIM bi-exponential, 4 parameters,
b = {0,10,20,50,100,200,400,600,800,1000} s/mm^2, 256x256x128 = 8,388,608
voxels, fp32 state with the GMW81 solve and gain-ratio test in fp64, at most
100 iterations per voxel, constant initialisation [max S, 0.1, 1e-2, 1e-3],
seeded synthetic signals (uniform true parameters, Rician noise at SNR 50).

One step = one full fit of every voxel: the fitter state is reset from the
initial parameters and run(100) is called. Inputs (335 MB of signals) are
larger than L2 (129 MB), so no L2 flush is needed between steps.

Reported (one JSON line from rank 0):
  value        fits/s with inputs resident in HBM (whole job over ranks)
  e2e          fits/s through the public API from pinned host buffers,
               host->device copies of signals and initial parameters and the
               device->host read of fitted parameters and status inside the
               timed region
  roofline     HBM roofline of the LM kernel: algorithmic bytes
               (4M + 4P + 1 per voxel: signals in, parameters and status out)
               over the kernel's event-timed duration, against the measured
               copy bandwidth in MEASURED_PEAKS.json
  cpu_baseline the CPU oracle (the reference algorithm in fp32) on a bounded
               sample on all host cores
  accuracy     median relative error of the fitted maps against the all-FP64
               GPU fitter (same LM, same initialisation)

`--impl reference` times the reference's CPU implementation instead (its own
generated kernel built for the host when available, else the CPU oracle in the
reference's fp32 arithmetic) on all host threads, one bounded sample per step.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

M_IVIM10 = 10
P_IVIM = 4


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            pk = json.load(f)
        return float(pk["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", str(self.gpu)], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def cpu_sample(iters: int, target_s: float, dtype_mode: str = "reference", min_voxels: int = 16384,
               parity_out: dict | None = None):
    """Time the CPU reference implementation on a bounded IVIM-10 sample.

    Uses the reference's generated kernel built for the host (oracle/_ref)
    when present, else the CPU oracle in the reference's fp32 arithmetic. The
    sample doubles until one run takes at least target_s/4 seconds, then the
    last size is timed once. Returns (fits_per_s, kind, cores, sample_text).
    With ``parity_out``, the GPU fitter is run on the same sample (FP64 solve
    and fp32 solve) and its agreement with the CPU fit is recorded there.
    """
    from oracle import OracleModel, RefIVIM, ref_available
    from pycompute_gb300 import synth

    w = synth.ivim()
    cores = os.cpu_count() or 1
    if ref_available(M_IVIM10):
        impl, kind = RefIVIM(M_IVIM10), "reference"
        run = lambda p, d, i, lb, ub, prot: impl.lm_run(p, prot, d, lb, ub, iters)  # noqa: E731
    else:
        impl, kind = OracleModel(w.expr, w.pars, w.consts), "port"
        impl.set_threads(cores)
        run = lambda p, d, i, lb, ub, prot: impl.lm_run(p, prot, d, lb, ub, iters)  # noqa: E731
    n = min_voxels
    while True:
        true, data, init, lb, ub, prot = w.generate(n, seed=7)
        p = init.copy()
        t0 = time.perf_counter()
        res = run(p, data, init, lb, ub, prot)
        el = time.perf_counter() - t0
        if el >= target_s / 4 or n >= (1 << 22):
            break
        n *= 2 if el > 0.05 else 8
    sample = (f"{n} IVIM-10 voxels x {iters} iterations ({'reference generated kernel' if kind == 'reference' else 'fp32 oracle port'}, "
              f"{cores} threads), {el:.2f} s")
    if parity_out is not None:
        parity_out.update(gpu_vs_cpu_parity(w, data, init, lb, ub, prot, p, res["step_type"], iters, kind))
    return n / el, kind, cores, sample


def gpu_vs_cpu_parity(w, data, init, lb, ub, prot, p_cpu, st_cpu, iters, kind):
    """The GPU fitter on the CPU sample's inputs, compared with the CPU fit
    (parameters and convergence flags, step_type == 0)."""
    import torch
    from pycompute_gb300 import Expr, SecondOrderLevenbergMarquardt, parity

    out = {"cpu": kind, "voxels": int(data.shape[1]), "iters": iters}
    for solve, tdt in (("f64", torch.float64), ("f32", torch.float32)):
        solm = SecondOrderLevenbergMarquardt(Expr(w.expr, w.pars, w.consts), None, w.M, torch.float32,
                                             solve_dtype=tdt)
        t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
        pars = t(init)
        solm.setup(pars, t(prot), t(data), t(lb), t(ub))
        solm.run(iters)
        torch.cuda.synchronize()
        rep = parity.compare_params(pars.cpu().numpy(), p_cpu)
        out[f"solve_{solve}"] = {"median_rel_err": rep["median_rel"], "frac_gt_1e-4": rep["frac_gt_1e-4"],
                                 "flags_agree": parity.flags_agree(solm.step_type_t.cpu().numpy()[0], st_cpu)}
    return out


def _median_rel_gpu(a, b):
    """Median over voxels of the worst per-parameter relative error (on the GPU)."""
    import torch
    r = (a.double() - b.double()).abs() / b.double().abs().clamp_min(1e-30)
    r = torch.nan_to_num(r, nan=float("inf")).amax(dim=0)
    return float(r.median()), float((r > 1e-4).double().mean())


def _time_ms(fn, warmup=2, reps=3):
    import torch
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s.record()
    for _ in range(reps):
        fn()
    e.record()
    torch.cuda.synchronize()
    return s.elapsed_time(e) / reps


def budget_for_tolerance(run_with, ref, budgets, tol=1e-4):
    """Smallest iteration budget whose fit has median relative error <= tol vs ref."""
    curve = {}
    for k in budgets:
        med, frac = _median_rel_gpu(run_with(k), ref)
        curve[k] = (med, frac)
        if med <= tol:
            return k, curve
    return None, curve


def fp64_reference(w, data, iters=1000):
    """All-FP64 fit (same LM, constant init, tolerance 1e-30) as the error reference."""
    import torch
    from pycompute_gb300 import Expr, SecondOrderLevenbergMarquardt, pipeline
    dev = data.device
    solm = SecondOrderLevenbergMarquardt(Expr(w.expr, w.pars, w.consts), None, w.M, torch.float64)
    p = pipeline.init_constant(data, w.init_values).double()
    solm.setup(p, torch.tensor(w.protocol, device=dev).double(), data.double(), torch.tensor(w.lb, device=dev).double(),
               torch.tensor(w.ub, device=dev).double())
    solm.run(iters, tol=1e-30)
    torch.cuda.synchronize()
    return p


def warm_start_comparison(n_eval=1 << 24, n_train=1 << 21, epochs=64, seed=77, lam0=3e-3):
    """C5: IVIM-16, MLP warm start + LM + fallback vs plain LM, fits/s at 1e-4 vs FP64."""
    import torch
    from pycompute_gb300 import Expr, SecondOrderLevenbergMarquardt, pipeline, synth
    from pycompute_gb300.warmstart import WarmStartMLP
    dev = torch.device("cuda")
    w = synth.ivim(synth.ivim_b16(), name="ivim16")
    expr = Expr(w.expr, w.pars, w.consts)
    prot = torch.tensor(w.protocol, device=dev)
    lb = torch.tensor(w.lb, device=dev)
    ub = torch.tensor(w.ub, device=dev)
    t0 = time.perf_counter()
    _, tr = pipeline.synth_gpu(w, n_train, seed=seed, device=dev)
    lab = pipeline.init_constant(tr, w.init_values)
    s = SecondOrderLevenbergMarquardt(expr, None, w.M, torch.float32)
    s.setup(lab, prot, tr, lb, ub)
    s.run(100)
    net = WarmStartMLP(16, 4, [0, 1, 2, 2], w.lb, w.ub, dev, seed=seed)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    net.train(tr, lab, epochs=epochs, batch=8192, lr=2e-3)
    train_s = time.perf_counter() - t1
    del tr, lab, s
    _, data = pipeline.synth_gpu(w, n_eval, seed=seed + 1, device=dev)
    ref = fp64_reference(w, data, iters=300)
    pars = torch.empty((4, n_eval), device=dev)
    plain = SecondOrderLevenbergMarquardt(expr, None, w.M, torch.float32)

    def run_plain(k):
        pipeline.init_constant(data, w.init_values, out=pars)
        plain.setup(pars, prot, data, lb, ub)
        plain.run(k)
        return pars

    wf = pipeline.WarmStartFitter(w, net)
    state = {}

    def run_warm(k, timings=None):
        state["res"] = wf.fit(data, iters_warm=k, iters_fallback=k_plain or 30, pars_out=pars, lam0=lam0,
                              timings=timings)
        return state["res"]["pars"]

    k_plain, curve_plain = budget_for_tolerance(run_plain, ref, range(1, 31))
    k_warm, curve_warm = budget_for_tolerance(run_warm, ref, range(0, 21))
    out = {"workload": "ivim16_warm_vs_plain", "voxels": n_eval, "train_voxels": n_train, "epochs": epochs,
           "train_s": round(train_s, 3), "setup_s": round(time.perf_counter() - t0, 1),
           "plain_iters_for_1e-4": k_plain, "warm_iters_for_1e-4": k_warm,
           "plain_curve": {k: v[0] for k, v in curve_plain.items()},
           "warm_curve": {k: v[0] for k, v in curve_warm.items()}}
    if k_plain is not None:
        ms = _time_ms(lambda: run_plain(k_plain))
        med, frac = _median_rel_gpu(run_plain(k_plain), ref)
        out["plain"] = {"fits_per_s": n_eval / (ms / 1e3), "ms": ms, "median_rel_err": med, "frac_gt_1e-4": frac}
    if k_warm is not None:
        ms = _time_ms(lambda: run_warm(k_warm))
        med, frac = _median_rel_gpu(run_warm(k_warm), ref)
        tm = {}
        run_warm(k_warm, timings=tm)
        out["warm"] = {"fits_per_s": n_eval / (ms / 1e3), "ms": ms, "median_rel_err": med, "frac_gt_1e-4": frac,
                       "fallback_voxels": state["res"]["n_fallback"], "refits_kept": state["res"]["n_refit_kept"],
                       "stage_ms": {k: round(v, 3) for k, v in tm.items()}}
    if "plain" in out and "warm" in out:
        out["speedup"] = out["warm"]["fits_per_s"] / out["plain"]["fits_per_s"]
    return out


def mixed_batch_comparison(n_per_model=1 << 20, iters=100, seed=300):
    """C3: VFA-T1 + T2* + IVIM + bi-exp T2, 1M voxels each, one persistent
    launch (autotuned) vs one single-model launch per model."""
    import torch
    from pycompute_gb300 import Expr, SecondOrderLevenbergMarquardt, pipeline, synth
    from pycompute_gb300.multi import MultiJob, MultiModelFitter, autotune
    dev = torch.device("cuda")
    ws = [synth.vfa_t1(), synth.t2star(), synth.ivim(), synth.biexp_t2()]
    gens = []
    for k, w in enumerate(ws):
        true, data = pipeline.synth_gpu(w, n_per_model, seed=seed + k, device=dev)
        gens.append((data, pipeline.init_constant(data, w.init_values)))
    models = [(Expr(w.expr, w.pars, w.consts), w.M) for w in ws]

    def make_jobs(frac=1.0):
        jobs = []
        for w, (data, init) in zip(ws, gens):
            n = max(1024, int(data.shape[1] * frac))
            jobs.append(MultiJob(init[:, :n].clone(), data[:, :n].contiguous(), w.protocol, w.lb, w.ub))
        return jobs

    t0 = time.perf_counter()
    tuned = autotune(models, lambda: make_jobs(0.125), iters=20)
    tune_s = time.perf_counter() - t0
    fitter = MultiModelFitter(models, block=tuned["block"], maxrreg=tuned["maxrreg"])
    fitter.chunk = tuned["chunk"]
    fitter.order = tuned.get("order")
    jobs = make_jobs()
    inits = [j.pars.clone() for j in jobs]

    def run_multi():
        for j, i0 in zip(jobs, inits):
            j.reset(i0)
        fitter.fit(jobs, iters)

    graph = fitter.capture(jobs, iters)

    def run_graph():
        for j, i0 in zip(jobs, inits):
            j.reset(i0)
        graph.replay()

    singles = []
    for w, (data, init) in zip(ws, gens):
        solm = SecondOrderLevenbergMarquardt(Expr(w.expr, w.pars, w.consts), None, w.M, torch.float32)
        p = init.clone()
        solm.setup(p, torch.tensor(w.protocol, device=dev), data, torch.tensor(w.lb, device=dev),
                   torch.tensor(w.ub, device=dev))
        singles.append((solm, p, init))

    def run_singles():
        for solm, p, init in singles:
            p.copy_(init)
            solm.lam_t.fill_(5.0)
            solm.step_type_t.fill_(1)
            solm.run(iters)

    total = sum(int(d.shape[1]) for d, _ in gens)
    ms_multi = _time_ms(run_multi)
    ms_graph = _time_ms(run_graph)
    ms_single = _time_ms(run_singles)
    its = [float(j.iters.double().mean()) for j in jobs]
    return {"workload": "mixed_vfa8_t2s16_ivim10_biexp32", "voxels": total, "iters": iters,
            "autotuned": {k: tuned.get(k) for k in ("block", "maxrreg", "chunk", "order", "ms")},
            "tune_s": round(tune_s, 1),
            "one_launch_fits_per_s": total / (ms_multi / 1e3), "graph_fits_per_s": total / (ms_graph / 1e3),
            "per_model_launches_fits_per_s": total / (ms_single / 1e3), "mean_iters_per_model": its,
            "ms": {"one_launch": ms_multi, "graph": ms_graph, "per_model": ms_single}}


def run_reference_arm(args):
    ws, rank, local = _dist()
    if rank != 0:
        return 0
    vals = []
    for s in range(args.warmup + args.steps):
        v, kind, cores, sample = cpu_sample(args.iters, target_s=args.cpu_seconds, min_voxels=16384)
        if s >= args.warmup:
            vals.append(v)
    value = statistics.median(vals)
    line = {
        "impl": "reference", "metric": "IVIM voxel fits/s", "value": value, "unit": "fits/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded IVIM-10, Rician SNR 50)",
        "config": {"workload": "ivim10_plain_lm_cpu_sample", "iters": args.iters},
        "cpu_baseline": {"value": value, "unit": "fits/s", "cores": cores, "kind": kind, "sample": sample},
        "e2e": {"value": value, "unit": "fits/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--voxels", type=int, default=256 * 256 * 128)
    ap.add_argument("--iters", type=int, default=100)
    ap.add_argument("--solve", default="f64", choices=["f64", "f32"])
    ap.add_argument("--block", type=int, default=0)
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-fp64-check", action="store_true")
    ap.add_argument("--no-warm", action="store_true", help="skip the warm-start comparison (IVIM-16)")
    ap.add_argument("--warm-voxels", type=int, default=1 << 24)
    ap.add_argument("--only-warm", action="store_true", help="run only the warm-start comparison")
    ap.add_argument("--only-mixed", action="store_true", help="run only the mixed-model batch comparison")
    ap.add_argument("--no-mixed", action="store_true")
    ap.add_argument("--warm-epochs", type=int, default=64)
    ap.add_argument("--warm-lam0", type=float, default=3e-3)
    ap.add_argument("--warm-train", type=int, default=1 << 21)
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference_arm(args)
    if args.only_mixed:
        print(json.dumps(mixed_batch_comparison()), flush=True)
        return 0
    if args.only_warm:
        print(json.dumps(warm_start_comparison(n_eval=args.warm_voxels, epochs=args.warm_epochs,
                                               lam0=args.warm_lam0, n_train=args.warm_train)), flush=True)
        return 0

    import torch
    import torch.distributed as dist

    from pycompute_gb300 import Expr, SecondOrderLevenbergMarquardt, parity, synth

    from pycompute_gb300.shard import max_over_ranks

    ws, rank, local = _dist()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if ws > 1:
        dist.init_process_group("nccl", device_id=dev)

    w = synth.ivim()
    N = args.voxels
    # each rank fits its own shard (weak scaling): seeds differ per rank
    true, data, init, lb, ub, prot = w.generate(N, seed=1000 + rank)
    solve = torch.float64 if args.solve == "f64" else torch.float32
    expr = Expr(w.expr, w.pars, w.consts)
    solm = SecondOrderLevenbergMarquardt(expr, None, w.M, torch.float32, solve_dtype=solve)

    data_d = torch.from_numpy(data).to(dev)
    init_d = torch.from_numpy(init).to(dev)
    prot_d = torch.from_numpy(prot).to(dev)
    lb_d = torch.from_numpy(lb).to(dev)
    ub_d = torch.from_numpy(ub).to(dev)
    pars_d = init_d.clone()
    solm.setup(pars_d, prot_d, data_d, lb_d, ub_d)
    stream = torch.cuda.current_stream()

    def reset():
        pars_d.copy_(init_d)
        solm.lam_t.fill_(5.0)
        solm.step_type_t.fill_(1)
        solm.f_t.zero_()
        solm.iters_t.zero_()

    # ---- device-resident timing -------------------------------------------
    for _ in range(args.warmup):
        reset()
        solm.run(args.iters, block=args.block)
    torch.cuda.synchronize()
    k_start = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    k_end = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    t_start = torch.cuda.Event(enable_timing=True)
    t_end = torch.cuda.Event(enable_timing=True)
    if ws > 1:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        t_start.record(stream)
        for s in range(args.steps):
            reset()
            k_start[s].record(stream)
            solm.run(args.iters, block=args.block)
            k_end[s].record(stream)
        t_end.record(stream)
        torch.cuda.synchronize()
    if ws > 1:
        dist.barrier()
    step_ms = t_start.elapsed_time(t_end) / args.steps
    kern_ms = statistics.mean(k_start[s].elapsed_time(k_end[s]) for s in range(args.steps))
    step_ms, kern_ms = max_over_ranks([step_ms, kern_ms], device=dev)
    fitted = pars_d.cpu().numpy()
    st = solm.step_type_t.cpu().numpy()[0]
    its = solm.iters_t.cpu().numpy()[0].astype(np.int64)

    # ---- end to end through the public API from pinned host buffers -------
    data_h = torch.from_numpy(data).pin_memory()
    init_h = torch.from_numpy(init).pin_memory()
    out_pars_h = torch.empty_like(init_h).pin_memory()
    out_st_h = torch.empty((1, N), dtype=torch.int8).pin_memory()
    data_e = torch.empty_like(data_d)
    pars_e = torch.empty_like(init_d)
    solm_e = SecondOrderLevenbergMarquardt(expr, None, w.M, torch.float32, solve_dtype=solve)

    def e2e_step():
        data_e.copy_(data_h, non_blocking=True)
        pars_e.copy_(init_h, non_blocking=True)
        solm_e.setup(pars_e, prot_d, data_e, lb_d, ub_d)
        solm_e.run(args.iters, block=args.block)
        out_pars_h.copy_(pars_e, non_blocking=True)
        out_st_h.copy_(solm_e.step_type_t, non_blocking=True)

    for _ in range(max(1, args.warmup)):
        e2e_step()
    torch.cuda.synchronize()
    if ws > 1:
        dist.barrier()
    e_start = torch.cuda.Event(enable_timing=True)
    e_end = torch.cuda.Event(enable_timing=True)
    e_start.record(stream)
    for _ in range(args.steps):
        e2e_step()
    e_end.record(stream)
    torch.cuda.synchronize()
    e2e_ms = max_over_ranks([e_start.elapsed_time(e_end) / args.steps], device=dev)[0]
    assert np.array_equal(out_pars_h.numpy(), fitted), "e2e result differs from the device-resident run"
    h2d = data.nbytes + init.nbytes
    d2h = init.nbytes + N

    # ---- accuracy against the all-FP64 fitter (untimed) -------------------
    acc = None
    if not args.no_fp64_check:
        solm64 = SecondOrderLevenbergMarquardt(expr, None, w.M, torch.float64)
        p64 = init_d.double()
        solm64.setup(p64, prot_d.double(), data_d.double(), lb_d.double(), ub_d.double())
        t0 = time.perf_counter()
        solm64.run(args.iters)
        torch.cuda.synchronize()
        t64 = time.perf_counter() - t0
        rep = parity.compare_params(fitted, p64.cpu().numpy())
        acc = {"vs": "all-FP64 GPU fitter, same LM and init", "median_rel_err": rep["median_rel"],
               "frac_voxels_gt_1e-4": rep["frac_gt_1e-4"], "per_param_median": rep["per_param_median"],
               "converged_frac_fp64": float(np.mean(solm64.step_type_t.cpu().numpy() == 0)),
               "fp64_fit_s": round(t64, 3)}
        del p64, solm64

    # ---- fits/s at the budget that reaches 1e-4 median error vs FP64 -------
    at_tol = None
    if not args.no_fp64_check:
        ref64 = fp64_reference(w, data_d)

        def run_k(k):
            reset()
            solm.run(k, block=args.block)
            return pars_d

        k_tol, curve = budget_for_tolerance(run_k, ref64, range(2, 41))
        at_tol = {"iters": k_tol, "curve": {k: v[0] for k, v in curve.items()}}
        if k_tol is not None:
            ms = _time_ms(lambda: run_k(k_tol))
            at_tol["fits_per_s"] = ws * N / (ms / 1e3)
        del ref64

    warm = None
    if rank == 0 and ws == 1 and not args.no_warm:
        warm = warm_start_comparison(n_eval=args.warm_voxels, epochs=args.warm_epochs, lam0=args.warm_lam0,
                                     n_train=args.warm_train)

    mixed = None
    if rank == 0 and ws == 1 and not args.no_mixed:
        mixed = mixed_batch_comparison()

    # ---- CPU baseline (rank 0, N=1 only) ----------------------------------
    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu:
        par = {}
        v, kind, cores, sample = cpu_sample(args.iters, target_s=args.cpu_seconds, parity_out=par)
        cpu = {"value": v, "unit": "fits/s", "cores": cores, "kind": kind, "sample": sample, "gpu_parity": par}

    if rank == 0:
        hbm, peak_kind = _peaks()
        bytes_per_voxel = 4 * M_IVIM10 + 4 * P_IVIM + 1
        achieved = bytes_per_voxel * N / (kern_ms / 1e3) / 1e9
        traffic = None
        tf = os.path.join(ROOT, "profiles", "lm_ivim10_traffic.json")
        if os.path.exists(tf):
            with open(tf) as f:
                tr = json.load(f)
            traffic = tr["dram_bytes_per_voxel"] * N
        value = ws * N / (step_ms / 1e3)
        line = {
            "metric": "IVIM voxel fits/s (plain LM, 100 iters max)", "value": value, "unit": "fits/s",
            "n_gpus": ws, "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 (f64 GMW81 solve + gain ratio)" if args.solve == "f64" else "f32",
            "data": "synthetic (seeded IVIM-10, Rician SNR 50)",
            "config": {"workload": "ivim10_plain_lm_8.4M", "voxels_per_gpu": N, "ndata": M_IVIM10,
                       "nparam": P_IVIM, "iters": args.iters, "solve": args.solve, "init": "constant",
                       "l2": "inputs larger than L2 (335 MB signals)", "parallelism": f"voxel shards x{ws}"},
            "e2e": {"value": ws * N / (e2e_ms / 1e3), "unit": "fits/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "ms_per_step": e2e_ms},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                         "frac": achieved / hbm, "traffic": traffic, "peak_source": peak_kind,
                         "algorithmic_bytes_per_voxel": bytes_per_voxel,
                         "note": "iterative per-voxel solver: FP64/FP32 issue bound, not HBM bound"},
            "kernel_ms": kern_ms,
            "fit_stats": {"mean_iters": float(its.mean()), "converged_frac": float(np.mean(st == 0)),
                          "voxel_iters_per_s": float(its.sum()) * ws / (kern_ms / 1e3)},
            "accuracy": acc,
            "at_1e-4_vs_fp64": at_tol,
            "warm_start": warm,
            "mixed_batch": mixed,
            "cpu_baseline": cpu,
            "gpu_launches": args.steps,
            "clocks": clk.summary(),
        }
        print(json.dumps(line), flush=True)
    if ws > 1:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
