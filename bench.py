"""Benchmark: IVIM voxel fits/s at 1e-4 relative error vs FP64, MLP warm start
vs plain LM, on GB300.

Headline workload: IVIM bi-exponential, 4 parameters, 16 b-values (0-1000
s/mm^2, log-spaced above 10), 16,777,216 voxels, seeded synthetic signals
(uniform true parameters S0 in [500, 1500], f in [0.05, 0.35], D* in
[5e-3, 5e-2], D in [0.5e-3, 2.5e-3], Rician noise sigma = S0/50), fp32 state
with the GMW81 solve and gain-ratio test in fp64.

Untimed setup: the warm-start network (16 -> 128 -> 128 -> 128 -> 4, GELU,
bf16 weights, fp32 accumulation) is trained on 2,097,152 other synthetic
signals with the plain LM's converged fits as labels; the all-FP64 fit (same
LM, constant start, 300 iterations, tolerance 1e-30) of the evaluation voxels
is the error reference; for each method the iteration budget is the smallest
whose median relative error (per voxel the worst parameter) is <= 1e-4.

One step = one fit of every voxel at that budget:
  warm start   network -> LM (k_warm iterations from lambda 3e-3) -> fused
               fallback check -> plain-LM refit of flagged voxels on a device
               list -> keep the lower cost (WarmStartFitter.fit)
  plain LM     constant start -> LM (k_plain iterations), reported beside it
Inputs (1.07 GB of signals) are larger than L2 (129 MB): no flush needed.

Reported (one JSON line from rank 0):
  value         warm-start fits/s with inputs resident in HBM (whole job)
  plain_lm      plain-LM fits/s at its own 1e-4 budget, and the speedup
  e2e           warm-start fits/s through the public API
                (WarmStartFitter.fit_stream over the timed steps): every step
                copies all of its signals in from pinned host memory and all
                of its fitted parameters back, overlapped with the
                neighbouring steps' fits; single_volume = one volume alone
                through fit_host (chunks whose copies overlap the previous
                chunk's fit)
  roofline      the LM kernel of the warm step (the dominant kernel):
                algorithmic bytes 4M + 8P + 1 per voxel (signals in,
                parameters in and out, status) over its event-timed duration,
                against the measured copy bandwidth; roofline_network the
                tensor-core network kernel against measured bf16 throughput
  cpu_baseline  the reference algorithm (plain LM, fp32) on the host cores at
                its own 1e-4 budget on a bounded IVIM-16 sample
  plain_lm_ivim10_8.4M  the plain LM at scale (IVIM-10, 8,388,608 voxels,
                100 iterations) with its accuracy against the FP64 fitter
  mixed_batch   four models in one persistent launch vs one launch per model,
                with each model's accuracy against the all-FP64 fitter
  precision_stress  ill-conditioned IVIM-10 (SNR 10-20, small f): per-parameter
                error quantiles of the FP64-solve and fp32-solve fitters
                against the all-FP64 fitter

`--impl reference` runs the reference arm: the reference algorithm on the host
cores (its own generated kernel built for the host when available, else the
CPU oracle in the reference's fp32 arithmetic) at its 1e-4 budget, one bounded
sample per step; where its generated kernel was also built for the GPU, the
line adds that kernel's fits/s on this GPU, launched as the reference's run()
does (`gpu_reference_kernel`, informational).
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
M_IVIM16 = 16
P_IVIM = 4
TOL = 1e-4
METRIC = "IVIM voxel fits/s at 1e-4 rel err vs FP64: MLP-warm-start vs plain LM, 1 GB300"
# network FLOPs per voxel: 2 * (16*128 + 128*128 + 128*128 + 128*4)
NET_FLOP_PER_VOXEL = 2 * (16 * 128 + 2 * 128 * 128 + 128 * 4)
# Binding-unit work per unit, from ncu opcode counts (sass__inst_executed per
# opcode over one launch, divided by the units it processed): FP64-pipe
# instructions (56 DFMA + 24 DMUL + 2 DADD) per IVIM-16 voxel-iteration of the
# FP64-solve warm LM (4,194,304 warm-started voxels x 3 iterations) and MUFU
# instructions per voxel of the tcgen05 network (1,048,576 IVIM-16 voxels;
# 240 tanh for the 240 activations of the tanh columns, 16 log, 3 exp/rcp).
FP64_OPS_PER_VOXEL_ITER = 82
MUFU_PER_VOXEL_NET = 259
# issue rates per SM per clock on sm_103a: FP64 at 1/64 of the 128 FP32 lanes,
# MUFU 16 lanes
FP64_PER_SM_CLK = 2
MUFU_PER_SM_CLK = 16


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            pk = json.load(f)
        return float(pk["hbm_gbs"]), float(pk["bf16_tflops"]), "measured"
    except Exception:
        return 6800.0, 1900.0, "fallback"


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
                                          "-lms", "100", "-i", str(self.gpu)], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            # nvidia-smi's start-up (driver queries) is kept out of the timed
            # region: the caller's work starts once the first sample has
            # arrived, and callers enter the sampler before their warm-up
            t0 = time.perf_counter()
            while not self.lines and self.proc.poll() is None and time.perf_counter() - t0 < 5.0:
                time.sleep(0.01)
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
        return {"sm_mhz": statistics.median(sm), "sm_mhz_min": min(sm), "sm_max_mhz": max(mx),
                "reasons": sorted(reasons), "samples": len(sm)}


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


# ---- CPU reference ------------------------------------------------------------

def _median_rel_np(a, b):
    """Median over voxels of the worst per-parameter relative error, and the
    fraction of voxels above 1e-4 (the GPU helper's definition)."""
    r = np.abs(a.astype(np.float64) - b.astype(np.float64)) / np.maximum(np.abs(b.astype(np.float64)), 1e-30)
    r = np.nan_to_num(r, nan=np.inf).max(axis=0)
    return float(np.median(r)), float(np.mean(r > TOL))


_CPU_INPUTS = {}  # the timed sample's host inputs, kept for the repeated timings


def cpu_reference_at_tol(target_s: float, n_ref: int = 16384, max_iters: int = 30, plan: dict | None = None,
                         n_fixed: int | None = None):
    """The reference algorithm (plain LM, fp32) on the host cores, on IVIM-16
    at the smallest iteration budget whose median error against the all-FP64
    CPU fit (same LM, constant start, 300 iterations) is <= 1e-4. The sample
    grows until one fit takes at least target_s / 4 (or is ``n_fixed`` voxels);
    that size is timed once. With ``plan`` (the result of an earlier call) the
    budget and the sample size are reused and only the timed fit runs again
    (on the inputs made by the first call).
    """
    from oracle import OracleModel, RefIVIM, ref_available
    from pycompute_gb300 import synth

    w = synth.ivim(synth.ivim_b16(), name="ivim16")
    cores = os.cpu_count() or 1
    port = OracleModel(w.expr, w.pars, w.consts)
    port.set_threads(cores)
    if ref_available(M_IVIM16):
        impl, kind = RefIVIM(M_IVIM16), "reference"
    else:
        impl, kind = port, "port"
    if plan is not None:
        k_run, n = plan["iters"], plan["n"]
        data, init, lb, ub, prot = _CPU_INPUTS[n]
        p = init.copy()
        t0 = time.perf_counter()
        impl.lm_run(p, prot, data, lb, ub, k_run)
        el = time.perf_counter() - t0
        return dict(plan, value=n / el, sample=plan["sample"].rsplit(", ", 1)[0] + f", {el:.2f} s")
    _, data, init, lb, ub, prot = w.generate(n_ref, seed=7)
    p64 = init.astype(np.float64)
    port.lm_run(p64, prot.astype(np.float64), data.astype(np.float64), lb.astype(np.float64),
                ub.astype(np.float64), 300, tol=1e-30)
    curve, k_tol = {}, None
    for k in range(1, max_iters + 1):
        p = init.copy()
        impl.lm_run(p, prot, data, lb, ub, k)
        curve[k] = _median_rel_np(p, p64)[0]
        if curve[k] <= TOL:
            k_tol = k
            break
    k_run = k_tol if k_tol is not None else max_iters
    n = n_fixed or (1 << 16)
    while True:
        _, data, init, lb, ub, prot = w.generate(n, seed=8)
        p = init.copy()
        t0 = time.perf_counter()
        impl.lm_run(p, prot, data, lb, ub, k_run)
        el = time.perf_counter() - t0
        if n_fixed or el >= target_s / 4 or n >= (1 << 23):
            break
        n *= 2 if el > 0.05 else 8
    _CPU_INPUTS.clear()
    _CPU_INPUTS[n] = (data, init, lb, ub, prot)
    what = "reference generated kernel" if kind == "reference" else "fp32 oracle port"
    sample = (f"{n} IVIM-16 voxels x {k_run} iterations (the 1e-4 budget on {n_ref} voxels vs the all-FP64 CPU fit; "
              f"{what}, {cores} threads), {el:.2f} s")
    return {"value": n / el, "unit": "fits/s", "cores": cores, "kind": kind, "sample": sample, "iters": k_run,
            "curve": curve, "n": n}


def cpu_parity_ivim10(n: int = 1 << 18, iters: int = 100):
    """The GPU fitter against the reference algorithm on the host, same IVIM-10
    inputs: parameter agreement and convergence flags (step_type == 0)."""
    import torch
    from oracle import OracleModel, RefIVIM, ref_available
    from pycompute_gb300 import Expr, SecondOrderLevenbergMarquardt, parity, synth

    w = synth.ivim()
    if ref_available(M_IVIM10):
        impl, kind = RefIVIM(M_IVIM10), "reference"
    else:
        impl, kind = OracleModel(w.expr, w.pars, w.consts), "port"
        impl.set_threads(os.cpu_count() or 1)
    _, data, init, lb, ub, prot = w.generate(n, seed=7)
    p_cpu = init.copy()
    st_cpu = impl.lm_run(p_cpu, prot, data, lb, ub, iters)["step_type"]
    out = {"cpu": kind, "voxels": n, "iters": iters}
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


def parity_c2(n: int = 256 * 256 * 128, iters: int = 100):
    """The checker at the plain-LM-at-scale size (IVIM-10, 8,388,608 voxels,
    100 iterations): the fitter against the reference's own generated kernel
    (oracle/_ref, built from the reference tree for sm_103a, launched as its
    run() does) on the same voxels, both free-running and in lockstep, and
    both against the all-FP64 fitter (same LM, same start, 100 iterations,
    tol 1e-8). Not timed."""
    import torch
    from oracle import lockstep, ref_gpu
    from pycompute_gb300 import Expr, SecondOrderLevenbergMarquardt, parity, pipeline, synth

    w = synth.ivim()
    if not ref_gpu.available(w.M):
        return {"unavailable": "oracle/_ref cubin not built (no reference tree where build() ran)"}
    dev = torch.device("cuda", torch.cuda.current_device())
    _, data = pipeline.synth_gpu(w, n, seed=2024, device=dev)
    init = pipeline.init_constant(data, w.init_values)
    prot = torch.tensor(w.protocol, device=dev)
    lb_t, ub_t = torch.tensor(w.lb, device=dev), torch.tensor(w.ub, device=dev)
    tile = lambda v, k: v[:, None].expand(k, n).contiguous()  # noqa: E731

    def reference(lockstep_with=None):
        r = ref_gpu.RefGpuIVIM(w.M)
        p = init.clone()
        r.setup(p, tile(prot, w.M), data, tile(lb_t, 4), tile(ub_t, 4))
        if lockstep_with is None:
            r.run(iters)
            torch.cuda.synchronize()
            return r, None
        s = lockstep_with
        s.setup(init.clone(), list(w.protocol), data, list(w.lb), list(w.ub))
        per = lockstep.lockstep_gpu(r, s, iters, w.protocol, w.lb, w.ub)
        return r, lockstep.summarise(per)

    def ours(dtype, solve):
        s = SecondOrderLevenbergMarquardt(Expr(w.expr, w.pars, w.consts), None, w.M, dtype, solve_dtype=solve)
        p = init.to(dtype).clone()
        s.setup(p, list(w.protocol), data.to(dtype), list(w.lb), list(w.ub))
        s.run(iters)
        torch.cuda.synchronize()
        return p, s.step_type_t[0].clone()

    r, _ = reference()
    p_ref, st_ref = r.pars.clone(), r.step_type[0].clone()
    del r
    p64, st64 = ours(torch.float64, torch.float64)
    mask = (st64 == 0) & torch.all((p64 > lb_t.double()[:, None] * (1 + 1e-6) + 1e-30) &
                                   (p64 < ub_t.double()[:, None] * (1 - 1e-6)), dim=0)
    out = {"workload": "ivim10_8.4M (C2), 100 iterations", "voxels": n,
           "reference": "the reference's generated LM kernel for sm_103a (oracle/_ref)",
           "fp64_fit": "all-FP64 fitter, same LM and start, 100 iterations, tol 1e-8",
           "fp64_converged_interior_voxels": int(mask.sum())}

    def block(p, st):
        med, frac = _median_rel_gpu(p, p_ref)
        medm, fracm = _median_rel_gpu(p[:, mask], p_ref[:, mask])
        m64, f64 = _median_rel_gpu(p[:, mask], p64[:, mask])
        conv_o, conv_r = st == 0, st_ref == 0
        both = int((conv_o & conv_r).sum())
        return {"vs_reference": {"median_rel_err": med, "frac_voxels_gt_1e-4": frac,
                                 "fp64_converged_interior": {"median_rel_err": medm, "frac_voxels_gt_1e-4": fracm}},
                "vs_fp64_on_fp64_converged_interior": {"median_rel_err": m64, "frac_voxels_gt_1e-4": f64},
                "flags_agree": float((conv_o == conv_r).double().mean()),
                "converged": int(conv_o.sum()), "converged_reference": int(conv_r.sum()),
                "converged_recall": both / max(1, int(conv_r.sum())),
                "converged_precision": both / max(1, int(conv_o.sum()))}

    m64r, f64r = _median_rel_gpu(p_ref[:, mask], p64[:, mask])
    out["reference_vs_fp64_on_fp64_converged_interior"] = {"median_rel_err": m64r, "frac_voxels_gt_1e-4": f64r}
    for name, solve in (("f32_state_f64_solve", torch.float64), ("f32_state_f32_solve", torch.float32)):
        p, st = ours(torch.float32, solve)
        out[name] = block(p, st)
        del p
        s = SecondOrderLevenbergMarquardt(Expr(w.expr, w.pars, w.consts), None, w.M, torch.float32, solve_dtype=solve)
        r, ls = reference(lockstep_with=s)
        out[name]["lockstep"] = ls
        del r, s
        torch.cuda.empty_cache()
    return out


# ---- GPU helpers -------------------------------------------------------------

def _median_rel_gpu(a, b):
    """Median over voxels of the worst per-parameter relative error (on the GPU)."""
    import torch
    r = (a.double() - b.double()).abs() / b.double().abs().clamp_min(1e-30)
    r = torch.nan_to_num(r, nan=float("inf")).amax(dim=0)
    return float(r.median()), float((r > TOL).double().mean())


def _per_param_median(a, b):
    r = (a.double() - b.double()).abs() / b.double().abs().clamp_min(1e-30)
    return [float(x) for x in r.median(dim=1).values]


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


def budget_for_tolerance(run_with, ref, budgets, tol=TOL):
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


def _unit_roofline(ops, ms, per_sm_clk, clocks, source):
    """Achieved vs peak issue rate of one execution unit (instructions per
    second over all SMs at the SM clock sampled under load)."""
    import torch
    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    mhz = (clocks or {}).get("sm_mhz") or (clocks or {}).get("sm_max_mhz") or 2070.0
    peak = per_sm_clk * sms * mhz * 1e6
    achieved = ops / (ms / 1e3)
    return {"achieved": achieved, "peak": peak, "unit": "instructions/s", "frac": achieved / peak,
            "work_source": source, "peak_source": f"{per_sm_clk} per SM per clock x {sms} SMs x {mhz:.0f} MHz"}


def _stage_ms(events, a, b):
    """Elapsed ms between the events named a and b of one fit's event list."""
    d = dict(events)
    return d[a].elapsed_time(d[b])


def fallback_rule_report(run_warm, run_pre, run_plain, plain, k_warm, k_plain, ref, w, N):
    """The implemented fallback rule against the one that needs the plain fit.

    The pipeline refits a voxel when its warm fit lands on a bound, has a
    non-finite cost, or does not end below the cost at the plain fitter's
    constant start. The rule that compares with the plain fit's own final
    cost needs the plain fit of every voxel, which is what the warm start
    avoids. Here (outside every timed region) the plain LM runs at its 1e-4
    budget on all voxels; the report counts the voxels the implemented rule
    leaves unflagged whose warm cost ends above the plain fit's (strictly, and
    by more than relative margins at and above the cost's fp32 resolution),
    and the accuracy against the FP64 fit of the pipeline as run and of the
    pipeline with the plain-cost rule applied on top (each such voxel taking
    the plain fit). The flagged voxels are split by the criterion that flags
    them, with the share whose refit is kept."""
    import torch

    pre_pars, pre_cost, const_cost = run_pre(k_warm)
    lo = torch.tensor(w.lb, device=pre_pars.device)[:, None]
    hi = torch.tensor(w.ub, device=pre_pars.device)[:, None]
    on_bound = ((pre_pars <= lo) | (pre_pars >= hi)).any(0)
    cost_bad = ~torch.isfinite(pre_cost) | ~(pre_cost < const_cost)
    res = run_warm(k_warm)
    w_pars, w_cost = res.pars.clone(), res.cost.clone()
    n_fb = res.n_fallback
    flagged = torch.zeros(N, dtype=torch.bool, device=w_pars.device)
    if n_fb:
        flagged[res.fallback_idx[:n_fb].long()] = True
    kept = flagged & (w_pars != pre_pars).any(0)
    p_pl = run_plain(k_plain).clone()
    c_pl = plain.cost()
    unflagged = ~flagged
    cls = {}
    for name, m in (("bound_only", on_bound & ~cost_bad), ("cost_only", cost_bad & ~on_bound),
                    ("bound_and_cost", on_bound & cost_bad)):
        cls[name] = {"voxels": int(m.sum()), "refit_kept": int((m & kept).sum())}
    out = {"voxels": N, "flagged": int(flagged.sum()), "flagged_by": cls,
           "flag_classes_consistent": bool(torch.equal(flagged, on_bound | cost_bad)),
           "rule": "refit when the warm fit's cost is not finite or not below the cost at the constant start, "
                   "or a parameter is on a bound"}
    worse = {}
    for name, margin in (("strict", 0.0), ("rel_1e-6", 1e-6), ("rel_1e-5", 1e-5), ("rel_1e-4", 1e-4),
                         ("rel_1e-3", 1e-3)):
        m = unflagged & (w_cost > c_pl * (1.0 + margin))
        worse[name] = int(m.sum())
    out["unflagged_warm_cost_above_plain"] = worse
    out["unflagged_frac_above_plain_rel_1e-4"] = worse["rel_1e-4"] / N
    med, frac = _median_rel_gpu(w_pars, ref)
    above = unflagged & (w_cost > c_pl)
    ideal = torch.where(above[None], p_pl, w_pars)
    med_i, frac_i = _median_rel_gpu(ideal, ref)
    out["accuracy_as_run"] = {"median_rel_err": med, "frac_voxels_gt_1e-4": frac}
    out["accuracy_with_plain_cost_rule"] = {"median_rel_err": med_i, "frac_voxels_gt_1e-4": frac_i}
    for name, margin in (("rel_1e-4", 1e-4), ("rel_1e-2", 1e-2)):
        big = unflagged & (w_cost > c_pl * (1.0 + margin))
        if int(big.sum()):
            ew = _median_rel_gpu(w_pars[:, big], ref[:, big])
            ep = _median_rel_gpu(p_pl[:, big], ref[:, big])
            out[f"voxels_above_plain_{name}"] = {"voxels": int(big.sum()), "warm_median_rel_err": ew[0],
                                                 "warm_frac_gt_1e-4": ew[1], "plain_median_rel_err": ep[0],
                                                 "plain_frac_gt_1e-4": ep[1]}
    # candidate proxies for "the warm fit ends above the plain fit's cost":
    # the last warm iteration still lowered the cost by more than delta
    # (relative); newly flagged voxels would be refitted and keep the lower
    # cost of the two fits (the select), which is evaluated here directly
    if k_warm >= 1:
        _, c_prev, _ = run_pre(k_warm - 1) if k_warm > 1 else (None, const_cost, None)
        target = unflagged & (w_cost > c_pl * (1.0 + 1e-4))
        prox = {}
        for delta in (1e-2, 1e-3, 1e-4, 1e-5):
            extra = unflagged & ((c_prev - pre_cost) > delta * pre_cost)
            take = extra & (c_pl < w_cost)
            med_x, frac_x = _median_rel_gpu(torch.where(take[None], p_pl, w_pars), ref)
            prox[f"last_iter_drop_gt_{delta:g}"] = {
                "extra_flagged": int(extra.sum()), "extra_flagged_frac": float(extra.double().mean()),
                "recall_of_above_plain_rel_1e-4": float((extra & target).sum()) / max(1, int(target.sum())),
                "accuracy_if_refitted": {"median_rel_err": med_x, "frac_voxels_gt_1e-4": frac_x}}
        out["proxies"] = prox
    del p_pl, ideal, pre_pars
    return out


# ---- headline: warm start vs plain LM at 1e-4 -----------------------------------

def warm_headline(args, ws, rank, local, dev):
    """IVIM-16: network + LM + fallback vs plain LM, both at their 1e-4 budgets."""
    import torch
    import torch.distributed as dist
    from pycompute_gb300 import Expr, SecondOrderLevenbergMarquardt, pipeline, synth
    from pycompute_gb300.shard import max_over_ranks
    from pycompute_gb300.warmstart import WarmStartMLP

    w = synth.ivim(synth.ivim_b16(), name="ivim16")
    expr = Expr(w.expr, w.pars, w.consts)
    N = args.warm_voxels
    t0 = time.perf_counter()
    # training set: other synthetic signals, labels = the plain LM's converged fits
    _, tr = pipeline.synth_gpu(w, args.warm_train, seed=77 + 1000 * rank, device=dev)
    lab = pipeline.init_constant(tr, w.init_values)
    s = SecondOrderLevenbergMarquardt(expr, None, w.M, torch.float32)
    s.setup(lab, list(w.protocol), tr, list(w.lb), list(w.ub))
    s.run(100)
    net = WarmStartMLP(16, 4, [0, 1, 2, 2], w.lb, w.ub, dev, seed=77)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    net.train(tr, lab, epochs=args.warm_epochs, batch=8192, lr=args.warm_lr)
    torch.cuda.synchronize()
    train_s = time.perf_counter() - t1
    del tr, lab, s
    # evaluation voxels (each rank its own shard) and their FP64 reference
    _, data = pipeline.synth_gpu(w, N, seed=78 + 1000 * rank, device=dev)
    ref = fp64_reference(w, data, iters=300)
    pars = torch.empty((4, N), device=dev)
    plain = SecondOrderLevenbergMarquardt(expr, None, w.M, torch.float32)

    def run_plain(k):
        pipeline.init_constant(data, w.init_values, out=pars)
        plain.setup(pars, list(w.protocol), data, list(w.lb), list(w.ub))
        plain.run(k)
        return pars

    wf = pipeline.WarmStartFitter(w, net)
    lam0 = args.warm_lam0
    k_plain, curve_plain = budget_for_tolerance(run_plain, ref, range(1, 31))
    k_fb = k_plain or 30

    def run_warm(k, data_in=data, out=pars, events=None):
        return wf.fit(data_in, iters_warm=k, iters_fallback=k_fb, pars_out=out, lam0=lam0, events=events)

    k_warm, curve_warm = budget_for_tolerance(lambda k: run_warm(k).pars, ref, range(0, 21))
    setup_s = time.perf_counter() - t0
    if k_warm is None or k_plain is None:
        raise RuntimeError(f"no budget reached {TOL}: plain {curve_plain}, warm {curve_warm}")

    # ---- timed: warm-start steps, device resident --------------------------
    stream = torch.cuda.current_stream()
    step_events = []
    t_start, t_end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    # the sampler runs from before the warm-up steps, so its start-up is over
    # before the timed steps begin
    with ClockSampler(local) as clk:
        for _ in range(args.warmup):
            run_warm(k_warm)
        torch.cuda.synchronize()
        if ws > 1:
            dist.barrier()
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_push("warm_steps")  # lets a profiler select the timed launches
        t_start.record(stream)
        for _ in range(args.steps):
            ev = []
            res = run_warm(k_warm, events=ev)
            step_events.append(ev)
        t_end.record(stream)
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_pop()
    if ws > 1:
        dist.barrier()
    step_ms = t_start.elapsed_time(t_end) / args.steps
    stages = {}
    for a, b in (("start", "network"), ("network", "setup"), ("setup", "lm_warm"), ("lm_warm", "check"),
                 ("check", "refit"), ("refit", "select")):
        stages[b] = statistics.mean(_stage_ms(ev, a, b) for ev in step_events)
    step_ms, lm_ms, net_ms = max_over_ranks([step_ms, stages["lm_warm"], stages["network"]], device=dev)
    med_w, frac_w = _median_rel_gpu(res.pars, ref)
    pp_w = _per_param_median(res.pars, ref)
    warm_pars_h = res.pars.cpu()
    n_fb, n_kept = res.n_fallback, res.n_refit_kept

    # ---- plain LM at its budget, same voxels --------------------------------
    plain_ms = _time_ms(lambda: run_plain(k_plain), warmup=max(1, args.warmup), reps=args.steps)
    plain_ms = max_over_ranks([plain_ms], device=dev)[0]
    p_plain = run_plain(k_plain)
    med_p, frac_p = _median_rel_gpu(p_plain, ref)
    pp_p = _per_param_median(p_plain, ref)

    # ---- the fallback rule against the plain fit's cost (untimed) -------------
    def run_pre(k):
        """The warm fit before the fallback: parameters, cost, and the cost at
        the constant start (the quantities the fallback check reads)."""
        p = net.infer(data).clone()
        s = SecondOrderLevenbergMarquardt(expr, None, w.M, torch.float32)
        s.setup(p, list(w.protocol), data, list(w.lb), list(w.ub))
        s.lam_t.fill_(lam0)
        s.run(k)
        c = s.cost()
        c0 = s.cost(pipeline.init_constant(data, w.init_values))
        return p, c, c0

    fb_rule = fallback_rule_report(run_warm, run_pre, run_plain, plain, k_warm, k_plain, ref, w, N)

    # ---- the reference's own data-driven start (the IVIM notebook's segmented
    # log-linear fits: b <= 100 and b >= 193 s/mm^2), same fixed bounds ---------
    def run_seg(k):
        p0, _, _ = pipeline.ivim_segmented_init(data, w.protocol, (0, 9), (10, 16), w.lb, w.ub, bounds=False)
        pars.copy_(p0)
        plain.setup(pars, list(w.protocol), data, list(w.lb), list(w.ub))
        plain.run(k)
        return pars

    k_seg, curve_seg = budget_for_tolerance(run_seg, ref, range(0, 31))
    seg = {"iters_for_1e-4": k_seg, "curve": {k: v[0] for k, v in curve_seg.items()}}
    if k_seg is not None:
        seg_ms = max_over_ranks([_time_ms(lambda: run_seg(k_seg), warmup=1, reps=args.steps)], device=dev)[0]
        seg.update({"fits_per_s": ws * N / (seg_ms / 1e3), "ms_per_step": seg_ms})

    # ---- end to end through the public API from pinned host buffers ---------
    # WarmStartFitter.fit_stream fits the steps as a sequence of host-resident
    # volumes: every step copies all of its signals in and all of its fitted
    # parameters out, overlapped with the neighbouring steps' fits (two device
    # slots). The timed region holds every copy of every step.
    data_h = data.cpu().pin_memory()
    outs = [torch.empty((4, N), dtype=torch.float32).pin_memory() for _ in range(2)]

    def e2e_steps(k):
        return wf.fit_stream([(data_h, outs[i % 2]) for i in range(k)], iters_warm=k_warm, iters_fallback=k_fb,
                             lam0=lam0)

    e_start, e_end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as e2e_clk:  # started before the warm-up volumes (see the device steps)
        e2e_steps(max(2, args.warmup))
        torch.cuda.synchronize()
        if ws > 1:
            dist.barrier()
        e_start.record(stream)
        e2e_steps(args.steps)
        e_end.record(stream)
        torch.cuda.synchronize()
    e2e_ms = max_over_ranks([e_start.elapsed_time(e_end) / args.steps], device=dev)[0]
    e2e_same = bool(torch.equal(outs[(args.steps - 1) % 2], warm_pars_h))
    # the host link's own rates right after the timed region (copies alone,
    # nothing else running): the end-to-end step is bound by them when they
    # exceed the fit (the link is shared with the machine's other GPUs)
    link = {}
    dbuf = torch.empty_like(data)
    for name, fn, nbytes in (("h2d_gbs", lambda: dbuf.copy_(data_h, non_blocking=True), data_h.nbytes),
                             ("d2h_gbs", lambda: outs[0].copy_(pars, non_blocking=True), outs[0].nbytes)):
        fn()
        torch.cuda.synchronize()
        l0, l1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        l0.record(stream)
        for _ in range(3):
            fn()
        l1.record(stream)
        torch.cuda.synchronize()
        link[name] = 3 * nbytes / (l0.elapsed_time(l1) / 1e3) / 1e9
    # the two directions run at the same time in the stream
    link["h2d_ms_per_step"] = data_h.nbytes / link["h2d_gbs"] / 1e6
    link["d2h_ms_per_step"] = outs[0].nbytes / link["d2h_gbs"] / 1e6
    del dbuf
    # one volume on its own, streamed in chunks (WarmStartFitter.fit_host)
    wf.fit_host(data_h, outs[0], iters_warm=k_warm, iters_fallback=k_fb, lam0=lam0, chunks=args.e2e_chunks)
    torch.cuda.synchronize()
    e1_start, e1_end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e1_start.record(stream)
    for _ in range(3):
        wf.fit_host(data_h, outs[0], iters_warm=k_warm, iters_fallback=k_fb, lam0=lam0, chunks=args.e2e_chunks)
    e1_end.record(stream)
    torch.cuda.synchronize()
    e2e_single_ms = max_over_ranks([e1_start.elapsed_time(e1_end) / 3], device=dev)[0]

    return {
        "N": N, "step_ms": step_ms, "plain_ms": plain_ms, "e2e_ms": e2e_ms, "lm_ms": lm_ms, "net_ms": net_ms,
        "e2e_single_ms": e2e_single_ms, "host_link": link,
        "stages": stages, "clocks": clk.summary(), "e2e_clocks": e2e_clk.summary(), "h2d": data_h.nbytes,
        "d2h": outs[0].nbytes,
        "k_warm": k_warm, "k_plain": k_plain, "e2e_same": e2e_same, "e2e_chunks": args.e2e_chunks,
        "detail": {
            "train_voxels": args.warm_train, "epochs": args.warm_epochs, "lr": args.warm_lr, "train_s": round(train_s, 3),
            "setup_s": round(setup_s, 1), "lam0": lam0,
            "warm_curve": {k: v[0] for k, v in curve_warm.items()},
            "plain_curve": {k: v[0] for k, v in curve_plain.items()},
            "warm_accuracy": {"median_rel_err": med_w, "frac_voxels_gt_1e-4": frac_w, "per_param_median": pp_w},
            "plain_accuracy": {"median_rel_err": med_p, "frac_voxels_gt_1e-4": frac_p, "per_param_median": pp_p},
            "fallback_voxels": n_fb, "refits_kept": n_kept, "fallback_rule": fb_rule, "segmented_init_lm": seg,
            "stage_ms": {k: round(v, 3) for k, v in stages.items()},
            "accuracy_reference": "all-FP64 GPU fit, same LM, constant start, 300 iterations, tol 1e-30",
        },
    }


# ---- secondary: plain LM at scale, IVIM-10 ------------------------------------------

def plain_ivim10_block(args, dev, fp64_check=True):
    """IVIM-10, 8,388,608 voxels, plain LM, 100 iterations (the reference's
    run(100) at scale): fits/s, kernel time, accuracy against the FP64 fitter
    and fits/s at the 1e-4 budget."""
    import torch
    from pycompute_gb300 import Expr, SecondOrderLevenbergMarquardt, parity, synth

    w = synth.ivim()
    N = args.voxels
    true, data, init, lb, ub, prot = w.generate(N, seed=1000)
    solve = torch.float64 if args.solve == "f64" else torch.float32
    expr = Expr(w.expr, w.pars, w.consts)
    solm = SecondOrderLevenbergMarquardt(expr, None, w.M, torch.float32, solve_dtype=solve)
    data_d = torch.from_numpy(data).to(dev)
    init_d = torch.from_numpy(init).to(dev)
    pars_d = init_d.clone()
    solm.setup(pars_d, [float(x) for x in prot], data_d, [float(x) for x in lb], [float(x) for x in ub])

    def reset():
        pars_d.copy_(init_d)
        solm.lam_t.fill_(5.0)
        solm.step_type_t.fill_(1)
        solm.f_t.zero_()
        solm.iters_t.zero_()

    for _ in range(args.warmup):
        reset()
        solm.run(args.iters, block=args.block)
    torch.cuda.synchronize()
    ks = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ke = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0.record()
    for s in range(args.steps):
        reset()
        ks[s].record()
        solm.run(args.iters, block=args.block)
        ke[s].record()
    t1.record()
    torch.cuda.synchronize()
    step_ms = t0.elapsed_time(t1) / args.steps
    kern_ms = statistics.mean(ks[s].elapsed_time(ke[s]) for s in range(args.steps))
    fitted = pars_d.cpu().numpy()
    its = solm.iters_t.cpu().numpy()[0].astype(np.int64)
    st = solm.step_type_t.cpu().numpy()[0]
    hbm, _, peak_kind = _peaks()
    bpv = 4 * M_IVIM10 + 4 * P_IVIM + 1
    out = {"workload": "ivim10_plain_lm_8.4M", "voxels": N, "iters": args.iters, "solve": args.solve,
           "fits_per_s": N / (step_ms / 1e3), "ms_per_step": step_ms, "kernel_ms": kern_ms,
           "mean_iters": float(its.mean()), "converged_frac": float(np.mean(st == 0)),
           "voxel_iters_per_s": float(its.sum()) / (kern_ms / 1e3),
           "hbm_roofline": {"achieved_gbs": bpv * N / (kern_ms / 1e3) / 1e9, "peak_gbs": hbm,
                            "algorithmic_bytes_per_voxel": bpv, "peak_source": peak_kind}}
    if fp64_check:
        dd = data_d.double()
        solm64 = SecondOrderLevenbergMarquardt(expr, None, w.M, torch.float64)
        p64 = init_d.double()
        solm64.setup(p64, torch.from_numpy(prot).to(dev).double(), dd, torch.from_numpy(lb).to(dev).double(),
                     torch.from_numpy(ub).to(dev).double())
        solm64.run(args.iters)
        torch.cuda.synchronize()
        rep = parity.compare_params(fitted, p64.cpu().numpy())
        out["accuracy"] = {"vs": "all-FP64 GPU fitter, same LM, init and iterations",
                           "median_rel_err": rep["median_rel"], "frac_voxels_gt_1e-4": rep["frac_gt_1e-4"],
                           "per_param_median": rep["per_param_median"],
                           "converged_frac_fp64": float(np.mean(solm64.step_type_t.cpu().numpy() == 0))}
        del solm64, p64, dd
        ref64 = fp64_reference(w, data_d, iters=1000)

        def run_k(k):
            reset()
            solm.run(k, block=args.block)
            return pars_d

        k_tol, curve = budget_for_tolerance(run_k, ref64, range(2, 41))
        at = {"iters": k_tol, "curve": {k: v[0] for k, v in curve.items()}}
        if k_tol is not None:
            at["fits_per_s"] = N / (_time_ms(lambda: run_k(k_tol)) / 1e3)
        out["at_1e-4_vs_fp64"] = at
    return out


def mixed_batch_comparison(n_per_model=1 << 20, iters=100, seed=300):
    """VFA-T1 + T2* + IVIM + bi-exp T2, 1M voxels each, one persistent
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
    fitter = MultiModelFitter(models, block=tuned["block"], maxrreg=tuned["maxrreg"], lanes=tuned.get("lanes"))
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
    # accuracy of the one-launch results against the all-FP64 fitter (same LM,
    # same start, same iterations), per model
    run_multi()
    torch.cuda.synchronize()
    acc = {}
    for w, j, i0 in zip(ws, jobs, inits):
        s64 = SecondOrderLevenbergMarquardt(Expr(w.expr, w.pars, w.consts), None, w.M, torch.float64)
        p64 = i0.double()
        s64.setup(p64, list(w.protocol), j.data.double(), list(w.lb), list(w.ub))
        s64.run(iters)
        med, frac = _median_rel_gpu(j.pars, p64)
        acc[w.name] = {"median_rel_err": med, "frac_voxels_gt_1e-4": frac,
                       "per_param_median": _per_param_median(j.pars, p64)}
        # the model's own 1e-4 budget: error against the converged all-FP64
        # fit (300 iterations, tol 1e-30) of the fp32 fitter at growing
        # budgets, once with the batch's convergence tolerance (1e-8: the
        # projected-gradient test on unscaled parameters stops a voxel whose
        # cost is flat in one parameter, e.g. T1 in ms, before that parameter
        # settles) and once with tol 1e-30 like the reference fit (every
        # budget iteration runs: the error left is the fp32 fitter's own)
        s64.setup(p64.copy_(i0.double()), list(w.protocol), j.data.double(), list(w.lb), list(w.ub))
        s64.run(300, tol=1e-30)
        s32 = SecondOrderLevenbergMarquardt(Expr(w.expr, w.pars, w.consts), None, w.M, torch.float32)
        for key, tol in (("vs_fp64_converged", 1e-8), ("vs_fp64_converged_tol_1e-30", 1e-30)):
            curve, k_tol = {}, None
            for k in (25, 50, 100, 200, 400):
                p32 = i0.clone()
                s32.setup(p32, list(w.protocol), j.data, list(w.lb), list(w.ub))
                s32.run(k, tol=tol)
                curve[k] = _median_rel_gpu(p32, p64)[0]
                if k_tol is None and curve[k] <= TOL:
                    k_tol = k
            acc[w.name][key] = {"tol": tol, "median_rel_err_by_iters": curve, "iters_for_1e-4": k_tol,
                                "per_param_median_at_400": _per_param_median(p32, p64)}
        del s64, p64, s32
    return {"workload": "mixed_vfa8_t2s16_ivim10_biexp32", "voxels": total, "iters": iters,
            "autotuned": {k: tuned.get(k) for k in ("block", "maxrreg", "chunk", "order", "lanes", "ms")},
            "lanes_per_voxel_trials": tuned.get("lane_trials"),
            "tune_s": round(tune_s, 1),
            "one_launch_fits_per_s": total / (ms_multi / 1e3), "graph_fits_per_s": total / (ms_graph / 1e3),
            "per_model_launches_fits_per_s": total / (ms_single / 1e3), "mean_iters_per_model": its,
            "ms": {"one_launch": ms_multi, "graph": ms_graph, "per_model": ms_single},
            "accuracy_vs_fp64_same_iters": acc}


def precision_stress(n=1 << 21, iters=100, seed=400):
    """Ill-conditioned IVIM-10 (SNR 10-20, f in [0.005, 0.05]): the FP32-bulk /
    FP64-solve fitter and the fp32-solve fitter against the all-FP64 fitter
    (same LM, same start, same iterations; and against its converged fit)."""
    import torch
    from pycompute_gb300 import Expr, SecondOrderLevenbergMarquardt, pipeline, synth

    w = synth.ivim(snr=(10.0, 20.0), f_range=(0.005, 0.05), name="ivim10_stress")
    _, data = pipeline.synth_gpu(w, n, seed=seed, device="cuda")
    init = pipeline.init_constant(data, w.init_values)
    prot, lb, ub = list(w.protocol), list(w.lb), list(w.ub)

    def fit(dtype, solve, k, tol=1e-8):
        solm = SecondOrderLevenbergMarquardt(Expr(w.expr, w.pars, w.consts), None, w.M, dtype, solve_dtype=solve)
        p = init.to(dtype).clone()
        solm.setup(p, prot, data.to(dtype), lb, ub)
        solm.run(k, tol=tol)
        torch.cuda.synchronize()
        return p

    p64_same = fit(torch.float64, torch.float64, iters)
    p64_conv = fit(torch.float64, torch.float64, 300, tol=1e-30)

    def report(p, ref):
        r = ((p.double() - ref).abs() / ref.abs().clamp_min(1e-30))
        r = torch.nan_to_num(r, nan=float("inf"))
        q = torch.quantile(r.float(), torch.tensor([0.5, 0.9, 0.99], device=r.device), dim=1).T
        worst = r.amax(dim=0)
        return {"per_param_q50_q90_q99": [[float(x) for x in row] for row in q],
                "median_rel_err": float(worst.median()), "frac_voxels_gt_1e-4": float((worst > 1e-4).double().mean())}

    out = {"workload": "ivim10_stress_2M (SNR 10-20, f in [0.005, 0.05])", "voxels": n, "iters": iters,
           "params": list(w.pars)}
    for name, solve in (("f32_state_f64_solve", torch.float64), ("f32_state_f32_solve", torch.float32)):
        p = fit(torch.float32, solve, iters)
        out[name] = {"vs_fp64_same_iters": report(p, p64_same), "vs_fp64_converged": report(p, p64_conv)}
    return out


def _config(args, ws):
    """The workload, identical in both arms (iteration budgets are results and
    travel outside it)."""
    return {"workload": "ivim16_warm_start_vs_plain_lm_16.7M", "voxels_per_gpu": args.warm_voxels,
            "ndata": M_IVIM16, "nparam": P_IVIM, "tolerance": TOL,
            "network": "16-128-128-128-4 GELU, bf16 weights, fp32 accumulate",
            "train_voxels": args.warm_train, "solve": "f64", "init_plain": "constant [max S, 0.1, 1e-2, 1e-3]",
            "l2": "inputs larger than L2 (1.07 GB signals per GPU)", "parallelism": f"voxel shards x{ws}"}


def _torch_ivim_inputs(bvals, n, seed, dev):
    """Seeded Rician IVIM signals (M, n) and the reference notebook's constant
    start, made with PyTorch alone (the reference arm loads none of this
    package's native code): true parameters uniform over the benchmark
    ranges, sigma = S0 / 50."""
    import torch
    g = torch.Generator(device=dev)
    g.manual_seed(seed)
    u = lambda lo, hi: lo + (hi - lo) * torch.rand(n, generator=g, device=dev, dtype=torch.float64)  # noqa: E731
    s0, f, dstar, d = u(500.0, 1500.0), u(0.05, 0.35), u(5e-3, 5e-2), u(0.5e-3, 2.5e-3)
    b = torch.tensor(bvals, device=dev, dtype=torch.float64)[:, None]
    clean = s0 * (f * torch.exp(-b * dstar) + (1 - f) * torch.exp(-b * d))
    sigma = s0 / 50.0
    n1 = torch.randn(clean.shape, generator=g, device=dev, dtype=torch.float64)
    n2 = torch.randn(clean.shape, generator=g, device=dev, dtype=torch.float64)
    data = torch.sqrt((clean + sigma * n1) ** 2 + (sigma * n2) ** 2).float().contiguous()
    del clean, n1, n2
    init = torch.stack([data.amax(dim=0), torch.full((n,), 0.1, device=dev), torch.full((n,), 1e-2, device=dev),
                        torch.full((n,), 1e-3, device=dev)]).contiguous()
    return data, init


def reference_gpu_kernel(steps: int = 3):
    """The reference's own LM kernel on this GPU, launched as its run() does
    (oracle/_ref cubin built from the reference tree; 32-thread blocks, one
    launch per iteration): IVIM-10 8,388,608 voxels x 100 iterations, and
    IVIM-16 16,777,216 voxels at the plain LM's 1e-4 budget (8 iterations).
    Inputs are made with PyTorch alone: this process maps none of the
    package's native libraries."""
    import torch
    from oracle import ref_gpu
    from pycompute_gb300 import synth

    out = {"kernel": "reference generated LM kernel (printf dropped, parameter loads bounded), sm_103a",
           "launch": "ceil(N/32) blocks x 32 threads, one launch per iteration, protocol tiled per voxel"}
    dev = torch.device("cuda", torch.cuda.current_device())
    for name, bvals, n, iters in (("ivim10_8.4M_100it", synth.IVIM_B10, 256 * 256 * 128, 100),
                                  ("ivim16_16.7M_8it_at_1e-4", synth.ivim_b16(), 1 << 24, 8)):
        M = len(bvals)
        if not ref_gpu.available(M):
            out[name] = {"unavailable": f"oracle/_ref cubin for {M} samples not built"}
            continue
        data, init = _torch_ivim_inputs(bvals, n, 1000, dev)
        consts = torch.tensor(bvals, device=dev, dtype=torch.float32)[:, None].expand(M, n).contiguous()
        lb = torch.tensor(synth.IVIM_LB, device=dev)[:, None].expand(4, n).contiguous()
        ub = torch.tensor(synth.IVIM_UB, device=dev)[:, None].expand(4, n).contiguous()
        ref = ref_gpu.RefGpuIVIM(M)
        pars = init.clone()

        def step():
            pars.copy_(init)
            ref.setup(pars, consts, data, lb, ub)
            ref.run(iters)

        ms = _time_ms(step, warmup=1, reps=steps)
        out[name] = {"voxels": n, "iters": iters, "fits_per_s": n / (ms / 1e3), "ms_per_fit": ms}
        del ref, pars, consts, lb, ub, data, init
        torch.cuda.empty_cache()
    return out


def _mapped_native_libraries():
    """Shared objects of this repository mapped into this process (Linux)."""
    try:
        with open("/proc/self/maps") as f:
            paths = {line.split()[-1] for line in f if line.rstrip().endswith(".so") or ".so." in line}
    except OSError:
        return None
    return sorted(os.path.relpath(p, ROOT) for p in paths if p.startswith(ROOT + os.sep))


def run_reference_arm(args):
    ws, rank, local = _dist()
    if rank != 0:
        return 0
    # the budget is settled once on a small sample; every step then times one
    # host fit of the full workload (all voxels of a GPU's shard)
    plan = cpu_reference_at_tol(target_s=args.cpu_seconds, n_fixed=args.warm_voxels)
    vals, last = [], plan
    for s in range(args.warmup + args.steps):
        last = cpu_reference_at_tol(target_s=args.cpu_seconds, plan=plan)
        if s >= args.warmup:
            vals.append(last["value"])
    value = statistics.median(vals)
    gpu = None
    try:
        import torch
        if torch.cuda.is_available():
            torch.cuda.set_device(local)
            gpu = reference_gpu_kernel()
    except Exception as e:  # informational only: the reference arm's value is the CPU measurement
        gpu = {"unavailable": f"{type(e).__name__}: {e}"}
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "fits/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": args.warm_voxels / value * 1e3,
        "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded IVIM-16, Rician SNR 50)",
        "config": _config(args, ws),
        "method": "plain LM from the constant start (the reference has no warm start)",
        "iters_plain": last["iters"],
        "cpu_baseline": {"value": value, "unit": "fits/s", "cores": last["cores"], "kind": last["kind"],
                         "sample": last["sample"]},
        "e2e": {"value": value, "unit": "fits/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "gpu_reference_kernel": gpu,
        "native_libraries_mapped": _mapped_native_libraries(),
    }
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--warm-voxels", type=int, default=1 << 24)
    ap.add_argument("--warm-epochs", type=int, default=128)
    ap.add_argument("--warm-lr", type=float, default=8e-3, help="peak Adam learning rate (cosine decay)")
    ap.add_argument("--warm-lam0", type=float, default=3e-3)
    ap.add_argument("--warm-train", type=int, default=1 << 21)
    ap.add_argument("--e2e-chunks", type=int, default=8, help="voxel chunks of the streamed end-to-end fit")
    ap.add_argument("--voxels", type=int, default=256 * 256 * 128, help="IVIM-10 plain-LM block")
    ap.add_argument("--iters", type=int, default=100, help="IVIM-10 plain-LM block")
    ap.add_argument("--solve", default="f64", choices=["f64", "f32"], help="IVIM-10 plain-LM block")
    ap.add_argument("--block", type=int, default=0)
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-ivim10", action="store_true", help="skip the IVIM-10 plain-LM block")
    ap.add_argument("--no-mixed", action="store_true")
    ap.add_argument("--no-stress", action="store_true", help="skip the precision-stress block")
    ap.add_argument("--no-fp64-check", action="store_true", help="IVIM-10 block without its FP64 comparison")
    ap.add_argument("--only-ivim10", action="store_true", help="print only the IVIM-10 plain-LM block")
    ap.add_argument("--only-mixed", action="store_true", help="print only the mixed-model block")
    ap.add_argument("--only-warm", action="store_true", help="print only the warm-start headline fields")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference_arm(args)

    import torch
    import torch.distributed as dist

    ws, rank, local = _dist()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if args.only_mixed:
        print(json.dumps(mixed_batch_comparison()), flush=True)
        return 0
    if args.only_ivim10:
        print(json.dumps(plain_ivim10_block(args, dev, fp64_check=not args.no_fp64_check)), flush=True)
        return 0
    if ws > 1:
        dist.init_process_group("nccl", device_id=dev)

    h = warm_headline(args, ws, rank, local, dev)
    if args.only_warm:
        if rank == 0:
            print(json.dumps({k: v for k, v in h.items() if k != "clocks"}), flush=True)
        if ws > 1:
            dist.destroy_process_group()
        return 0
    N = h["N"]
    single = rank == 0 and ws == 1
    ivim10 = plain_ivim10_block(args, dev, fp64_check=not args.no_fp64_check) if single and not args.no_ivim10 \
        else None
    mixed = mixed_batch_comparison() if single and not args.no_mixed else None
    stress = precision_stress() if single and not args.no_stress else None
    cpu = None
    if single and not args.no_cpu:
        cpu = cpu_reference_at_tol(target_s=args.cpu_seconds)
        cpu["gpu_parity_ivim10"] = cpu_parity_ivim10()
        cpu["parity_c2"] = parity_c2()

    if rank == 0:
        hbm, bf16_peak, peak_kind = _peaks()
        bpv = 4 * M_IVIM16 + 8 * P_IVIM + 1
        lm_gbs = bpv * N / (h["lm_ms"] / 1e3) / 1e9
        net_tf = NET_FLOP_PER_VOXEL * N / (h["net_ms"] / 1e3) / 1e12
        traffic = None
        tf = os.path.join(ROOT, "profiles", "lmw_ivim16_warm_traffic.json")
        if os.path.exists(tf):
            with open(tf) as f:
                traffic = json.load(f)["dram_bytes_per_voxel"] * N
        value = ws * N / (h["step_ms"] / 1e3)
        plain_value = ws * N / (h["plain_ms"] / 1e3)
        line = {
            "metric": METRIC, "value": value, "unit": "fits/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": h["step_ms"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 state, f64 GMW81 solve + gain ratio, bf16 network",
            "data": "synthetic (seeded IVIM-16, Rician SNR 50; network trained on other seeded signals)",
            "config": _config(args, ws),
            "iters_warm": h["k_warm"], "iters_plain": h["k_plain"],
            "plain_lm": {"value": plain_value, "unit": "fits/s", "ms_per_step": h["plain_ms"],
                         "iters": h["k_plain"], "speedup_warm_vs_plain": value / plain_value},
            "e2e": {"value": ws * N / (h["e2e_ms"] / 1e3), "unit": "fits/s", "h2d_bytes_per_step": h["h2d"],
                    "d2h_bytes_per_step": h["d2h"], "ms_per_step": h["e2e_ms"],
                    "api": "WarmStartFitter.fit_stream: the timed steps as a sequence of pinned host volumes, "
                           "each copied in and back, copies overlapped with the neighbouring steps' fits",
                    "matches_device_run": h["e2e_same"], "clocks": h["e2e_clocks"], "host_link": h["host_link"],
                    "single_volume": {"value": ws * N / (h["e2e_single_ms"] / 1e3), "ms_per_step": h["e2e_single_ms"],
                                      "api": f"WarmStartFitter.fit_host, {h['e2e_chunks']} chunks"}},
            "roofline": {"bound": "hbm", "achieved": lm_gbs, "peak": hbm, "unit": "GB/s", "frac": lm_gbs / hbm,
                         "traffic": traffic, "peak_source": peak_kind, "kernel": "pcgb_lmw (warm LM with the fallback check as its epilogue)",
                         "algorithmic_bytes_per_voxel": bpv, "kernel_ms": h["lm_ms"],
                         "note": "per-voxel iterative solver: bound by the FP64 pipe (GMW81 solve + gain ratio), "
                                 "not by HBM; ncu summaries in profiles/"},
            "roofline_network": {"bound": "tensor", "achieved": net_tf, "peak": bf16_peak, "unit": "TFLOP/s",
                                 "frac": net_tf / bf16_peak, "kernel": "mlp_infer_tc_kernel (tcgen05)",
                                 "flop_per_voxel": NET_FLOP_PER_VOXEL, "kernel_ms": h["net_ms"],
                                 "peak_source": peak_kind,
                                 "mufu": _unit_roofline(MUFU_PER_VOXEL_NET * N, h["net_ms"], MUFU_PER_SM_CLK,
                                                        h["clocks"], "MUFU instructions per voxel, ncu opcode counts")},
            "roofline_fp64": dict(_unit_roofline(FP64_OPS_PER_VOXEL_ITER * N * h["k_warm"], h["lm_ms"],
                                                 FP64_PER_SM_CLK, h["clocks"],
                                                 "FP64-pipe instructions (DFMA + DMUL + DADD) per voxel-iteration, "
                                                 "ncu opcode counts"),
                                  kernel="pcgb_lmw (warm LM with the fallback check as its epilogue)",
                                  bound="fp64 pipe"),
            "warm_start": h["detail"],
            "plain_lm_ivim10_8.4M": ivim10,
            "mixed_batch": mixed,
            "precision_stress": stress,
            "cpu_baseline": cpu,
            # our kernels per warm-start step: tcgen05 network, warm LM with the
            # fallback check as its epilogue, refit with the select as its
            # epilogue (counted from an ncu launch list of the timed steps)
            "gpu_launches": 3 * args.steps,
            "clocks": h["clocks"],
        }
        print(json.dumps(line), flush=True)
    if ws > 1:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
