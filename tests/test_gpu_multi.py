"""Mixed-model persistent batch: VFA-T1 (2 params, 8 angles), T2* (3, 16),
IVIM (4, 10) and bi-exponential T2 (5, 32) fitted in one launch agree with
the single-model fitter voxel by voxel; a captured CUDA graph replays the same
fit; the autotuner returns a cached configuration."""
import pytest
import torch

from pycompute_gb300 import Expr, SecondOrderLevenbergMarquardt, parity, synth
from pycompute_gb300.multi import MultiJob, MultiModelFitter, autotune

pytestmark = pytest.mark.gpu
DEV = "cuda:0"
WORKLOADS = [synth.vfa_t1, synth.t2star, synth.ivim, synth.biexp_t2]


def _make(n=3000, seed=0):
    ws = [f() for f in WORKLOADS]
    gens = [w.generate(n + 17 * k, seed=seed + k) for k, w in enumerate(ws)]
    return ws, gens


def _jobs(ws, gens):
    jobs = []
    for w, (true, data, init, lb, ub, prot) in zip(ws, gens):
        jobs.append(MultiJob(torch.from_numpy(init.copy()).to(DEV), torch.from_numpy(data).to(DEV), prot, lb, ub))
    return jobs


def test_mixed_batch_matches_single_model_fits():
    ws, gens = _make()
    fitter = MultiModelFitter([(Expr(w.expr, w.pars, w.consts), w.M) for w in ws])
    jobs = _jobs(ws, gens)
    fitter.fit(jobs, 60)
    torch.cuda.synchronize()
    for w, (true, data, init, lb, ub, prot), j in zip(ws, gens, jobs):
        solm = SecondOrderLevenbergMarquardt(Expr(w.expr, w.pars, w.consts), None, w.M, torch.float32)
        p = torch.from_numpy(init.copy()).to(DEV)
        solm.setup(p, torch.from_numpy(prot).to(DEV), torch.from_numpy(data).to(DEV), torch.from_numpy(lb).to(DEV),
                   torch.from_numpy(ub).to(DEV))
        solm.run(60)
        torch.cuda.synchronize()
        rep = parity.compare_params(j.pars.cpu().numpy(), p.cpu().numpy())
        assert rep["median_rel"] <= 1e-6 and rep["frac_gt_1e-4"] <= 0.02, (w.name, rep)
        assert parity.flags_agree(j.step_type.cpu().numpy(), solm.step_type_t.cpu().numpy()) >= 0.99
        assert torch.all(j.iters > 0)


def test_graph_replay_and_chunk_sizes_agree():
    ws, gens = _make(2000, seed=5)
    fitter = MultiModelFitter([(Expr(w.expr, w.pars, w.consts), w.M) for w in ws])
    jobs = _jobs(ws, gens)
    inits = [j.pars.clone() for j in jobs]
    fitter.fit(jobs, 40, chunk=32)
    torch.cuda.synchronize()
    eager = [j.pars.clone() for j in jobs]
    for j, i0 in zip(jobs, inits):
        j.reset(i0)
    g = fitter.capture(jobs, 40, chunk=256)
    for j, i0 in zip(jobs, inits):
        j.reset(i0)
    g.replay()
    torch.cuda.synchronize()
    for a, j in zip(eager, jobs):
        assert torch.equal(a, j.pars)  # each voxel's fit does not depend on the schedule


def test_autotune_picks_and_caches():
    ws, gens = _make(1024, seed=9)
    models = [(Expr(w.expr, w.pars, w.consts), w.M) for w in ws]
    best = autotune(models, lambda: _jobs(ws, gens), iters=10, blocks=(64, 128), maxrregs=(0, 128), chunks=(32, 128),
                    use_cache=False)
    assert best["ms"] > 0 and best["block"] in (64, 128) and len(best["trials"]) >= 4
    again = autotune(models, lambda: _jobs(ws, gens), iters=10, blocks=(64, 128), maxrregs=(0, 128),
                     chunks=(32, 128))
    assert again["block"] == best["block"] and again["chunk"] == best["chunk"]


def test_two_lanes_per_voxel_match_one_lane():
    """Two lanes per voxel (each accumulates half of the samples; the shares
    are summed across the pair) against one lane per voxel, in one launch of
    the four models: after one iteration every parameter agrees to fp32
    summation order (1e-5 on all but a handful of entries); after 60
    iterations both summation orders are equally close to the all-FP64 fit
    (same LM, same start, same iterations): the two-lane median error at most
    1.5 times the one-lane one (the ill-conditioned bi-exponential T2 fits
    of the two orders differ from each other by more than either does from
    the FP64 fit)."""
    ws, gens = _make(4000, seed=11)
    models = [(Expr(w.expr, w.pars, w.consts), w.M) for w in ws]
    res = {}
    for lanes in ([1, 1, 1, 1], [2, 2, 2, 2]):
        fitter = MultiModelFitter(models, lanes=lanes)
        for iters in (1, 60):
            jobs = _jobs(ws, gens)
            fitter.fit(jobs, iters)
            torch.cuda.synchronize()
            res[(lanes[0], iters)] = [(j.pars.cpu().numpy(), j.step_type.cpu().numpy(), j.iters.cpu().numpy())
                                      for j in jobs]
    for w, a, b in zip(ws, res[(1, 1)], res[(2, 1)]):
        rel = parity.rel_err(b[0], a[0])
        assert float((rel <= 1e-5).mean()) > 0.999, (w.name, float((rel <= 1e-5).mean()))
        assert float((b[1] == a[1]).mean()) > 0.999, w.name
    for w, (true, data, init, lb, ub, prot), a, b in zip(ws, gens, res[(1, 60)], res[(2, 60)]):
        s64 = SecondOrderLevenbergMarquardt(Expr(w.expr, w.pars, w.consts), None, w.M, torch.float64)
        p64 = torch.from_numpy(init.astype("float64")).to(DEV)
        s64.setup(p64, list(w.protocol), torch.from_numpy(data).to(DEV).double(), list(w.lb), list(w.ub))
        s64.run(60)
        torch.cuda.synchronize()
        ref = p64.cpu().numpy()
        e1 = parity.compare_params(a[0], ref)["median_rel"]
        e2 = parity.compare_params(b[0], ref)["median_rel"]
        assert e2 <= 1.5 * e1 + 1e-7, (w.name, e1, e2)
        assert (b[2] > 0).all()
