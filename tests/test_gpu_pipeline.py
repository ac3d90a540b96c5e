"""Fit-pipeline kernels: constant initialisation, forward-model evaluation,
the warm-start fallback, and what the trained network gains over the plain
fit at the same iteration budget (median error against the all-FP64 fit)."""
import numpy as np
import pytest
import torch

from pycompute_gb300 import Expr, SecondOrderLevenbergMarquardt, parity, pipeline, synth
from pycompute_gb300.warmstart import WarmStartMLP

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


def test_init_constant_and_model_eval():
    w = synth.ivim()
    true, data = pipeline.synth_gpu(w, 5000, seed=1, device=DEV)
    p0 = pipeline.init_constant(data, w.init_values).cpu().numpy()
    d = data.cpu().numpy()
    np.testing.assert_array_equal(p0[0], d.max(axis=0))
    np.testing.assert_array_equal(p0[1:], np.broadcast_to(np.array([0.1, 1e-2, 1e-3], np.float32)[:, None], (3, 5000)))
    # forward model against an independent numpy evaluation
    solm = SecondOrderLevenbergMarquardt(Expr(w.expr, w.pars, w.consts), None, w.M, torch.float32)
    solm.setup(true.clone(), torch.tensor(w.protocol, device=DEV), data, torch.tensor(w.lb, device=DEV),
               torch.tensor(w.ub, device=DEV))
    m = solm.model_eval(true).cpu().numpy()
    want = w.model_numpy(true.cpu().numpy().astype(np.float64), np.array(w.protocol))
    np.testing.assert_allclose(m, want, rtol=2e-6)
    # the Rician signals scatter around the model at the set SNR
    resid = (d - want) / (true.cpu().numpy()[0] / 50.0)
    assert 0.8 < resid.std() < 1.3


def _fp64_fit(w, data, iters=1000):
    solm = SecondOrderLevenbergMarquardt(Expr(w.expr, w.pars, w.consts), None, w.M, torch.float64)
    p = pipeline.init_constant(data, w.init_values).double()
    solm.setup(p, torch.tensor(w.protocol, device=DEV).double(), data.double(), torch.tensor(w.lb, device=DEV).double(),
               torch.tensor(w.ub, device=DEV).double())
    solm.run(iters, tol=1e-30)
    torch.cuda.synchronize()
    return p.cpu().numpy()


def _plain_fit(w, data, iters):
    solm = SecondOrderLevenbergMarquardt(Expr(w.expr, w.pars, w.consts), None, w.M, torch.float32)
    p = pipeline.init_constant(data, w.init_values)
    solm.setup(p, torch.tensor(w.protocol, device=DEV), data, torch.tensor(w.lb, device=DEV),
               torch.tensor(w.ub, device=DEV))
    solm.run(iters)
    return p, solm.cost()


class _BadNet:
    """Stand-in network that returns a deliberately poor start for every 3rd voxel."""

    def __init__(self, w):
        self.w = w

    def infer(self, data, out=None):
        p = pipeline.init_constant(data, self.w.init_values)
        p[:, ::3] = torch.tensor(self.w.ub, device=data.device)[:, None]  # on the upper bound
        p[1, 1::3] = 0.9                                                    # far from the fit
        if out is not None:
            out.copy_(p)
            return out
        return p


def test_fallback_refits_flagged_voxels():
    w = synth.ivim(synth.ivim_b16(), name="ivim16")
    true, data = pipeline.synth_gpu(w, 30000, seed=2, device=DEV)
    res = pipeline.WarmStartFitter(w, _BadNet(w)).fit(data, iters_warm=3, iters_fallback=30)
    torch.cuda.synchronize()
    assert res["n_fallback"] >= 10000  # at least every 3rd voxel starts on a bound
    p_plain, c_plain = _plain_fit(w, data, 30)
    cost = res["cost"].cpu().numpy()
    # every voxel ends at a cost no worse than the warm fit and, where it was
    # refitted, no worse than the plain fit's
    pars = res["pars"].cpu().numpy()
    assert np.all(np.isfinite(pars))
    refit = np.zeros(30000, bool)
    refit[::3] = True
    assert np.all(cost[refit] <= c_plain.cpu().numpy()[refit] * (1 + 1e-6) + 1e-3)


@pytest.mark.parametrize("per_voxel_bounds,schedule,mode", [(False, "grid", True), (True, "grid", True),
                                                            (False, "refill", True), (False, "grid", "epilogue"),
                                                            (True, "grid", "epilogue"), (False, "grid", "select"),
                                                            (True, "grid", "select")])
def test_fused_fallback_matches_separate_kernels(per_voxel_bounds, schedule, mode):
    """Check + refit + select as three fused kernels, or as the epilogues of
    the warm LM and the refit launches (no host read of the flagged count
    either way), give the same fits, costs and counts as the separate
    pipeline kernels."""
    w = synth.ivim(synth.ivim_b16(), name="ivim16")
    _, data = pipeline.synth_gpu(w, 50001, seed=7, device=DEV)
    out = []
    for fused in (False, mode):
        wf = pipeline.WarmStartFitter(w, _BadNet(w))
        wf.refit_schedule = schedule
        if per_voxel_bounds:
            N = data.shape[1]
            lbt = torch.tensor(w.lb, device=DEV)[:, None].expand(w.P, N).contiguous()
            ubt = torch.tensor(w.ub, device=DEV)[:, None].expand(w.P, N).contiguous()
            wf._consts = lambda dev, lbt=lbt, ubt=ubt: (list(w.protocol), lbt, ubt)
        res = wf.fit(data, iters_warm=3, iters_fallback=20, fused=fused)
        torch.cuda.synchronize()
        out.append((res.pars.cpu().numpy().copy(), res.cost.cpu().numpy().copy(), res.n_fallback, res.n_refit_kept))
    (p0, c0, n0, k0), (p1, c1, n1, k1) = out
    assert n0 == n1 and n0 >= 16667
    assert k0 == k1
    np.testing.assert_array_equal(p0, p1)
    np.testing.assert_array_equal(c0, c1)


@pytest.mark.parametrize("per_voxel_bounds,iters", [(False, 3), (True, 3), (False, 0)])
def test_lean_warm_lm_with_check_epilogue_matches_select_pipeline(per_voxel_bounds, iters):
    """The warm LM from a fresh start with the check as its epilogue
    (fused="lean") against the pipeline with the check as its own kernel
    (fused="select"): the same warm iterations and rule, but the warm fit's cost
    comes from the iterations instead of a second evaluation, so the two costs
    a decision compares differ by rounding. The flagged sets may differ only on
    voxels whose warm cost and constant-start cost tie to 1e-5; voxels flagged
    by neither end bit-equal; voxels flagged by both end equal unless the
    select compared a tie (final costs within 1e-5). With no warm iteration
    the epilogue evaluates the warm cost itself, as the check kernel does."""
    w = synth.ivim(synth.ivim_b16(), name="ivim16")
    _, data = pipeline.synth_gpu(w, 50001, seed=17, device=DEV)
    N = data.shape[1]
    lbt = torch.tensor(w.lb, device=DEV)[:, None].expand(w.P, N).contiguous()
    ubt = torch.tensor(w.ub, device=DEV)[:, None].expand(w.P, N).contiguous()
    out = []
    for fused in ("select", "lean"):
        wf = pipeline.WarmStartFitter(w, _BadNet(w))
        if per_voxel_bounds:
            wf._consts = lambda dev: (list(w.protocol), lbt, ubt)
        res = wf.fit(data, iters_warm=iters, iters_fallback=20, fused=fused)
        torch.cuda.synchronize()
        flagged = np.zeros(N, dtype=bool)
        flagged[res.fallback_idx[:res.n_fallback].cpu().numpy()] = True
        out.append((res.pars.cpu().numpy().copy(), res.cost.cpu().numpy().copy(), flagged))
    (p0, c0, f0), (p1, c1, f1) = out
    assert f0.sum() >= 16667
    # the warm fit and its two costs, evaluated as the separate check does
    wf = pipeline.WarmStartFitter(w, _BadNet(w))
    warm = wf.net.infer(data)
    solm = wf._fitter()
    solm.setup(warm, list(w.protocol), data, list(w.lb), list(w.ub))
    solm.run_fresh(iters, 1e-3)
    cw = solm.cost().cpu().numpy().astype(np.float64)
    cs = solm.cost(pipeline.init_constant(data, w.init_values)).cpu().numpy().astype(np.float64)
    torch.cuda.synchronize()
    differ = f0 != f1
    assert differ.mean() <= 1e-3, differ.mean()
    assert np.all(np.abs(cw[differ] - cs[differ]) <= 1e-5 * cs[differ]), np.where(differ)[0][:10]
    neither = ~f0 & ~f1
    np.testing.assert_array_equal(p0[:, neither], p1[:, neither])
    np.testing.assert_allclose(c1[neither], c0[neither], rtol=1e-5)
    both = f0 & f1
    same = np.all(p0 == p1, axis=0)
    assert (both & ~same).sum() <= 1e-3 * both.sum() + 1
    np.testing.assert_allclose(c1[both], c0[both], rtol=1e-5)


@pytest.mark.parametrize("kernel", ["check", "lean"])
def test_fallback_flags_match_the_rule_on_the_oracle(kernel):
    """The fused check's flagged set against the fallback rule evaluated on the
    CPU by the oracle, on the same warm fits: a voxel is flagged when its cost
    is not finite or not below the cost at the plain fitter's constant start,
    or a parameter is not strictly inside its bounds. GPU and oracle costs
    differ by fp32 rounding, so the two sets may differ only on voxels whose
    two costs are within 1e-5 relative of each other. ``check``: the check as
    its own kernel after the warm LM; ``lean``: the check as the epilogue of
    the warm LM from a fresh start (the warm cost taken from the iterations)."""
    from oracle import OracleModel
    w = synth.ivim(synth.ivim_b16(), name="ivim16")
    _, data = pipeline.synth_gpu(w, 50001, seed=9, device=DEV)
    N = data.shape[1]
    wf = pipeline.WarmStartFitter(w, _BadNet(w))
    pars = wf.net.infer(data)
    solm = wf._fitter()
    prot, lb, ub = wf._consts(DEV)
    b = wf._buffers(w.P, N, DEV)
    if kernel == "check":
        solm.setup(pars, prot, data, lb, ub)
        solm.lam_t.fill_(3e-3)
        solm.run(2)
        warm = pars.cpu().numpy().copy()
        wf._warm_check(solm, data, pars, b)
    else:
        warm_t = pars.clone()
        solm.setup(warm_t, prot, data, lb, ub, init_state=False)
        solm.run_fresh(2, 3e-3)
        warm = warm_t.cpu().numpy().copy()
        solm.setup(pars, prot, data, lb, ub, init_state=False)
        wf._warm_lm_check(solm, data, pars, b, 2, 3e-3)
    torch.cuda.synchronize()
    n_fb = int(b["counts"][0].item())
    flagged_gpu = np.zeros(N, dtype=bool)
    flagged_gpu[b["idx"][:n_fb].cpu().numpy()] = True

    d = data.cpu().numpy()
    om = OracleModel(w.expr, w.pars, w.consts)
    consts = np.asarray(w.protocol, dtype=np.float32)
    c = om.cost(warm, consts, d)
    p0 = pipeline.init_constant(data, w.init_values).cpu().numpy()
    c0 = om.cost(p0, consts, d)
    lo = np.asarray(w.lb, dtype=np.float32)[:, None]
    hi = np.asarray(w.ub, dtype=np.float32)[:, None]
    on_bound = np.any(~((warm > lo) & (warm < hi)), axis=0)
    with np.errstate(invalid="ignore"):
        flagged_cpu = ~np.isfinite(c) | ~(c < c0) | on_bound
        near_tie = np.abs(c.astype(np.float64) - c0) <= 1e-5 * np.maximum(np.abs(c0), 1e-30)
    differ = flagged_gpu != flagged_cpu
    assert n_fb > 0 and flagged_cpu.any()
    assert np.all(near_tie[differ]), np.where(differ & ~near_tie)[0][:10]


@pytest.mark.parametrize("N,chunks", [(100003, 3), (65536, 8), (1000, 4)])
def test_fit_host_streams_chunks_with_fit_results(N, chunks):
    """fit_host (chunked copies overlapping the fits) gives every voxel the
    result of one device-resident fit() of all voxels."""
    w = synth.ivim(synth.ivim_b16(), name="ivim16")
    true, data = pipeline.synth_gpu(w, N, seed=12, device=DEV)
    net = WarmStartMLP(16, 4, [0, 1, 2, 2], w.lb, w.ub, DEV, seed=5)  # untrained: a per-voxel start all the same
    net.fit_normalisation(data, true)
    wf = pipeline.WarmStartFitter(w, net)
    ref = wf.fit(data, iters_warm=3, iters_fallback=20)
    torch.cuda.synchronize()
    p_ref, n_ref = ref.pars.cpu().numpy().copy(), ref.n_fallback
    data_h = data.cpu().pin_memory()
    out_h = torch.full((w.P, N), float("nan")).pin_memory()
    counts = wf.fit_host(data_h, out_h, iters_warm=3, iters_fallback=20, chunks=chunks)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(out_h.numpy(), p_ref)
    assert int(counts[0]) == n_ref


def test_fit_stream_volumes_with_fit_results():
    """fit_stream (volumes double-buffered, copies overlapping fits) gives each
    volume the result of fit() on it."""
    w = synth.ivim(synth.ivim_b16(), name="ivim16")
    net = WarmStartMLP(16, 4, [0, 1, 2, 2], w.lb, w.ub, DEV, seed=5)
    true, d0 = pipeline.synth_gpu(w, 70001, seed=13, device=DEV)
    net.fit_normalisation(d0, true)
    wf = pipeline.WarmStartFitter(w, net)
    vols, refs = [], []
    for k, n in enumerate((70001, 1000, 70001, 4099)):
        _, d = pipeline.synth_gpu(w, n, seed=20 + k, device=DEV)
        refs.append(wf.fit(d, iters_warm=2, iters_fallback=8).pars.cpu().numpy().copy())
        vols.append((d.cpu().pin_memory(), torch.full((w.P, n), float("nan")).pin_memory()))
    counts = wf.fit_stream(vols, iters_warm=2, iters_fallback=8)
    torch.cuda.synchronize()
    for (_, out), ref in zip(vols, refs):
        np.testing.assert_array_equal(out.numpy(), ref)
    assert int(counts[0]) >= 0


def test_warm_fit_of_zero_voxels():
    w = synth.ivim(synth.ivim_b16(), name="ivim16")
    net = WarmStartMLP(16, 4, [0, 1, 2, 2], w.lb, w.ub, DEV, seed=5)
    wf = pipeline.WarmStartFitter(w, net)
    data = torch.empty((16, 0), device=DEV)
    res = wf.fit(data, iters_warm=2, iters_fallback=8)
    counts = wf.fit_host(torch.empty((16, 0)).pin_memory(), torch.empty((4, 0)).pin_memory(), 2, 8)
    torch.cuda.synchronize()
    assert res.pars.shape == (4, 0) and res.n_fallback == 0 and int(counts.sum()) == 0


def test_trained_network_beats_plain_lm_at_equal_iterations():
    w = synth.ivim(synth.ivim_b16(), name="ivim16")
    # training set: signals and the plain LM's fits of them as labels
    _, tr_data = pipeline.synth_gpu(w, 1 << 18, seed=10, device=DEV)
    labels, _ = _plain_fit(w, tr_data, 100)
    net = WarmStartMLP(16, 4, [0, 1, 2, 2], w.lb, w.ub, DEV, seed=0)
    net.train(tr_data, labels, epochs=12, batch=4096, lr=2e-3)
    # evaluation set, unseen seed
    _, data = pipeline.synth_gpu(w, 1 << 16, seed=11, device=DEV)
    ref = _fp64_fit(w, data)
    K = 3
    p_plain, _ = _plain_fit(w, data, K)
    res = pipeline.WarmStartFitter(w, net).fit(data, iters_warm=K, iters_fallback=30)
    torch.cuda.synchronize()
    e_plain = parity.compare_params(p_plain.cpu().numpy(), ref)["median_rel"]
    e_warm = parity.compare_params(res["pars"].cpu().numpy(), ref)["median_rel"]
    print(f"median rel err after {K} iterations: plain {e_plain:.3e}, warm start {e_warm:.3e}")
    # the network start is worth several LM iterations
    assert e_warm < 0.1 * e_plain, (e_warm, e_plain)
    assert res["n_fallback"] < 0.2 * data.shape[1]


def test_bpolyfit_and_ivim_segmented_init_match_oracle():
    from oracle import lsq_oracle
    w = synth.ivim(synth.IVIM_B21, name="ivim21")
    true, data = pipeline.synth_gpu(w, 20000, seed=4, device=DEV)
    d = data.cpu().numpy()
    b = np.array(w.protocol)
    for deg in (1, 2, 3):
        got = pipeline.bpolyfit(data, deg, x_shared=list(-b[2:14] / 1000.0), row0=2, rows=12, log_y=True)
        want = lsq_oracle.bpolyfit(-b[2:14] / 1000.0, np.log(d[2:14]), deg)
        np.testing.assert_allclose(got.cpu().numpy(), want, rtol=2e-5, atol=2e-5 * np.abs(want).max())
    # per-voxel x
    xv = torch.from_numpy(np.ascontiguousarray(np.broadcast_to(-b[:10, None], (10, 20000)).astype(np.float32)))
    got = pipeline.bpolyfit(data, 1, x=xv.to(DEV), rows=10, log_y=True)
    want = lsq_oracle.bpolyfit(-b[:10], np.log(d[:10]), 1)
    np.testing.assert_allclose(got.cpu().numpy(), want, rtol=2e-5, atol=1e-7)
    # the notebook recipe on 21 b-values: rows [0, 10) and [15, 21)
    pars, lbv, ubv = pipeline.ivim_segmented_init(data, w.protocol, (0, 10), (15, 21), w.lb, w.ub)
    p_o, lb_o, ub_o = lsq_oracle.ivim_segmented_init(d, w.protocol, slice(0, 10), slice(15, 21), w.lb, w.ub)
    np.testing.assert_allclose(pars.cpu().numpy(), p_o, rtol=1e-4, atol=1e-6)
    np.testing.assert_allclose(lbv.cpu().numpy(), lb_o, rtol=1e-4, atol=1e-8)
    np.testing.assert_allclose(ubv.cpu().numpy(), ub_o, rtol=1e-4, atol=1e-8)
