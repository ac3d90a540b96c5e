"""The refill schedule (persistent grid, converged lanes take new voxels)
against the one-voxel-per-thread grid: every output buffer must be bitwise
identical, since each voxel runs the same arithmetic in the same order and
only the lane that runs it changes."""
import numpy as np
import pytest
import torch

from pycompute_gb300 import Expr, SecondOrderLevenbergMarquardt, synth

pytestmark = pytest.mark.gpu
DEV = "cuda:0"
BUFS = ("pars_t", "step_t", "lam_t", "step_type_t", "f_t", "first_f", "last_f", "iters_t")


def _setup(w, N, dtype=torch.float32, solve=torch.float64, per_voxel=False, seed=3):
    _, data, init, lb, ub, prot = w.generate(N, seed=seed, dtype=np.float64)
    solm = SecondOrderLevenbergMarquardt(Expr(w.expr, w.pars, w.consts), None, w.M, dtype, solve_dtype=solve)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dtype).to(DEV)  # noqa: E731
    if per_voxel:
        solm.detect_shared = False
        consts = t(np.broadcast_to(prot[:, None], (len(prot), N)))
        lbt, ubt = t(np.broadcast_to(lb[:, None], (len(lb), N))), t(np.broadcast_to(ub[:, None], (len(ub), N)))
    else:
        consts, lbt, ubt = t(prot), t(lb), t(ub)
    solm.setup(t(init), consts, t(data), lbt, ubt)
    solm.first_f.fill_(-1.0)  # left unwritten by a zero-iteration run: start both fitters equal
    solm.last_f.fill_(-1.0)
    return solm


def _state(solm):
    return {k: getattr(solm, k).clone() for k in BUFS}


def _assert_same(a, b):
    for k in BUFS:
        x, y = a[k], b[k]
        same = (x == y) | (torch.isnan(x) & torch.isnan(y)) if x.is_floating_point() else (x == y)
        assert bool(same.all()), f"{k}: {int((~same).sum())} of {x.numel()} differ"


def _pair(w, N, iters, **kw):
    g = _setup(w, N, **kw)
    r = _setup(w, N, **kw)
    g.run(iters, 1e-8)
    r.run(iters, 1e-8, schedule="refill")
    torch.cuda.synchronize()
    return g, r


@pytest.mark.parametrize("N", [1, 31, 33, 1025, 100003])
def test_refill_matches_grid_ragged(N):
    g, r = _pair(synth.ivim(), N, 40)
    _assert_same(_state(g), _state(r))


@pytest.mark.parametrize("wl", [synth.t2star, synth.vfa_t1, synth.biexp_t2])
@pytest.mark.parametrize("solve", [torch.float32, torch.float64])
def test_refill_matches_grid_models(wl, solve):
    g, r = _pair(wl(), 50000, 60, solve=solve)
    _assert_same(_state(g), _state(r))


def test_refill_matches_grid_fp64_and_per_voxel():
    w = synth.ivim()
    g, r = _pair(w, 20000, 30, dtype=torch.float64, solve=torch.float64)
    _assert_same(_state(g), _state(r))
    g, r = _pair(w, 20000, 30, per_voxel=True)
    _assert_same(_state(g), _state(r))


@pytest.mark.parametrize("iters", [0, 1])
def test_refill_zero_and_one_iteration(iters):
    g, r = _pair(synth.ivim(), 4099, iters)
    _assert_same(_state(g), _state(r))


def test_refill_continues_converged_state():
    """A second run starts with most voxels already converged (step_type 0)."""
    w = synth.ivim()
    g, r = _setup(w, 30000), _setup(w, 30000)
    g.run(60, 1e-3)
    r.run(60, 1e-3, schedule="refill")
    torch.cuda.synchronize()
    _assert_same(_state(g), _state(r))
    assert float((g.step_type_t == 0).float().mean()) > 0.3
    g.run(25, 1e-8)
    r.run(25, 1e-8, schedule="refill")
    torch.cuda.synchronize()
    _assert_same(_state(g), _state(r))


def test_refill_subset_matches_grid_subset():
    w = synth.t2star()
    N = 40000
    g, r = _setup(w, N), _setup(w, N)
    gen = torch.Generator().manual_seed(5)
    idx = torch.randperm(N, generator=gen)[:12345].to(torch.int32).to(DEV)
    pad = torch.cat([idx, torch.full((100,), -7, dtype=torch.int32, device=DEV)])  # entries past n_items unused
    g.run_subset(pad, 12345, 50, 1e-8)
    r.run_subset(pad, 12345, 50, 1e-8, schedule="refill")
    torch.cuda.synchronize()
    _assert_same(_state(g), _state(r))
    untouched = torch.ones(N, dtype=torch.bool, device=DEV)
    untouched[idx.long()] = False
    assert bool((r.iters_t[0][untouched] == 0).all())
    r.run_subset(pad, 0, 50, 1e-8, schedule="refill")  # empty subset: no launch, no change
    torch.cuda.synchronize()
    _assert_same(_state(g), _state(r))


def test_refill_rejects_bad_schedule():
    solm = _setup(synth.ivim(), 64)
    with pytest.raises(ValueError):
        solm.run(5, schedule="bogus")
