"""The GPU fitter against the reference's own LM kernel running on the same
GPU (built from the reference tree into oracle/_ref; skipped where it was not
built), on the same seeded IVIM-10 inputs and the reference's launch
sequence. The fp32-solve build follows the reference's arithmetic: after one
iteration parameters agree to float rounding (the two compilers contract
different products into FMAs) and step codes agree. In lockstep (both
fitters start every iteration of a 100-iteration run from the reference's
state) every decision that fp32 resolves is the reference's; after 100
free-running iterations the comparison is statistical (see tests/test_gpu_lm.py
for why) and held to the CPU noise floor."""
import numpy as np
import pytest
import torch

import json
import os

from oracle import lockstep, ref_gpu
from pycompute_gb300 import Expr, SecondOrderLevenbergMarquardt, parity, synth

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not ref_gpu.available(10), reason="reference kernel not built (no reference tree)")]
DEV = "cuda:0"


def _inputs(N, seed):
    w = synth.ivim()
    _, data, init, lb, ub, prot = w.generate(N, seed=seed)
    return w, data, init, lb, ub, prot


def _ref_fit(data, init, lb, ub, prot, iters):
    N = data.shape[1]
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(DEV)  # noqa: E731
    ref = ref_gpu.RefGpuIVIM(10)
    pars = t(init)
    ref.setup(pars, t(np.broadcast_to(prot[:, None], (10, N))), t(data), t(np.broadcast_to(lb[:, None], (4, N))),
              t(np.broadcast_to(ub[:, None], (4, N))))
    ref.run(iters)
    torch.cuda.synchronize()
    return pars.cpu().numpy(), ref.step_type.cpu().numpy()[0], ref.last_f.cpu().numpy()[0]


def _our_fit(w, data, init, lb, ub, prot, iters, solve):
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(DEV)  # noqa: E731
    solm = SecondOrderLevenbergMarquardt(Expr(w.expr, w.pars, w.consts), None, w.M, torch.float32, solve_dtype=solve)
    pars = t(init)
    solm.setup(pars, t(prot), t(data), t(lb), t(ub))
    solm.run(iters)
    torch.cuda.synchronize()
    return pars.cpu().numpy(), solm.step_type_t.cpu().numpy()[0], solm.last_f.cpu().numpy()[0]


def test_one_iteration_matches_reference_kernel():
    w, data, init, lb, ub, prot = _inputs(65536, seed=21)
    p_ref, st_ref, f_ref = _ref_fit(data, init, lb, ub, prot, 1)
    p, st, f = _our_fit(w, data, init, lb, ub, prot, 1, torch.float32)
    # both kernels contract a*b+c into FMAs, not always the same ones: all but
    # a handful of entries agree to 1e-5, every entry to 1e-3
    rel = np.abs(p - p_ref) / np.maximum(np.abs(p_ref), 1e-30)
    assert float(np.mean(rel <= 1e-5)) > 0.9999, float(np.mean(rel <= 1e-5))
    np.testing.assert_allclose(p, p_ref, rtol=1e-3, atol=1e-12)
    np.testing.assert_allclose(f, f_ref, rtol=1e-5)
    assert float(np.mean(st == st_ref)) > 0.9999


@pytest.mark.parametrize("solve", [torch.float32, torch.float64])
def test_full_fit_matches_reference_kernel_within_noise_floor(solve):
    w, data, init, lb, ub, prot = _inputs(65536, seed=22)
    p_ref, st_ref, _ = _ref_fit(data, init, lb, ub, prot, 100)
    p, st, _ = _our_fit(w, data, init, lb, ub, prot, 100, solve)
    rep = parity.compare_params(p, p_ref)
    # the CPU noise floor between two correct fp32 builds (plain vs FMA-contracted):
    # median 1e-6, 7.8 % of voxels beyond 1e-4, flags 99.59 %
    assert rep["median_rel"] < 1e-5, rep
    assert rep["frac_gt_1e-4"] < 0.078 + 0.03, rep
    assert parity.flags_agree(st, st_ref) > 0.9959 - 0.02


@pytest.mark.parametrize("solve", [torch.float32, torch.float64])
def test_lockstep_every_iteration_matches_reference_kernel(solve):
    """1,048,576 IVIM-10 voxels, 100 iterations. Before every iteration the
    reference kernel's parameters, damping, step code and cost are copied into
    the fitter; each then runs one iteration. On every voxel-iteration whose
    decisions (convergence test, gain-ratio branch, damping update) lie
    outside the fp32 error bound of their thresholds, the step codes - 0
    included - must be the reference's on at least 99.9 % of voxels at every
    iteration; the fp32-solve build's parameters must then also agree to 1e-5
    on 99.5 % of those voxel-iterations (the rest are ill-conditioned voxels
    whose fp32 steps differ along a flat direction; measured on the host 99.7 %).
    Late in the run most voxels are at rest (their actual cost reduction is
    ~1e-6 of the cost's fp32 rounding error), and there the two builds'
    rounding decides; the raw agreement over all voxels is reported and held
    to the level measured on the host between the reference kernel and the
    fp32 oracle (96 %)."""
    N = 1 << 20
    w, data, init, lb, ub, prot = _inputs(N, seed=23)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(DEV)  # noqa: E731
    ref = ref_gpu.RefGpuIVIM(10)
    ref.setup(t(init), t(np.broadcast_to(prot[:, None], (10, N))), t(data), t(np.broadcast_to(lb[:, None], (4, N))),
              t(np.broadcast_to(ub[:, None], (4, N))))
    solm = SecondOrderLevenbergMarquardt(Expr(w.expr, w.pars, w.consts), None, w.M, torch.float32, solve_dtype=solve)
    solm.setup(t(init), t(prot), t(data), t(lb), t(ub))
    per_it = lockstep.lockstep_gpu(ref, solm, 100, prot, lb, ub)
    torch.cuda.synchronize()
    rep = lockstep.summarise(per_it)
    out = os.environ.get("PCGB_REPORT_DIR")
    if out:
        with open(os.path.join(out, f"lockstep_ivim10_1m_{'f64' if solve == torch.float64 else 'f32'}.json"), "w") as f:
            json.dump({"summary": rep, "per_iteration": per_it}, f)
    assert rep["min_same_step_code_resolved"] >= 0.999, rep
    assert rep["min_same_step_code"] >= 0.95, rep
    assert rep["min_same_lambda"] >= 0.95, rep
    if solve == torch.float32:
        assert rep["params_within_1e-5_resolved"] >= 0.995, rep
    assert rep["converged_recall"] >= 0.8, rep
