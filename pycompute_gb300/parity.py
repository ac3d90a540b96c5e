"""Accuracy metrics for parameter maps.

Two fits of the same voxels are compared per parameter with the relative
error |a - b| / max(|b|, tiny), and per voxel with its worst parameter.

Why the comparison is statistical beyond one iteration: the reference fitter
stops improving a voxel when the fp32 cost can no longer resolve the predicted
decrease (the gain-ratio test rejects every step and the damping grows), so
each fp32 implementation comes to rest at a slightly different point inside
the cost's rounding noise. Two fp32 implementations that differ only in the
rounding of common subexpressions (the reference's generated kernel and a
restatement of it) agree to a median of ~1e-6 but disagree by more than 1e-4
on a few percent of IVIM voxels, even on voxels whose fit is well conditioned.
Parity is therefore stated as: identical after one iteration to float
rounding; in lockstep (both fitters starting every iteration from the
reference's state) identical decisions on every voxel-iteration whose
decisions fp32 resolves; after a free-running full run a median relative
error, a fraction of voxels beyond 1e-4 and a convergence-flag agreement no
worse than that fp32-vs-fp32 noise floor (flags: 99.6 % of IVIM-10 voxels
between the reference's kernel and its restatement, because the convergence
test at tol 1e-8 fires on ~0.3 % of voxels, on a rounding-noise event).
"""
from __future__ import annotations

import numpy as np


def rel_err(a, b) -> np.ndarray:
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return np.abs(a - b) / np.maximum(np.abs(b), 1e-30)


def compare_params(a, b, mask=None) -> dict:
    """Per-voxel worst relative error of parameter maps a vs b, both (P, N)."""
    r = rel_err(a, b)
    r = np.where(np.isnan(r), np.inf, r)
    worst = r.max(axis=0)
    if mask is not None:
        worst = worst[mask]
        r = r[:, mask]
    if worst.size == 0:
        return dict(n=0, median_rel=0.0, max_rel=0.0, frac_gt_1e_4=0.0, **{"frac_gt_1e-4": 0.0})
    out = dict(
        n=int(worst.size),
        median_rel=float(np.median(worst)),
        max_rel=float(worst.max()),
        per_param_median=[float(np.median(x)) for x in r],
        per_param_q99=[float(np.quantile(x, 0.99)) for x in r],
    )
    out["frac_gt_1e-4"] = float(np.mean(worst > 1e-4))
    return out


def flags_agree(st_a, st_b) -> float:
    """Fraction of voxels whose convergence flag (step_type == 0) agrees."""
    a = np.asarray(st_a).reshape(-1) == 0
    b = np.asarray(st_b).reshape(-1) == 0
    return float(np.mean(a == b)) if a.size else 1.0


def interior_mask(p, lb, ub, rtol=1e-6) -> np.ndarray:
    """Voxels whose parameters are all strictly inside their bounds."""
    p = np.asarray(p, dtype=np.float64)
    lb = np.asarray(lb, dtype=np.float64).reshape(p.shape[0], -1)
    ub = np.asarray(ub, dtype=np.float64).reshape(p.shape[0], -1)
    tol_l = rtol * np.maximum(np.abs(lb), 1e-30)
    tol_u = rtol * np.maximum(np.abs(ub), 1e-30)
    return np.all((p > lb + tol_l) & (p < ub - tol_u), axis=0)
