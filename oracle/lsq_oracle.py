"""CPU oracle of the segmented initialisation (TEST INFRASTRUCTURE ONLY).

bpolyfit restates pycompute/cuda/lsq.py:18-26 (a batched pinv of the
Vandermonde matrix times y); ivim_segmented_init restates the IVIM notebook's
recipe (test/ivim/test_ivim.ipynb cell 6: two degree-1 fits of log S against
-b on the low- and high-b rows; cell 10: data-driven bounds).
"""
from __future__ import annotations

import numpy as np


def bpolyfit(x, y, deg):
    """x: (rows, N) or (rows,), y: (rows, N) -> (deg + 1, N) coefficients of x^0..x^deg."""
    y = np.asarray(y, dtype=np.float64)
    rows, N = y.shape
    x = np.broadcast_to(np.asarray(x, dtype=np.float64).reshape(rows, -1), (rows, N))
    A = np.ones((N, rows, deg + 1))
    for i in range(1, deg + 1):
        A[:, :, i] = (x ** i).T
    pA = np.linalg.pinv(A)
    return (pA @ y.T[:, :, None])[:, :, 0].T


def ivim_segmented_init(data, bvals, low, high, lb, ub):
    """Initial IVIM parameters and per-voxel bounds from the segmented fits."""
    b = np.asarray(bvals, dtype=np.float64)
    d = np.asarray(data, dtype=np.float64)
    lo = bpolyfit(-b[low], np.log(d[low]), 1)
    hi = bpolyfit(-b[high], np.log(d[high]), 1)
    lo[0] = np.exp(lo[0])
    hi[0] = np.exp(hi[0])
    with np.errstate(all="ignore"):
        p = np.stack([lo[0], 1.0 - hi[0] / lo[0], lo[1], hi[1]])
    p = np.nan_to_num(p, nan=0.0, posinf=0.0, neginf=0.0)
    p = np.clip(p, np.asarray(lb)[:, None], np.asarray(ub)[:, None])
    lbv = np.stack([np.maximum(p[0] / 2, 500), np.maximum(p[1] - 0.4, 0.001), np.maximum(p[2] / 200.0, 1e-6),
                    np.maximum(p[3] / 200.0, 1e-8)])
    ubv = np.stack([np.minimum(p[0] * 2, 20000), np.minimum(p[1] + 0.4, 0.999), np.minimum(p[2] * 200.0, 0.1),
                    np.minimum(p[3] * 200.0, 0.02)])
    return p, lbv, ubv
