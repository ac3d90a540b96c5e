"""Seeded synthetic qMRI workloads.

The reference measured on dipy's ``ivim`` sample volume, which is not shipped
with it; these generators stand in for it with the shapes, protocols, parameter
ranges and noise model of the benchmark configurations:

* signals S = sqrt((S_true + sigma*n1)^2 + (sigma*n2)^2), n1, n2 ~ N(0, 1)
  (Rician magnitude noise),
* parameters drawn uniformly from per-model ranges,
* layouts as the reference uses them: structure-of-arrays with the voxel
  index fastest, params (P, N), data (M, N), one protocol row per sample.

Model expressions are written the way the reference writes IVIM
(``test/ivim/test_ivim.ipynb`` cell 11: ``S0*(f*exp(-b*D_1)+(1-f)*exp(-b*D_2))``
with parameters ``[S0, f, D_1, D_2]``, D_1 the pseudo-diffusion D*).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

IVIM_EXPR = "S0*(f*exp(-b*D_1)+(1-f)*exp(-b*D_2))"
IVIM_PARS = ["S0", "f", "D_1", "D_2"]
IVIM_B10 = [0, 10, 20, 50, 100, 200, 400, 600, 800, 1000]
IVIM_B21 = [0, 10, 20, 30, 40, 50, 60, 70, 80, 90, 100, 120, 140, 160, 180, 200, 300, 400, 500, 600, 1000]
# bounds of the IVIM notebook (test_ivim.ipynb cell 10, the commented fixed set)
IVIM_LB = [0.0, 1e-3, 1e-6, 1e-8]
IVIM_UB = [20000.0, 0.999, 0.1, 0.02]


def ivim_b16() -> list[float]:
    """b = 0 and 15 log-spaced values in [10, 1000] s/mm^2."""
    return [0.0] + [float(x) for x in np.geomspace(10.0, 1000.0, 15)]


@dataclass
class Workload:
    """One fitting workload: a model, a protocol and a parameter distribution."""

    name: str
    expr: str
    pars: list[str]
    consts: list[str]
    protocol: list[float]               # C*M values, constant k for sample i at k*M + i
    ranges: list[tuple[float, float]]   # uniform ranges of the true parameters
    lb: list[float]
    ub: list[float]
    snr: tuple[float, float] = (50.0, 50.0)   # sigma = S0 / snr, snr ~ U[lo, hi]
    init: str = "const"
    init_values: list[float] = field(default_factory=list)  # NaN entries = data-driven (max signal)

    @property
    def M(self) -> int:
        return len(self.protocol) // max(1, len(self.consts))

    @property
    def P(self) -> int:
        return len(self.pars)

    def model_numpy(self, p: np.ndarray, consts: np.ndarray) -> np.ndarray:
        """m for all voxels and samples, (M, N), evaluated in float64."""
        from . import codegen

        fns = codegen.numpy_functions(self.expr, self.pars, self.consts)
        m_fn = fns[0]
        M = self.M
        cs = [consts[k * M:(k + 1) * M, None] for k in range(len(self.consts))]
        out = m_fn(*[p[k][None, :] for k in range(self.P)], *cs)
        return np.broadcast_to(out, (M, p.shape[1])).astype(np.float64)

    def generate(self, n: int, seed: int = 0, dtype=np.float32):
        """Seeded (true_params, data, init_params, lb, ub, protocol).

        true/init params (P, n); data (M, n); lb/ub (P,) shared bounds;
        protocol (C*M,) shared.
        """
        rng = np.random.default_rng(seed)
        P, M = self.P, self.M
        true = np.empty((P, n), dtype=np.float64)
        for k, (lo, hi) in enumerate(self.ranges):
            true[k] = rng.uniform(lo, hi, n)
        prot = np.asarray(self.protocol, dtype=np.float64)
        clean = self.model_numpy(true, prot)
        snr = rng.uniform(self.snr[0], self.snr[1], n) if self.snr[0] != self.snr[1] else np.full(n, self.snr[0])
        sigma = true[0] / snr
        n1 = rng.standard_normal((M, n))
        n2 = rng.standard_normal((M, n))
        data = np.sqrt((clean + sigma * n1) ** 2 + (sigma * n2) ** 2)
        init = np.empty((P, n), dtype=np.float64)
        for k, v in enumerate(self.init_values):
            init[k] = data.max(axis=0) if np.isnan(v) else v
        return (true.astype(dtype), np.ascontiguousarray(data.astype(dtype)), np.ascontiguousarray(init.astype(dtype)),
                np.asarray(self.lb, dtype=dtype), np.asarray(self.ub, dtype=dtype), prot.astype(dtype))


def ivim(bvals=None, name="ivim10", snr=(50.0, 50.0), f_range=(0.05, 0.35)) -> Workload:
    """IVIM bi-exponential, params [S0, f, D*, D]; init [max S, 0.1, 1e-2, 1e-3]."""
    b = list(IVIM_B10 if bvals is None else bvals)
    return Workload(
        name=name, expr=IVIM_EXPR, pars=list(IVIM_PARS), consts=["b"], protocol=[float(x) for x in b],
        ranges=[(500.0, 1500.0), f_range, (5e-3, 5e-2), (0.5e-3, 2.5e-3)],
        lb=list(IVIM_LB), ub=list(IVIM_UB), snr=snr, init_values=[np.nan, 0.1, 1e-2, 1e-3])


def vfa_t1() -> Workload:
    """Variable flip angle T1 (TR = 15 ms folded as a literal), 8 angles 2-30 deg."""
    angles = np.deg2rad(np.linspace(2.0, 30.0, 8))
    return Workload(
        name="vfa8", expr="S0*sin(a)*(1-exp(-15/T1))/(1-cos(a)*exp(-15/T1))", pars=["S0", "T1"], consts=["a"],
        protocol=[float(x) for x in angles], ranges=[(500.0, 1500.0), (300.0, 3000.0)],
        lb=[0.0, 10.0], ub=[50000.0, 10000.0], snr=(30.0, 100.0), init_values=[np.nan, 1000.0])


def t2star() -> Workload:
    """Mono-exponential T2* decay with offset, 16 echoes TE = 2-40 ms (R2* in 1/s)."""
    te = np.linspace(2.0, 40.0, 16)
    return Workload(
        name="t2s16", expr="S0*exp(-TE*R2s/1000)+c", pars=["S0", "R2s", "c"], consts=["TE"],
        protocol=[float(x) for x in te], ranges=[(500.0, 1500.0), (10.0, 200.0), (0.0, 50.0)],
        lb=[0.0, 0.0, -1000.0], ub=[50000.0, 1000.0, 1000.0], snr=(30.0, 100.0),
        init_values=[np.nan, 50.0, 0.0])


def biexp_t2() -> Workload:
    """Bi-exponential T2 with offset, 32 echoes TE = 10-320 ms (5 params)."""
    te = np.linspace(10.0, 320.0, 32)
    return Workload(
        name="biexp32", expr="S0*(f*exp(-TE/T2s)+(1-f)*exp(-TE/T2l))+c", pars=["S0", "f", "T2s", "T2l", "c"],
        consts=["TE"], protocol=[float(x) for x in te],
        ranges=[(500.0, 1500.0), (0.1, 0.5), (10.0, 40.0), (60.0, 300.0), (0.0, 50.0)],
        lb=[0.0, 0.0, 1.0, 20.0, -1000.0], ub=[50000.0, 1.0, 60.0, 2000.0, 1000.0], snr=(30.0, 100.0),
        init_values=[np.nan, 0.3, 20.0, 100.0, 0.0])
