"""Lockstep comparison of a fitter with the reference's own LM kernel
(TEST INFRASTRUCTURE ONLY: parity tests and the checker block of the
benchmark's CPU-baseline leg).

Both fitters start every iteration from the reference's state: before each
iteration the reference kernel's parameters, damping, step code and cost are
copied into the fitter under test; then each runs one iteration. The
decisions of one iteration - the convergence test (pycompute/cuda/lsqnonlin.py:695-724,
called at :893-899), the gain-ratio accept/reject branch and the damping update
(:441-491) - are therefore compared on identical inputs at every iteration of
the whole run, without the drift that makes a full-run comparison of two fp32
implementations statistical.

Which decisions fp32 can resolve. Near the end of a fit most voxels come to
rest: the actual cost reduction of the trial step is of the order of the fp32
rounding error of the cost itself, and the accept/reject test then follows
that rounding. Two correct fp32 implementations whose residual, Jacobian and
Hessian expressions round differently (a different common-subexpression
association, a different choice of fused multiply-adds) decide such voxels
differently. Each voxel-iteration is therefore classified, from an FP64
re-evaluation of the compared quantities at both fitters' steps, as resolved
or as a tie: a tie when a threshold of one of its decisions lies within an
error bound of the fp32 evaluation -

  actual = (f - f_tp) / 2   vs 0, and vs mu * pred and eta * pred (rho > mu, eta)
  pred = s.g - s'hs / 2     vs 0
  |p - clamp(p - g)|^2      vs tol (1 + f), and p - g vs the bounds

with the bound of each quantity K u sum_i (terms of sample i) (u = 2^-24):
a residual r_i = m_i - d_i carries an absolute error of a few u |m_i|, so

  d(f)    = K u sum_i 2 |r_i| |m_i|  + M u f
  d(g_j)  = K u sum_i |J_ij| (|m_i| + |r_i|)
  d(pred) = K u sum_i (|s.J_i| (|m_i| + |r_i|) + (s.J_i)^2 + (|r_i| + |m_i|) |s' H_i s|)

Parity is stated on the resolved voxel-iterations (step codes identical),
next to the raw agreement over all voxels and the share of ties.

The IVIM model (the reference kernel's model) is evaluated here in FP64 with
its derivatives written out: m = S0 (f e1 + (1 - f) e2), e1 = exp(-b D*),
e2 = exp(-b D), parameters [S0, f, D*, D].
"""
from __future__ import annotations

import numpy as np

U32 = 2.0 ** -24
K_BOUND = 8.0


def _pk(i, j):
    return i * (i + 1) // 2 + j


def ivim_terms(p, b):
    """m (M, N), J (M, 4, N), packed Hessian of m (M, 10, N), all FP64
    tensors; p (4, N) and b (M,) torch tensors."""
    import torch

    p = p.double()
    b = b.double()[:, None]
    S0, f, ds, d = p[0][None], p[1][None], p[2][None], p[3][None]
    e1, e2 = torch.exp(-b * ds), torch.exp(-b * d)
    m = S0 * (f * e1 + (1 - f) * e2)
    J = torch.stack([f * e1 + (1 - f) * e2, S0 * (e1 - e2), -S0 * f * b * e1, -S0 * (1 - f) * b * e2], dim=1)
    z = torch.zeros_like(e1)
    H = torch.stack([z, e1 - e2, z, -f * b * e1, -S0 * b * e1, S0 * f * b * b * e1, -(1 - f) * b * e2, S0 * b * e2, z,
                     S0 * (1 - f) * b * b * e2], dim=1)
    return m, J, H


def _ties(p0, s, data, b, lb, ub, st_prev, tol, mu, eta, k=None):
    """Boolean (N,) tensor: voxels one of whose decisions, for step s, lies
    within the fp32 error bound of its threshold."""
    import torch

    k = K_BOUND if k is None else k
    p0 = p0.double()
    s = s.double()
    d = data.double()
    m, J, H = ivim_terms(p0, b)
    r = m - d
    f = (r * r).sum(0)
    mt, _, _ = ivim_terms(p0 - s, b)
    rt = mt - d
    ft = (rt * rt).sum(0)
    M = d.shape[0]
    a = 0.5 * (f - ft)
    df = k * U32 * (2 * r.abs() * m.abs()).sum(0) + M * U32 * f
    dft = k * U32 * (2 * rt.abs() * mt.abs()).sum(0) + M * U32 * ft
    da = 0.5 * (df + dft)
    g = (J * r[:, None]).sum(0)
    dg = k * U32 * (J.abs() * (m.abs() + r.abs())[:, None]).sum(0)
    sJ = (J * s[None]).sum(1)                                    # (M, N)
    sHs = torch.zeros_like(m)
    for i in range(4):
        for j in range(i + 1):
            t = H[:, _pk(i, j)] * s[i][None] * s[j][None]
            sHs = sHs + (t if i == j else 2 * t)
    q = (sJ * sJ + r * sHs).sum(0)
    pred = (s * g).sum(0) - 0.5 * q
    dpred = k * U32 * (sJ.abs() * (m.abs() + r.abs()) + sJ * sJ + (r.abs() + m.abs()) * sHs.abs()).sum(0)
    tie = (a.abs() <= da) | ((a - mu * pred).abs() <= da + mu * dpred) | \
          ((a - eta * pred).abs() <= da + eta * dpred) | (pred.abs() <= dpred)
    # convergence test: |p - clamp(p - g)|^2 < tol (1 + f), only where it can fire
    lo, hi = lb.double(), ub.double()
    t2 = p0 - g
    near_bound = ((t2 - lo).abs() <= dg) | ((t2 - hi).abs() <= dg)
    clamped = (t2 > hi) | (t2 < lo)
    tc = torch.minimum(torch.maximum(t2, lo), hi)
    dv = p0 - tc
    nrm = (dv * dv).sum(0)
    dnrm = (2 * dv.abs() * torch.where(clamped, torch.zeros_like(dg), dg)).sum(0)
    thr = tol * (1 + f)
    can_fire = ((st_prev.to(torch.int32) & 1) != 0) | clamped.any(0) | near_bound.any(0)
    tie |= can_fire & ((nrm - thr).abs() <= dnrm + tol * df)
    tie |= near_bound.any(0)
    return tie


def _iteration_stats(active, st_ours, st_ref, p_ours, p_ref, lam_ours, lam_ref, tie):
    import torch

    n = st_ref.numel()
    s = lambda t: int(t.sum().item())  # noqa: E731
    rel = ((p_ours.double() - p_ref.double()).abs() / p_ref.double().abs().clamp_min(1e-30))
    rel = torch.nan_to_num(rel, nan=float("inf")).amax(dim=0)
    same = st_ours == st_ref
    resolved = active & ~tie
    conv_o = (st_ours == 0) & active
    conv_r = (st_ref == 0) & active
    return {
        "active": s(active), "ties": s(active & tie),
        "same_step_code": s(same) / n,
        "same_step_code_resolved": s(same & resolved) / max(1, s(resolved)),
        "mismatch_resolved": s(~same & resolved),
        "converged_ref": s(conv_r), "converged_ours": s(conv_o), "converged_both": s(conv_o & conv_r),
        "params_within_1e-5": s(rel <= 1e-5) / n,
        "params_within_1e-5_same_code": s((rel <= 1e-5) & same) / max(1, s(same)),
        "params_within_1e-5_resolved": s((rel <= 1e-5) & same & resolved) / max(1, s(same & resolved)),
        "resolved_same": s(same & resolved), "resolved_same_within_1e-5": s((rel <= 1e-5) & same & resolved),
        "same_lambda": s(lam_ours == lam_ref) / n,
    }


def summarise(per_it: list[dict]) -> dict:
    """Worst iteration of each figure, totals of ties and mismatches, and the
    converged-set precision and recall summed over the run (each iteration's
    newly converged voxels)."""
    conv_r = sum(d["converged_ref"] for d in per_it)
    conv_o = sum(d["converged_ours"] for d in per_it)
    both = sum(d["converged_both"] for d in per_it)
    act = sum(d["active"] for d in per_it)
    return {
        "iterations": len(per_it),
        "min_same_step_code": min(d["same_step_code"] for d in per_it),
        "min_same_step_code_resolved": min(d["same_step_code_resolved"] for d in per_it),
        "mismatch_resolved_total": sum(d["mismatch_resolved"] for d in per_it),
        "tie_share_of_active": sum(d["ties"] for d in per_it) / max(1, act),
        "max_tie_share": max(d["ties"] / max(1, d["active"]) for d in per_it),
        "min_params_within_1e-5": min(d["params_within_1e-5"] for d in per_it),
        "min_params_within_1e-5_same_code": min(d["params_within_1e-5_same_code"] for d in per_it),
        "min_params_within_1e-5_resolved": min(d["params_within_1e-5_resolved"] for d in per_it),
        "params_within_1e-5_resolved": sum(d["resolved_same_within_1e-5"] for d in per_it) /
        max(1, sum(d["resolved_same"] for d in per_it)),
        "min_same_lambda": min(d["same_lambda"] for d in per_it),
        "converged_ref": conv_r, "converged_ours": conv_o, "converged_both": both,
        "converged_precision": both / conv_o if conv_o else 1.0,
        "converged_recall": both / conv_r if conv_r else 1.0,
    }


def lockstep_gpu(ref, solm, iters: int, bvals, lb, ub, tol=1e-8, mu=0.25, eta=0.75, acc=0.2, dec=2.0) -> list[dict]:
    """``ref``: RefGpuIVIM after setup(); ``solm``: a fitter after setup() on
    the same inputs (its own parameter tensor; shared protocol and bounds).
    ``bvals``, ``lb``, ``ub``: the protocol and bounds as sequences. Returns
    per-iteration stats."""
    import torch

    dev = ref.pars.device
    b = torch.tensor(list(bvals), dtype=torch.float64, device=dev)
    lo = torch.tensor(list(lb), dtype=torch.float64, device=dev)[:, None]
    hi = torch.tensor(list(ub), dtype=torch.float64, device=dev)[:, None]
    out = []
    for _ in range(iters):
        st_prev = ref.step_type[0].clone()
        active = st_prev != 0
        p0 = ref.pars.clone()
        solm.pars_t.copy_(ref.pars)
        solm.lam_t.copy_(ref.lam)
        solm.step_type_t.copy_(ref.step_type)
        solm.f_t.copy_(ref.f)
        solm.run(1, tol=tol, mu=mu, eta=eta, acc=acc, dec=dec)
        ref.run(1, tol=tol, mu=mu, eta=eta, acc=acc, dec=dec)
        tie = _ties(p0, ref.step, ref.data, b, lo, hi, st_prev, tol, mu, eta) | \
            _ties(p0, solm.step_t, ref.data, b, lo, hi, st_prev, tol, mu, eta)
        out.append(_iteration_stats(active, solm.step_type_t[0], ref.step_type[0], solm.pars_t, ref.pars,
                                    solm.lam_t[0], ref.lam[0], tie))
    return out


def lockstep_host(ref, ours, pars0, consts, data, lb, ub, iters: int, solve_dtype=None, tol=1e-8, mu=0.25,
                  eta=0.75) -> list[dict]:
    """The same on the host: ``ref`` a RefIVIM (the reference kernel built as
    host C++), ``ours`` an OracleModel; numpy inputs with a shared protocol
    ``consts`` (M,) and shared bounds (P,)."""
    import torch

    T = torch.from_numpy
    p_ref = pars0.copy()
    N = p_ref.shape[1]
    lam = np.full(N, 5.0, dtype=np.float32)
    st = np.ones(N, dtype=np.int8)
    f = np.zeros(N, dtype=np.float32)
    b = T(np.asarray(consts, dtype=np.float64))
    lo = T(np.asarray(lb, dtype=np.float64))[:, None]
    hi = T(np.asarray(ub, dtype=np.float64))[:, None]
    d = T(data)
    out = []
    for _ in range(iters):
        st_prev = st.copy()
        active = st_prev != 0
        p0 = p_ref.copy()
        p_o, lam_o, st_o, f_o = p_ref.copy(), lam.copy(), st.copy(), f.copy()
        r_o = ours.lm_run(p_o, consts, data, lb, ub, 1, lam=lam_o, step_type=st_o, f=f_o, solve_dtype=solve_dtype,
                          want_step=True)
        r_r = ref.lm_run(p_ref, consts, data, lb, ub, 1, lam=lam, step_type=st, f=f, want_step=True)
        tie = _ties(T(p0), T(r_r["step"]), d, b, lo, hi, T(st_prev), tol, mu, eta) | \
            _ties(T(p0), T(r_o["step"]), d, b, lo, hi, T(st_prev), tol, mu, eta)
        out.append(_iteration_stats(T(active), T(st_o), T(st), T(p_o), T(p_ref), T(lam_o), T(lam), tie))
    return out
