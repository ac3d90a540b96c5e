"""Fit pipeline on the GPU: synthetic signals, constant initialisation, and
the warm-started fit with its plain-LM fallback.

Warm-started fit (``WarmStartFitter.fit``):
  1. the network predicts initial parameters from each voxel's signals;
  2. the LM runs ``iters_warm`` iterations from there, starting with a small
     damping ``lam0`` (the start is already close: the reference's lam = 5
     would shrink the first steps to a sixth of a Gauss-Newton step);
  3. in the same kernel, a voxel is flagged when its warm fit lands on a
     bound, has a non-finite cost, or does not end below the cost of the
     constant initialisation (the plain fitter's starting point);
  4. flagged voxels are compacted into an index list and refitted by the
     plain LM from the constant initialisation for ``iters_fallback``
     iterations in one launch over that list;
  5. each refitted voxel keeps whichever of the two fits has the lower cost.
Every step is a kernel of libpcgb.so; PyTorch only holds the buffers.
"""
from __future__ import annotations

import ctypes

import torch

from . import _lib
from .lsqnonlin import Expr, SecondOrderLevenbergMarquardt
from .synth import Workload


def _p(t):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _dvec(vals):
    return (ctypes.c_double * len(vals))(*[float(v) for v in vals])


def init_constant(data: torch.Tensor, values, out: torch.Tensor | None = None) -> torch.Tensor:
    """(P, N) constant initial parameters; NaN entries take the voxel's largest sample."""
    M, N = data.shape
    P = len(values)
    out = torch.empty((P, N), dtype=torch.float32, device=data.device) if out is None else out
    rc = _lib.lib().pcgb_init_constant(_p(data), N, M, P, _dvec(values), _p(out), _stream())
    _lib.check("pcgb_init_constant", rc)
    return out


def synth_gpu(w: Workload, n: int, seed: int, device="cuda", snr=None):
    """Seeded synthetic signals on the GPU: (true params (P, n), signals (M, n)).

    Parameters uniform in the workload's ranges, signals from the fitter's own
    forward-model kernel, Rician magnitude noise with sigma = S0 / SNR.
    """
    dev = torch.device(device)
    g = torch.Generator(device=dev).manual_seed(seed)
    P, M = w.P, w.M
    true = torch.empty((P, n), dtype=torch.float32, device=dev)
    for k, (lo, hi) in enumerate(w.ranges):
        true[k] = torch.rand(n, generator=g, device=dev) * (hi - lo) + lo
    fitter = SecondOrderLevenbergMarquardt(Expr(w.expr, w.pars, w.consts), None, M, torch.float32)
    prot = torch.tensor(w.protocol, dtype=torch.float32, device=dev)
    lb = torch.tensor(w.lb, dtype=torch.float32, device=dev)
    ub = torch.tensor(w.ub, dtype=torch.float32, device=dev)
    dummy = torch.zeros((M, n), dtype=torch.float32, device=dev)
    fitter.setup(true.clone(), prot, dummy, lb, ub)
    clean = fitter.model_eval(true)
    lo, hi = snr if snr is not None else w.snr
    s = torch.rand(n, generator=g, device=dev) * (hi - lo) + lo if lo != hi else torch.full((n,), lo, device=dev)
    sigma = true[0] / s
    n1 = torch.randn((M, n), generator=g, device=dev)
    n2 = torch.randn((M, n), generator=g, device=dev)
    data = torch.sqrt((clean + sigma * n1) ** 2 + (sigma * n2) ** 2).contiguous()
    return true, data


class WarmStartFitter:
    """Network initialisation + LM + plain-LM fallback (see module docstring)."""

    def __init__(self, w: Workload, net, solve_dtype=torch.float64):
        self.w = w
        self.net = net
        self.solve_dtype = solve_dtype
        self.expr = Expr(w.expr, w.pars, w.consts)
        self._solm = None
        self._dev_consts = {}
        self.refit_schedule = "grid"  # or "refill": schedule of the fallback refit

    def _fitter(self):
        if self._solm is None:
            self._solm = SecondOrderLevenbergMarquardt(self.expr, None, self.w.M, torch.float32,
                                                       solve_dtype=self.solve_dtype, detect_shared=False)
        return self._solm

    def _consts(self, dev):
        # shared protocol and bounds as host values: setup() needs no device read-back
        w = self.w
        return list(w.protocol), list(w.lb), list(w.ub)

    def fit_host(self, data_h: torch.Tensor, out_h: torch.Tensor, iters_warm: int, iters_fallback: int,
                 lam0: float = 1e-3, chunks: int = 8, device=None) -> torch.Tensor:
        """Warm-started fit of host-resident signals, streamed through the GPU.

        data_h (M, N) and out_h (P, N) are float32 host tensors (pinned, so the
        copies overlap the fits). The voxels go through in ``chunks`` ranges:
        chunk c is copied in on one stream while chunk c-1 is fitted on
        another and chunk c-2's parameters are copied back on a third; every
        voxel's result equals fit()'s. Returns the device int32 tensor
        [fallback voxels, refits kept] summed over chunks. Work is ordered
        after the caller's current stream, and the caller's stream waits for
        the last copy back.
        """
        M, N = data_h.shape
        P = self.w.P
        if tuple(out_h.shape) != (P, N) or data_h.dtype != torch.float32 or out_h.dtype != torch.float32:
            raise ValueError("data_h must be (M, N) and out_h (P, N) float32")
        dev = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
        if N == 0:
            return torch.zeros(2, dtype=torch.int32, device=dev)
        chunks = max(1, min(int(chunks), (N + 127) // 128))
        n_c = (N + chunks - 1) // chunks
        n_c = (n_c + 127) // 128 * 128
        nchunk = (N + n_c - 1) // n_c
        slots = 2
        key = (M, P, n_c, str(dev))
        if getattr(self, "_host_key", None) != key:
            self._host = dict(data=[torch.empty(M * n_c, dtype=torch.float32, device=dev) for _ in range(slots)],
                              pars=[torch.empty(P * n_c, dtype=torch.float32, device=dev) for _ in range(slots)],
                              streams=[torch.cuda.Stream(device=dev) for _ in range(3)])
            self._host_key = key
        hb = self._host
        s_in, s_fit, s_out = hb["streams"]
        caller = torch.cuda.current_stream(dev)
        for st in (s_in, s_fit, s_out):
            st.wait_stream(caller)
        total = torch.zeros(2, dtype=torch.int32, device=dev)
        total.record_stream(s_fit)
        ev_in = [torch.cuda.Event() for _ in range(nchunk)]
        ev_fit = [torch.cuda.Event() for _ in range(nchunk)]
        ev_out = [torch.cuda.Event() for _ in range(nchunk)]
        for c in range(nchunk):
            lo = c * n_c
            n = min(N, lo + n_c) - lo
            k = c % slots
            d = hb["data"][k][:M * n].view(M, n)
            p = hb["pars"][k][:P * n].view(P, n)
            with torch.cuda.stream(s_in):
                if c >= slots:
                    s_in.wait_event(ev_fit[c - slots])  # the slot's signals are no longer read
                copy_rows(d, 0, data_h, lo, n)
                ev_in[c].record(s_in)
            with torch.cuda.stream(s_fit):
                s_fit.wait_event(ev_in[c])
                if c >= slots:
                    s_fit.wait_event(ev_out[c - slots])  # the slot's parameters are copied out
                res = self.fit(d, iters_warm, iters_fallback, pars_out=p, lam0=lam0)
                total.add_(res.counts)
                ev_fit[c].record(s_fit)
            with torch.cuda.stream(s_out):
                s_out.wait_event(ev_fit[c])
                copy_rows(out_h, lo, p, 0, n)
                ev_out[c].record(s_out)
        caller.wait_stream(s_fit)
        caller.wait_stream(s_out)
        return total

    def fit_stream(self, volumes, iters_warm: int, iters_fallback: int, lam0: float = 1e-3, device=None):
        """Warm-started fits of a sequence of host-resident volumes.

        volumes: iterable of (data_h (M, N), out_h (P, N)) float32 host tensors
        (pinned, so the copies overlap the fits; N may differ between
        volumes). Two device slots alternate: while volume i is fitted, volume
        i+1 is copied in and volume i-1's parameters are copied back, so in
        steady state each volume costs its fit alone. Every volume's result
        equals fit()'s. Returns the device int32 tensor [fallback voxels,
        refits kept] summed over volumes; the caller's stream waits for the
        last copy back.
        """
        dev = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
        P = self.w.P
        if getattr(self, "_stream_key", None) != str(dev):
            self._streams3 = [torch.cuda.Stream(device=dev) for _ in range(3)]
            self._stream_slots = [{}, {}]
            self._stream_key = str(dev)
        s_in, s_fit, s_out = self._streams3
        caller = torch.cuda.current_stream(dev)
        for st in (s_in, s_fit, s_out):
            st.wait_stream(caller)
        total = torch.zeros(2, dtype=torch.int32, device=dev)
        total.record_stream(s_fit)
        ev_fit, ev_out = [], []
        for i, (data_h, out_h) in enumerate(volumes):
            M, N = data_h.shape
            if tuple(out_h.shape) != (P, N) or data_h.dtype != torch.float32 or out_h.dtype != torch.float32:
                raise ValueError("each volume needs data (M, N) and out (P, N) float32 host tensors")
            slot = self._stream_slots[i % 2]
            if slot.get("shape") != (M, N):
                with torch.cuda.stream(s_in):  # the slot's previous buffers are released on s_in's order
                    slot.update(shape=(M, N), data=torch.empty((M, N), dtype=torch.float32, device=dev),
                                pars=torch.empty((P, N), dtype=torch.float32, device=dev))
            d, p = slot["data"], slot["pars"]
            d.record_stream(s_fit)  # the allocator may reuse the slots only after these streams' work
            p.record_stream(s_fit)
            p.record_stream(s_out)
            ev_in = torch.cuda.Event()
            with torch.cuda.stream(s_in):
                if i >= 2:
                    s_in.wait_event(ev_fit[i - 2])  # the slot's signals are no longer read
                d.copy_(data_h, non_blocking=True)
                ev_in.record(s_in)
            with torch.cuda.stream(s_fit):
                s_fit.wait_event(ev_in)
                if i >= 2:
                    s_fit.wait_event(ev_out[i - 2])  # the slot's parameters are copied out
                res = self.fit(d, iters_warm, iters_fallback, pars_out=p, lam0=lam0)
                total.add_(res.counts)
                ev_fit.append(torch.cuda.Event())
                ev_fit[-1].record(s_fit)
            with torch.cuda.stream(s_out):
                s_out.wait_event(ev_fit[-1])
                out_h.copy_(p, non_blocking=True)
                ev_out.append(torch.cuda.Event())
                ev_out[-1].record(s_out)
        caller.wait_stream(s_fit)
        caller.wait_stream(s_out)
        return total

    def _warm_check(self, solm, data, pars, b):
        """The fallback check as its own kernel (pcgb_warm_check)."""
        w = self.w
        pv, plen = solm._proto_args()
        rc = _lib.lib().pcgb_warm_check(
            solm.build().handle, _p(solm.consts_t), solm._cstride, _p(data), _p(solm.lower_bound_t),
            _p(solm.upper_bound_t), solm._bstride, pv, plen, _dvec(solm._lb_host) if solm._bstride == 0 else None,
            _dvec(solm._ub_host) if solm._bstride == 0 else None, _dvec(w.init_values), 5.0, _p(pars),
            _p(solm.lam_t), _p(solm.step_type_t), _p(solm.f_t), _p(b["cost"]), _p(b["backup"]), _p(b["cost_b"]),
            _p(b["idx"]), _p(b["counts"]), data.shape[1], _stream())
        _lib.check("pcgb_warm_check", rc)

    def _warm_lm_check(self, solm, data, pars, b, iters_warm, lam0, tol=1e-8, mu=0.25, eta=0.75, acc=0.2, dec=2.0):
        """The warm LM from a fresh start with the fallback check as its
        epilogue (pcgb_warm_lm_check)."""
        w = self.w
        pv, plen = solm._proto_args()
        rc = _lib.lib().pcgb_warm_lm_check(
            solm.build().handle, _p(solm.consts_t), solm._cstride, _p(data), _p(solm.lower_bound_t),
            _p(solm.upper_bound_t), solm._bstride, float(tol), float(mu), float(eta), float(acc), float(dec),
            int(iters_warm), float(lam0), pv, plen, _dvec(solm._lb_host) if solm._bstride == 0 else None,
            _dvec(solm._ub_host) if solm._bstride == 0 else None, _dvec(w.init_values), 5.0, _p(pars),
            _p(solm.lam_t), _p(solm.step_type_t), _p(solm.f_t), _p(b["cost"]), _p(b["backup"]), _p(b["cost_b"]),
            _p(b["idx"]), _p(b["counts"]), data.shape[1], 0, _stream())
        _lib.check("pcgb_warm_lm_check", rc)

    def _buffers(self, P: int, N: int, dev):
        key = (P, N, str(dev))
        if getattr(self, "_buf_key", None) != key:
            self._buf = dict(cost=torch.empty(N, dtype=torch.float32, device=dev),
                             backup=torch.empty((P, N), dtype=torch.float32, device=dev),
                             cost_b=torch.empty(N, dtype=torch.float32, device=dev),
                             idx=torch.empty(N, dtype=torch.int32, device=dev),
                             counts=torch.zeros(2, dtype=torch.int32, device=dev))
            self._buf_key = key
        # used on the current stream: replaced buffers are not reused before its work ends
        st = torch.cuda.current_stream(dev)
        for t in self._buf.values():
            t.record_stream(st)
        return self._buf

    def fit(self, data: torch.Tensor, iters_warm: int, iters_fallback: int, pars_out: torch.Tensor | None = None,
            lam0: float = 1e-3, timings: dict | None = None, fused="lean", events: list | None = None):
        """Warm-started fit of data (M, N); returns a WarmFit.

        ``fused="lean"`` (default) runs the warm LM from a fresh start and
        the check as one kernel (the warm fit's cost taken from the iterations
        instead of re-evaluated; the same rule, its cost comparisons on costs
        rounded differently, so a voxel whose two costs tie to rounding may be
        flagged differently) and the select as the refit's epilogue;
        ``fused="select"`` runs the fallback check as its own kernel and the
        select as the epilogue of the refit launch;
        ``fused="epilogue"`` also runs the check as the epilogue of the warm
        LM launch (the signals are read once, but the LM kernel then holds
        more registers); ``fused=True`` runs check, refit and select as three
        kernels of their own; ``fused=False`` as the separate pipeline kernels
        (cost, constant start, cost, flags, prepare, refit, cost, select).
        The flagged count never returns to the host except with
        ``fused=False``. All give the same results.
        ``timings`` (a dict) receives per-stage milliseconds (synchronises);
        ``events`` (a list) receives (stage, CUDA event) pairs recorded after
        each stage on the current stream, without synchronising.
        """
        w = self.w
        dev = data.device
        M, N = data.shape
        P = w.P
        prot, lb, ub = self._consts(dev)
        ev = []

        def mark(name):
            if timings is not None or events is not None:
                e = torch.cuda.Event(enable_timing=True)
                e.record()
                ev.append((name, e))
                if events is not None:
                    events.append((name, e))

        mark("start")
        pars = self.net.infer(data, out=pars_out)
        mark("network")
        solm = self._fitter()
        if fused in ("select", "lean"):
            # the warm LM reads no state and keeps only the parameters and step
            # codes; the check initialises the state of the voxels it flags
            solm.setup(pars, prot, data, lb, ub, init_state=False)
        else:
            solm.setup(pars, prot, data, lb, ub)
            solm.lam_t.fill_(lam0)
        mark("setup")
        if fused in ("epilogue", "select", "lean"):
            b = self._buffers(P, N, dev)
            if fused == "lean":  # fresh warm LM with the check as its epilogue
                self._warm_lm_check(solm, data, pars, b, iters_warm, lam0)
                mark("lm_warm")
                mark("check")
            elif fused == "epilogue":  # the check as the warm LM's epilogue
                solm.run_check(iters_warm, w.init_values, 5.0, b["cost"], b["backup"], b["cost_b"], b["idx"],
                               b["counts"])
                mark("lm_warm")
                mark("check")
            else:
                solm.run_fresh(iters_warm, lam0)
                mark("lm_warm")
                self._warm_check(solm, data, pars, b)
                mark("check")
            # the select as the refit's epilogue
            solm.run_select(iters_fallback, b["cost"], b["backup"], b["cost_b"], b["idx"], b["counts"])
            mark("refit")
            mark("select")
            if timings is not None:
                torch.cuda.synchronize()
                for (n0, e0), (n1, e1) in zip(ev[:-1], ev[1:]):
                    timings[n1] = timings.get(n1, 0.0) + e0.elapsed_time(e1)
            return WarmFit(pars, b["cost"], b["counts"], solm.step_type_t, b["idx"])
        solm.run(iters_warm)
        mark("lm_warm")
        if fused:
            b = self._buffers(P, N, dev)
            L = _lib.lib()
            prog = solm.build()
            pv, plen = solm._proto_args()
            self._warm_check(solm, data, pars, b)
            mark("check")
            solm.run_subset(b["idx"], N, iters_fallback, schedule=self.refit_schedule, n_items_dev=b["counts"])
            mark("refit")
            rc = L.pcgb_warm_select(prog.handle, _p(solm.consts_t), solm._cstride, _p(data), pv, plen, _p(pars),
                                    _p(b["cost"]), _p(b["backup"]), _p(b["cost_b"]), _p(b["idx"]), _p(b["counts"]),
                                    None, N, _stream())
            _lib.check("pcgb_warm_select", rc)
            mark("select")
            if timings is not None:
                torch.cuda.synchronize()
                for (n0, e0), (n1, e1) in zip(ev[:-1], ev[1:]):
                    timings[n1] = timings.get(n1, 0.0) + e0.elapsed_time(e1)
            return WarmFit(pars, b["cost"], b["counts"], solm.step_type_t, b["idx"])
        cost = solm.cost()
        # cost at the plain fitter's starting point
        p0 = init_constant(data, w.init_values)
        cost0 = solm.cost(p0)
        mark("costs")
        idx = torch.empty(N, dtype=torch.int32, device=dev)
        count = torch.zeros(1, dtype=torch.int32, device=dev)
        L = _lib.lib()
        rc = L.pcgb_fallback_flags(_p(pars), _p(cost), _p(cost0), N, P, _dvec(w.lb), _dvec(w.ub), None, _p(idx),
                                   _p(count), _stream())
        _lib.check("pcgb_fallback_flags", rc)
        nfb = int(count.item())
        mark("flags")
        kept_refit = 0
        if nfb:
            backup = torch.empty((P, nfb), dtype=torch.float32, device=dev)
            cost_b = torch.empty(nfb, dtype=torch.float32, device=dev)
            rc = L.pcgb_fallback_prepare(_p(idx), nfb, N, P, M, _dvec(w.init_values), _p(pars), _p(backup), _p(cost),
                                         _p(cost_b), _p(data), _p(solm.lam_t), 5.0, _p(solm.step_type_t),
                                         _p(solm.f_t), _stream())
            _lib.check("pcgb_fallback_prepare", rc)
            solm.run_subset(idx, nfb, iters_fallback)
            cost.index_fill_(0, idx[:nfb].long(), 0.0)
            solm.cost(vox_idx=idx, n_items=nfb, out=cost)
            which = torch.zeros(N, dtype=torch.int8, device=dev)
            rc = L.pcgb_fallback_select(_p(idx), nfb, N, P, _p(pars), _p(backup), _p(cost), _p(cost_b), _p(which),
                                        _stream())
            _lib.check("pcgb_fallback_select", rc)
            kept_refit = int(which.sum().item())
        mark("fallback")
        if timings is not None:
            torch.cuda.synchronize()
            for (n0, e0), (n1, e1) in zip(ev[:-1], ev[1:]):
                timings[n1] = timings.get(n1, 0.0) + e0.elapsed_time(e1)
        return WarmFit(pars, cost, torch.tensor([nfb, kept_refit], dtype=torch.int32), solm.step_type_t)


def copy_rows(dst: torch.Tensor, dst_col: int, src: torch.Tensor, src_col: int, ncols: int):
    """dst[:, dst_col:dst_col+ncols] = src[:, src_col:src_col+ncols] for 2-D float32
    row-major tensors (host or device), asynchronously on the current stream."""
    rows = src.shape[0]
    if dst.shape[0] != rows or dst.dtype != src.dtype or not (dst.is_contiguous() and src.is_contiguous()):
        raise ValueError("copy_rows needs contiguous 2-D tensors of the same dtype and row count")
    es = src.element_size()
    direction = 0 if (dst.is_cuda and not src.is_cuda) else (1 if (src.is_cuda and not dst.is_cuda) else 2)
    if not dst.is_cuda and not src.is_cuda:
        raise ValueError("copy_rows copies to or from the device")
    rc = _lib.lib().pcgb_copy_rows_async(ctypes.c_void_p(dst.data_ptr() + dst_col * es), dst.stride(0) * es,
                                         ctypes.c_void_p(src.data_ptr() + src_col * es), src.stride(0) * es,
                                         ncols * es, rows, direction, _stream())
    _lib.check("pcgb_copy_rows_async", rc)


class WarmFit:
    """Result of WarmStartFitter.fit: pars (P, N), cost (N), step_type (1, N)
    on the device; fallback_idx (int32, N) lists the flagged voxels in its
    first n_fallback entries (None for the unfused pipeline); n_fallback /
    n_refit_kept read the device counters (a sync)."""

    def __init__(self, pars, cost, counts, step_type, fallback_idx=None):
        self.pars, self.cost, self.counts, self.step_type = pars, cost, counts, step_type
        self.fallback_idx = fallback_idx

    @property
    def n_fallback(self) -> int:
        return int(self.counts[0].item())

    @property
    def n_refit_kept(self) -> int:
        return int(self.counts[1].item())

    def __getitem__(self, key):
        return getattr(self, key)


def bpolyfit(y: torch.Tensor, deg: int, x_shared=None, x: torch.Tensor | None = None, row0: int = 0,
             rows: int | None = None, log_y: bool = False) -> torch.Tensor:
    """Per-voxel polynomial least squares (the reference's bpolyfit, pycompute/cuda/lsq.py:18-26).

    Fits rows [row0, row0 + rows) of y (M, N) (or their log) on 1, x, ..., x^deg;
    x is a shared host sequence of `rows` values or a (rows, N) device tensor.
    Returns the (deg + 1, N) coefficients.
    """
    M, N = y.shape
    rows = M - row0 if rows is None else rows
    out = torch.empty((deg + 1, N), dtype=torch.float32, device=y.device)
    xs = _dvec(x_shared) if x_shared is not None else None
    rc = _lib.lib().pcgb_bpolyfit(_p(x), N if x is not None else 0, xs, _p(y), N, int(row0), int(rows), int(deg),
                                  int(log_y), _p(out), _stream())
    _lib.check("pcgb_bpolyfit", rc)
    return out


def ivim_segmented_init(data: torch.Tensor, bvals, low: tuple[int, int], high: tuple[int, int], lb, ub,
                        bounds: bool = True):
    """The IVIM notebook's initialisation (test_ivim.ipynb cells 6 and 10).

    Degree-1 fits of log S against -b on rows [low[0], low[1]) and
    [high[0], high[1]) give S0, f, D* and D; with ``bounds`` also the per-voxel
    data-driven bounds of the notebook. Returns (pars, lb, ub) as (4, N).
    """
    b = [float(v) for v in bvals]
    N = data.shape[1]
    lo = bpolyfit(data, 1, x_shared=[-v for v in b[low[0]:low[1]]], row0=low[0], rows=low[1] - low[0], log_y=True)
    hi = bpolyfit(data, 1, x_shared=[-v for v in b[high[0]:high[1]]], row0=high[0], rows=high[1] - high[0],
                  log_y=True)
    pars = torch.empty((4, N), dtype=torch.float32, device=data.device)
    lbo = torch.empty_like(pars) if bounds else None
    ubo = torch.empty_like(pars) if bounds else None
    rc = _lib.lib().pcgb_ivim_segmented_init(_p(lo), _p(hi), N, _dvec(lb), _dvec(ub), _p(pars), _p(lbo), _p(ubo),
                                             _stream())
    _lib.check("pcgb_ivim_segmented_init", rc)
    return pars, lbo, ubo
