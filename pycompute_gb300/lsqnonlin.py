"""Drop-in fitter classes with the reference's call surface.

Mirrors ``pycompute/cuda/lsqnonlin.py``: ``Expr``, ``F_GradF``, ``F``,
``SecondOrderLevenbergMarquardt`` (and ``GMW81Solver`` from
``pycompute/cuda/solver.py``), with the same constructor arguments, the same
``setup``/``run`` split, the same array layouts and the same result attributes
(``pars_t`` updated in place, ``f_t``, ``first_f``, ``last_f``,
``step_type_t``, ``lam_t``, ``step_t``).

Arrays are PyTorch CUDA tensors (CuPy arrays and anything else exporting
DLPack are accepted and viewed as tensors without a copy). PyTorch is used for
buffers and the current stream only; all fitting runs in libpcgb.so.

Differences from the reference, all deliberate:
* one launch runs every iteration of ``run`` (the reference launches once per
  iteration); results are the same per voxel;
* the GMW81 solve and gain-ratio test run in float64 for float32 fitters
  (``solve_dtype``); pass ``solve_dtype=torch.float32`` for the reference's
  all-fp32 arithmetic;
* a protocol shared by every voxel may be passed as a (C*M,) or (C*M, 1)
  tensor and bounds as (P,) or (P, 1); it is then held in the kernel's
  parameter bank instead of being read per voxel. A (C*M, N) consts tensor
  whose columns are all equal is detected and treated the same way;
* ``run`` validates its inputs and raises instead of reading out of bounds.
"""
from __future__ import annotations

import ctypes
from typing import Optional

import torch

from . import _lib, codegen

_TORCH_DTYPES = {torch.float32: 0, torch.float64: 1}


def _as_tensor(x, name: str) -> torch.Tensor:
    if isinstance(x, torch.Tensor):
        return x
    if hasattr(x, "__dlpack__"):
        return torch.from_dlpack(x)
    raise TypeError(f"{name} must be a torch tensor or a DLPack-capable array, got {type(x)}")


def _dtype(d) -> torch.dtype:
    if isinstance(d, torch.dtype):
        return d
    s = getattr(d, "name", None) or getattr(d, "__name__", None) or str(d)
    s = str(s).replace("numpy.", "").replace("cupy.", "")
    if s in ("float32", "f", "float"):
        return torch.float32
    if s in ("float64", "d", "double"):
        return torch.float64
    raise RuntimeError(f"does only support fp32 and fp64, got {d}")


def _stream_ptr() -> int:
    return torch.cuda.current_stream().cuda_stream


def _ptr(t: Optional[torch.Tensor]):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


class Expr:
    """Model specification (reference ``Expr``, lsqnonlin.py:21-28)."""

    def __init__(self, expr: str, pars_str: list[str], consts_str: list[str],
                 nonlin_terms: list[str] | None = None, nonlin_pars: list[int] | None = None):
        self.expr = expr
        self.pars_str = list(pars_str)
        self.consts_str = list(consts_str)
        self.nonlin_terms = nonlin_terms
        self.nonlin_pars = nonlin_pars


class F_GradF:
    """User-supplied model code (reference ``F_GradF``, lsqnonlin.py:32-39).

    In the reference ``f`` and ``gradf`` are CudaFunction objects whose device
    code computes the cost and the accumulated derivatives. Here the user
    supplies one model struct in the generated form (see ``codegen``):
    ``source`` defines ``struct <name>`` with ``P``, ``C``, ``H``, ``jnz``,
    ``hnz``, ``value`` and ``all``.
    """

    def __init__(self, source: str, nparam: int, nconst: int, name: str):
        self.source = source
        self.nparam = nparam
        self.nconst = nconst
        self.name = name


def _funcid(prefix: str, P: int, C: int, M: int, dtype: torch.dtype, tag: str) -> str:
    t = "f" if dtype == torch.float32 else "d"
    return f"{prefix}_{P}_{C}_{M}_{t}_{tag}"


class _Program:
    """One compiled fitter program (model x protocol length x precision)."""

    _cache: dict = {}

    def __init__(self, source: str, struct: str, P: int, C: int, M: int, dtype: torch.dtype,
                 solve_dtype: torch.dtype):
        L = _lib.lib()
        h = ctypes.c_void_p()
        dev = torch.cuda.current_device()
        rc = L.pcgb_fitter_create(source.encode(), struct.encode(), P, C, M, _TORCH_DTYPES[dtype],
                                  _TORCH_DTYPES[solve_dtype], _lib.cache_dir().encode(), ctypes.byref(h))
        _lib.check("pcgb_fitter_create", rc)
        self.handle = h
        self.device = dev
        self.P, self.C, self.M, self.dtype, self.solve_dtype = P, C, M, dtype, solve_dtype
        self.log = L.pcgb_fitter_log(h).decode(errors="replace")

    @classmethod
    def get(cls, source, struct, P, C, M, dtype, solve_dtype):
        key = (source, struct, P, C, M, dtype, solve_dtype, torch.cuda.current_device())
        prog = cls._cache.get(key)
        if prog is None:
            prog = cls(source, struct, P, C, M, dtype, solve_dtype)
            cls._cache[key] = prog
        return prog

    def __del__(self):
        try:
            if getattr(self, "handle", None):
                _lib.lib().pcgb_fitter_destroy(self.handle)
        except Exception:
            pass


def _model_from(model_expr, f_gradf, legacy) -> tuple[str, str, int, int, str, Optional[Expr]]:
    if legacy is not None:
        expr, pars_str, consts_str = legacy
        model_expr = Expr(expr, pars_str, consts_str)
    if model_expr is not None and f_gradf is None:
        gm = codegen.generate(model_expr.expr, model_expr.pars_str, model_expr.consts_str)
        return gm.source, gm.struct_name, gm.P, gm.C, gm.hash, model_expr
    if f_gradf is not None and model_expr is None:
        return f_gradf.source, f_gradf.name, f_gradf.nparam, f_gradf.nconst, f_gradf.name, None
    raise RuntimeError("One and only one of model_expr or f_gradf must be non None")


def _shared_rows(t, rows: int, n: int, name: str, detect: bool):
    """Classify a protocol/bounds argument: (device tensor or None, stride, host values).

    A host sequence (list, tuple, numpy array, CPU tensor) of ``rows`` values
    is a shared protocol and costs no device access; a (rows, 1) / (rows,)
    CUDA tensor is shared too (read back once); a (rows, N) CUDA tensor is per
    voxel unless ``detect`` finds all its columns equal.
    """
    if not isinstance(t, torch.Tensor) and not hasattr(t, "__dlpack__"):
        vals = [float(x) for x in (t.reshape(-1) if hasattr(t, "reshape") else t)]
        if len(vals) != rows:
            raise RuntimeError(f"{name} must have {rows} values, got {len(vals)}")
        return None, 0, vals
    t = _as_tensor(t, name)
    if not t.is_cuda:
        vals = t.reshape(-1).double().tolist()
        if len(vals) != rows:
            raise RuntimeError(f"{name} must have {rows} values, got {len(vals)}")
        return None, 0, vals
    if t.dim() == 1:
        t = t.reshape(rows, 1)
    if t.dim() != 2 or t.shape[0] != rows:
        raise RuntimeError(f"{name} must have {rows} rows, got shape {tuple(t.shape)}")
    if t.shape[1] == 1 and n != 1:
        return t, 0, t[:, 0].double().cpu().tolist()
    if t.shape[1] != n:
        raise RuntimeError(f"{name} must have 1 or {n} columns, got {t.shape[1]}")
    if detect and n > 0 and bool((t == t[:, :1]).all()):
        return t, 0, t[:, 0].double().cpu().tolist()
    return t, n, None


def _parse_ctor(args, kwargs, names):
    """Constructor arguments in the reference's two call forms.

    Expression form (lsqnonlin.py:950): ``(model_expr: Expr | None, [f_gradf,] ndata, dtype, write_to_file)``.
    Notebook form (test_ivim.ipynb cell 16): ``(expr: str, pars_str, consts_str, ndata=, dtype=, write_to_file=)``.
    Returns (model_expr, f_gradf, legacy, ndata, dtype, write_to_file).
    """
    args = list(args)
    kw = dict(kwargs)
    legacy = None
    if (args and isinstance(args[0], str)) or isinstance(kw.get("expr"), str):
        expr = args.pop(0) if args else kw.pop("expr")
        pars_str = args.pop(0) if args else kw.pop("pars_str")
        consts_str = args.pop(0) if args else kw.pop("consts_str")
        legacy = (expr, list(pars_str), list(consts_str))
        rest = [n for n in names if n not in ("model_expr", "f_gradf")]
        vals = {"model_expr": None, "f_gradf": None}
    else:
        rest = list(names)
        vals = {}
    for n in rest:
        if args:
            vals[n] = args.pop(0)
        elif n in kw:
            vals[n] = kw.pop(n)
    if args or kw:
        raise TypeError(f"unexpected constructor arguments: {args} {sorted(kw)}")
    return (vals.get("model_expr"), vals.get("f_gradf"), legacy, vals.get("ndata"),
            vals.get("dtype", torch.float32), vals.get("write_to_file", False))


class SecondOrderLevenbergMarquardt:
    """Batched second-order LM with GMW81 damped solves, one voxel per thread.

    Same surface as the reference class (lsqnonlin.py:949-1073)::

        solm = SecondOrderLevenbergMarquardt(Expr(expr, pars, consts), None, ndata, torch.float32)
        solm = SecondOrderLevenbergMarquardt(expr, pars, consts, ndata=21, dtype=torch.float32)  # notebook form
        solm.setup(pars_t, consts_t, data_t, lower_bound_t, upper_bound_t)
        solm.run(50, 1e-10)
        solm.pars_t, solm.first_f, solm.last_f, solm.step_type_t
    """

    def __init__(self, *args, solve_dtype=None, detect_shared: bool = True, **kwargs):
        model_expr, f_gradf, legacy, ndata, dtype, write_to_file = _parse_ctor(
            args, kwargs, ("model_expr", "f_gradf", "ndata", "dtype", "write_to_file"))
        if ndata is None or int(ndata) < 1:
            raise RuntimeError("ndata must be a positive integer")
        self.dtype = _dtype(dtype)
        self.solve_dtype = _dtype(solve_dtype) if solve_dtype is not None else torch.float64
        if self.dtype == torch.float64 and self.solve_dtype == torch.float32:
            raise RuntimeError("a float64 fitter solves in float64")
        src, struct, P, C, tag, mexpr = _model_from(model_expr, f_gradf, legacy)
        self.model_expr = mexpr
        self.expr = mexpr.expr if mexpr else None
        self.pars_str = list(mexpr.pars_str) if mexpr else None
        self.consts_str = list(mexpr.consts_str) if mexpr else None
        self.nparam, self.nconst, self.ndata = P, C, int(ndata)
        self.nhes = P * (P + 1) // 2
        self.write_to_file = write_to_file
        self.detect_shared = detect_shared
        self.funcid = _funcid("second_order_levenberg_marquardt", P, C, self.ndata, self.dtype, tag)
        self._source, self._struct = src, struct
        if write_to_file:
            with open(self.funcid + ".cu", "w") as f:
                f.write(src)
        self._prog = None
        self.Nprobs = 1

    def build(self):
        """Compile (NVRTC, sm_103a) and load the program on the current device."""
        if self._prog is None or self._prog.device != torch.cuda.current_device():
            self._prog = _Program.get(self._source, self._struct, self.nparam, self.nconst, self.ndata,
                                      self.dtype, self.solve_dtype)
        return self._prog

    def get_device_funcid(self):
        return self.funcid

    def get_kernel_funcid(self):
        return "k_" + self.funcid

    def setup(self, pars_t, consts_t, data_t, lower_bound_t, upper_bound_t, init_state: bool = True):
        """Bind caller-owned arrays and allocate the fitter state (lsqnonlin.py:1036-1056).

        ``init_state=False`` (no reference counterpart) allocates the damping,
        step-code and cost arrays without initialising them and keeps no step
        or iteration-count arrays: for callers whose next call is run_fresh(),
        which reads none of that state (the warm-start pipeline)."""
        pars_t = _as_tensor(pars_t, "pars_t")
        data_t = _as_tensor(data_t, "data_t")
        P, M, C = self.nparam, self.ndata, self.nconst
        if data_t.dim() != 2 or data_t.shape[0] != M:
            raise RuntimeError(f"data_t must be ({M}, N), got {tuple(data_t.shape)}")
        N = int(data_t.shape[1])
        for name, t in (("pars_t", pars_t), ("data_t", data_t), ("consts_t", consts_t),
                        ("lower_bound_t", lower_bound_t), ("upper_bound_t", upper_bound_t)):
            if not isinstance(t, torch.Tensor) or (name not in ("pars_t", "data_t") and not t.is_cuda):
                continue  # host protocol / bounds values
            if not t.is_cuda:
                raise RuntimeError(f"{name} must be a CUDA tensor")
            if t.dtype != self.dtype:
                raise RuntimeError(f"{name} must be {self.dtype}, got {t.dtype}")
            if not t.is_contiguous():
                raise RuntimeError(f"{name} must be C-contiguous")
        if tuple(pars_t.shape) != (P, N):
            raise RuntimeError(f"pars_t must be ({P}, {N}), got {tuple(pars_t.shape)}")
        self.Nprobs = N
        self.pars_t = pars_t
        self.data_t = data_t
        self.consts_t, self._cstride, self._protocol = _shared_rows(consts_t, C * M, N, "consts_t",
                                                                      self.detect_shared)
        self.lower_bound_t, bs_l, lbv = _shared_rows(lower_bound_t, P, N, "lower_bound_t", self.detect_shared)
        self.upper_bound_t, bs_u, ubv = _shared_rows(upper_bound_t, P, N, "upper_bound_t", self.detect_shared)
        if bs_l != bs_u:
            dev = pars_t.device

            def per_voxel(vals, t):
                if vals is not None:
                    return torch.tensor(vals, dtype=self.dtype, device=dev)[:, None].expand(P, N).contiguous()
                return t
            lt = per_voxel(lbv, self.lower_bound_t)
            ut = per_voxel(ubv, self.upper_bound_t)
            self.lower_bound_t, bs_l, lbv = lt, N, None
            self.upper_bound_t, bs_u, ubv = ut, N, None
        self._bstride = bs_l
        self._lb_host, self._ub_host = lbv, ubv
        dev = pars_t.device
        self.first_f = torch.empty((1, N), dtype=self.dtype, device=dev)
        self.last_f = torch.empty((1, N), dtype=self.dtype, device=dev)
        if init_state:
            self.lam_t = torch.full((1, N), 5.0, dtype=self.dtype, device=dev)
            self.step_t = torch.zeros((P, N), dtype=self.dtype, device=dev)
            self.f_t = torch.zeros((1, N), dtype=self.dtype, device=dev)
            self.step_type_t = torch.ones((1, N), dtype=torch.int8, device=dev)
            self.iters_t = torch.zeros((1, N), dtype=torch.int32, device=dev)
        else:
            self.lam_t = torch.empty((1, N), dtype=self.dtype, device=dev)
            self.f_t = torch.empty((1, N), dtype=self.dtype, device=dev)
            self.step_type_t = torch.empty((1, N), dtype=torch.int8, device=dev)
            self.step_t = None
            self.iters_t = None
        with torch.cuda.device(dev):
            self.build()

    def run(self, iters: int, tol=1e-8, mu=0.25, eta=0.75, acc=0.2, dec=2.0, block: int = 0,
            schedule: str = "grid"):
        """Run ``iters`` iterations on every voxel (lsqnonlin.py:1058-1073). Asynchronous; returns None.

        ``schedule="grid"`` gives each thread one voxel for the whole fit;
        ``schedule="refill"`` runs a persistent grid whose warps hand a new
        voxel to any lane whose voxel has converged (same results, fewer idle
        lanes when convergence is ragged).
        """
        if not hasattr(self, "pars_t"):
            raise RuntimeError("setup() must be called before run()")
        if schedule == "refill":
            return self._run_refill(iters, tol, mu, eta, acc, dec, block, None, 0)
        if schedule != "grid":
            raise ValueError("schedule must be 'grid' or 'refill'")
        with torch.cuda.device(self.pars_t.device):
            prog = self.build()
            L = _lib.lib()
            proto = (ctypes.c_double * max(1, len(self._protocol or [])))(*(self._protocol or [0.0]))
            lbh = (ctypes.c_double * self.nparam)(*(self._lb_host or [0.0] * self.nparam))
            ubh = (ctypes.c_double * self.nparam)(*(self._ub_host or [0.0] * self.nparam))
            rc = L.pcgb_lm_run(prog.handle, _ptr(self.consts_t), self._cstride, _ptr(self.data_t),
                               _ptr(self.lower_bound_t), _ptr(self.upper_bound_t), self._bstride,
                               float(tol), float(mu), float(eta), float(acc), float(dec),
                               _ptr(self.pars_t), _ptr(self.step_t), _ptr(self.lam_t), _ptr(self.step_type_t),
                               _ptr(self.f_t), _ptr(self.first_f), _ptr(self.last_f), _ptr(self.iters_t),
                               self.Nprobs, int(iters), proto if self._cstride == 0 else None,
                               len(self._protocol or []), lbh if self._bstride == 0 else None,
                               ubh if self._bstride == 0 else None, int(block), ctypes.c_void_p(_stream_ptr()))
            _lib.check("pcgb_lm_run", rc)
        return None

    def _lm_args(self, iters, tol, mu, eta, acc, dec, block):
        """The arguments every LM entry point starts with (pcgb_lm_run's, up to block)."""
        pv, plen = self._proto_args()
        lbh = (ctypes.c_double * self.nparam)(*(self._lb_host or [0.0] * self.nparam))
        ubh = (ctypes.c_double * self.nparam)(*(self._ub_host or [0.0] * self.nparam))
        return (self.build().handle, _ptr(self.consts_t), self._cstride, _ptr(self.data_t), _ptr(self.lower_bound_t),
                _ptr(self.upper_bound_t), self._bstride, float(tol), float(mu), float(eta), float(acc), float(dec),
                _ptr(self.pars_t), _ptr(self.step_t), _ptr(self.lam_t), _ptr(self.step_type_t), _ptr(self.f_t),
                _ptr(self.first_f), _ptr(self.last_f), _ptr(self.iters_t), self.Nprobs, int(iters), pv, plen,
                lbh if self._bstride == 0 else None, ubh if self._bstride == 0 else None, int(block))

    def run_fresh(self, iters: int, lam0: float, tol=1e-8, mu=0.25, eta=0.75, acc=0.2, dec=2.0, block: int = 0):
        """``iters`` iterations from a fresh start at damping ``lam0`` and
        step code 1 on every voxel, keeping only the parameters and step codes
        (pcgb_lm_run_fresh; no reference counterpart): the damping, cost and
        step arrays are neither read nor written."""
        with torch.cuda.device(self.pars_t.device):
            pv, plen = self._proto_args()
            lbh = (ctypes.c_double * self.nparam)(*(self._lb_host or [0.0] * self.nparam))
            ubh = (ctypes.c_double * self.nparam)(*(self._ub_host or [0.0] * self.nparam))
            rc = _lib.lib().pcgb_lm_run_fresh(
                self.build().handle, _ptr(self.consts_t), self._cstride, _ptr(self.data_t), _ptr(self.lower_bound_t),
                _ptr(self.upper_bound_t), self._bstride, float(tol), float(mu), float(eta), float(acc), float(dec),
                _ptr(self.pars_t), _ptr(self.step_type_t), self.Nprobs, int(iters), pv, plen,
                lbh if self._bstride == 0 else None, ubh if self._bstride == 0 else None, float(lam0), int(block),
                ctypes.c_void_p(_stream_ptr()))
            _lib.check("pcgb_lm_run_fresh", rc)

    def run_check(self, iters: int, init_values, lam_refit: float, cost, pars_backup, cost_backup, fb_idx, fb_count,
                  tol=1e-8, mu=0.25, eta=0.75, acc=0.2, dec=2.0, block: int = 0):
        """run() with the warm-start fallback check as its epilogue (pcgb_lm_run_check)."""
        with torch.cuda.device(self.pars_t.device):
            iv = (ctypes.c_double * self.nparam)(*[float(x) for x in init_values])
            rc = _lib.lib().pcgb_lm_run_check(*self._lm_args(iters, tol, mu, eta, acc, dec, block), iv,
                                               float(lam_refit), _ptr(cost), _ptr(pars_backup), _ptr(cost_backup),
                                               _ptr(fb_idx), _ptr(fb_count), ctypes.c_void_p(_stream_ptr()))
            _lib.check("pcgb_lm_run_check", rc)

    def run_select(self, iters: int, cost, pars_backup, cost_backup, fb_idx, fb_count, which=None, tol=1e-8,
                   mu=0.25, eta=0.75, acc=0.2, dec=2.0, block: int = 0):
        """Refit of the flagged voxels with the select as its epilogue (pcgb_lm_run_select)."""
        with torch.cuda.device(self.pars_t.device):
            rc = _lib.lib().pcgb_lm_run_select(*self._lm_args(iters, tol, mu, eta, acc, dec, block), _ptr(cost),
                                                _ptr(pars_backup), _ptr(cost_backup), _ptr(fb_idx), _ptr(fb_count),
                                                _ptr(which), ctypes.c_void_p(_stream_ptr()))
            _lib.check("pcgb_lm_run_select", rc)

    def _run_refill(self, iters, tol, mu, eta, acc, dec, block, vox_idx, n_items, grid: int = 0, n_items_dev=None):
        with torch.cuda.device(self.pars_t.device):
            prog = self.build()
            if getattr(self, "_counter", None) is None or self._counter.device != self.pars_t.device:
                self._counter = torch.zeros(1, dtype=torch.int32, device=self.pars_t.device)
            pv, plen = self._proto_args()
            lbh = (ctypes.c_double * self.nparam)(*(self._lb_host or [0.0] * self.nparam))
            ubh = (ctypes.c_double * self.nparam)(*(self._ub_host or [0.0] * self.nparam))
            rc = _lib.lib().pcgb_lm_run_refill(
                prog.handle, _ptr(self.consts_t), self._cstride, _ptr(self.data_t), _ptr(self.lower_bound_t),
                _ptr(self.upper_bound_t), self._bstride, float(tol), float(mu), float(eta), float(acc), float(dec),
                _ptr(self.pars_t), _ptr(self.step_t), _ptr(self.lam_t), _ptr(self.step_type_t), _ptr(self.f_t),
                _ptr(self.first_f), _ptr(self.last_f), _ptr(self.iters_t), self.Nprobs, int(iters), pv, plen,
                lbh if self._bstride == 0 else None, ubh if self._bstride == 0 else None, int(block),
                _ptr(vox_idx) if vox_idx is not None else None, int(n_items), _ptr(n_items_dev),
                _ptr(self._counter), int(grid), ctypes.c_void_p(_stream_ptr()))
            _lib.check("pcgb_lm_run_refill", rc)
        return None


    # ---- extensions used by the fit pipeline (no reference counterpart) -------
    def _proto_args(self):
        proto = (ctypes.c_double * max(1, len(self._protocol or [])))(*(self._protocol or [0.0]))
        return proto if self._cstride == 0 else None, len(self._protocol or [])

    def cost(self, pars_t=None, out=None, vox_idx=None, n_items=None) -> torch.Tensor:
        """Cost sum_i (m(p) - d_i)^2 at ``pars_t`` (default: the current fit), (N,) fp."""
        pars_t = self.pars_t if pars_t is None else pars_t
        out = torch.zeros(self.Nprobs, dtype=self.dtype, device=pars_t.device) if out is None else out
        with torch.cuda.device(pars_t.device):
            prog = self.build()
            pv, plen = self._proto_args()
            if vox_idx is None:
                rc = _lib.lib().pcgb_f_run(prog.handle, _ptr(pars_t), _ptr(self.consts_t), self._cstride,
                                           _ptr(self.data_t), None, _ptr(out), self.Nprobs, pv, plen,
                                           ctypes.c_void_p(_stream_ptr()))
                _lib.check("pcgb_f_run", rc)
            else:
                rc = _lib.lib().pcgb_f_run_subset(prog.handle, _ptr(pars_t), _ptr(self.consts_t), self._cstride,
                                                  _ptr(self.data_t), None, _ptr(out), self.Nprobs, pv, plen,
                                                  _ptr(vox_idx), int(n_items), ctypes.c_void_p(_stream_ptr()))
                _lib.check("pcgb_f_run_subset", rc)
        return out

    def run_subset(self, vox_idx: torch.Tensor, n_items: int, iters: int, tol=1e-8, mu=0.25, eta=0.75, acc=0.2,
                   dec=2.0, block: int = 0, schedule: str = "grid", n_items_dev: torch.Tensor | None = None):
        """run() restricted to the voxels listed in ``vox_idx`` (int32, first n_items entries).

        ``n_items_dev``: optional device int32 holding the list length; then
        min(n_items_dev[0], n_items) entries are fitted without a host read.
        """
        if schedule == "refill":
            return self._run_refill(iters, tol, mu, eta, acc, dec, block, vox_idx, n_items, n_items_dev=n_items_dev)
        if schedule != "grid":
            raise ValueError("schedule must be 'grid' or 'refill'")
        with torch.cuda.device(self.pars_t.device):
            prog = self.build()
            pv, plen = self._proto_args()
            lbh = (ctypes.c_double * self.nparam)(*(self._lb_host or [0.0] * self.nparam))
            ubh = (ctypes.c_double * self.nparam)(*(self._ub_host or [0.0] * self.nparam))
            rc = _lib.lib().pcgb_lm_run_subset(
                prog.handle, _ptr(self.consts_t), self._cstride, _ptr(self.data_t), _ptr(self.lower_bound_t),
                _ptr(self.upper_bound_t), self._bstride, float(tol), float(mu), float(eta), float(acc), float(dec),
                _ptr(self.pars_t), _ptr(self.step_t), _ptr(self.lam_t), _ptr(self.step_type_t), _ptr(self.f_t),
                _ptr(self.first_f), _ptr(self.last_f), _ptr(self.iters_t), self.Nprobs, int(iters), pv, plen,
                lbh if self._bstride == 0 else None, ubh if self._bstride == 0 else None, int(block),
                _ptr(vox_idx), int(n_items), _ptr(n_items_dev), ctypes.c_void_p(_stream_ptr()))
            _lib.check("pcgb_lm_run_subset", rc)

    def model_eval(self, pars_t: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
        """Model values m(p_v; c_i), (M, N), with the protocol given to setup()."""
        N = int(pars_t.shape[1])
        out = torch.empty((self.ndata, N), dtype=self.dtype, device=pars_t.device) if out is None else out
        with torch.cuda.device(pars_t.device):
            prog = self.build()
            pv, plen = self._proto_args()
            rc = _lib.lib().pcgb_model_eval(prog.handle, _ptr(pars_t), _ptr(self.consts_t), self._cstride,
                                            _ptr(out), N, pv, plen, ctypes.c_void_p(_stream_ptr()))
            _lib.check("pcgb_model_eval", rc)
        return out


class F:
    """Accumulating objective f += sum_i (m - d_i)^2 (reference ``F``, lsqnonlin.py:119-199)."""

    def __init__(self, *args, **kwargs):
        model_expr, _unused, legacy, ndata, dtype, write_to_file = _parse_ctor(
            args, kwargs, ("model_expr", "ndata", "dtype", "write_to_file"))
        self.dtype = _dtype(dtype)
        src, struct, P, C, tag, mexpr = _model_from(model_expr, None, legacy)
        self.nparam, self.nconst, self.ndata = P, C, int(ndata)
        self.funcid = _funcid("f", P, C, self.ndata, self.dtype, tag)
        self._source, self._struct = src, struct
        self._prog = None

    def build(self):
        if self._prog is None or self._prog.device != torch.cuda.current_device():
            self._prog = _Program.get(self._source, self._struct, self.nparam, self.nconst, self.ndata, self.dtype,
                                      self.dtype)
        return self._prog

    def run(self, pars, consts, data, step_type, f):
        pars, consts, data, f = (_as_tensor(x, n) for x, n in ((pars, "pars"), (consts, "consts"),
                                                              (data, "data"), (f, "f")))
        N = int(pars.shape[1])
        if tuple(data.shape) != (self.ndata, N) or f.numel() != N:
            raise RuntimeError("shape mismatch between pars, data and f")
        st = None
        if step_type is not None:
            st = _as_tensor(step_type, "step_type")
            if st.dtype != torch.int8 or st.numel() != N:
                st = None if st.numel() != N else st.to(torch.int8)
        consts, cstride, proto = _shared_rows(consts, self.nconst * self.ndata, N, "consts", True)
        with torch.cuda.device(pars.device):
            prog = self.build()
            pv = (ctypes.c_double * max(1, len(proto or [])))(*(proto or [0.0]))
            rc = _lib.lib().pcgb_f_run(prog.handle, _ptr(pars), _ptr(consts), cstride, _ptr(data), _ptr(st), _ptr(f),
                                       N, pv if cstride == 0 else None, len(proto or []),
                                       ctypes.c_void_p(_stream_ptr()))
            _lib.check("pcgb_f_run", rc)


class GMW81Solver:
    """Batched GMW81 modified-Cholesky solver (reference ``GMW81Solver``, solver.py:490-595)."""

    def __init__(self, ndim: int, dtype=torch.float32, write_to_file: bool = False):
        self.ndim = int(ndim)
        self.dtype = _dtype(dtype)
        names = [f"x{k}" for k in range(self.ndim)]
        gm = codegen.generate("+".join(names), names, [], struct_name=f"GmwShape{self.ndim}")
        self._source, self._struct = gm.source, gm.struct_name
        self._prog = None

    def run(self, mat, rhs, step_type=None, sol=None):
        mat, rhs, sol = _as_tensor(mat, "mat"), _as_tensor(rhs, "rhs"), _as_tensor(sol, "sol")
        n, N = int(rhs.shape[0]), int(rhs.shape[1])
        if n != self.ndim or tuple(mat.shape) != (n * (n + 1) // 2, N) or tuple(sol.shape) != (n, N):
            raise RuntimeError("mat must be (ndim*(ndim+1)/2, N), rhs and sol (ndim, N)")
        for t in (mat, rhs, sol):
            if t.dtype != self.dtype or not t.is_contiguous() or not t.is_cuda:
                raise RuntimeError("mat, rhs, sol must be contiguous CUDA tensors of the solver dtype")
        with torch.cuda.device(mat.device):
            if self._prog is None or self._prog.device != torch.cuda.current_device():
                self._prog = _Program.get(self._source, self._struct, self.ndim, 0, 1, self.dtype, self.dtype)
            rc = _lib.lib().pcgb_gmw81_solve(self._prog.handle, _ptr(mat), _ptr(rhs), _ptr(sol), N,
                                             ctypes.c_void_p(_stream_ptr()))
            _lib.check("pcgb_gmw81_solve", rc)


class SearchStep:
    """One cost-and-keep-best step (reference ``SearchStep``, lsqnonlin.py:1120-1199).

    ``run(f, best_f, p, best_p)``: f += cost(p) (the reference's cost function
    accumulates into f), then p replaces best_p where f < best_f.
    """

    def __init__(self, *args, **kwargs):
        model_expr, _unused, legacy, ndata, dtype, write_to_file = _parse_ctor(
            args, kwargs, ("model_expr", "ndata", "dtype", "write_to_file"))
        if legacy is not None:
            self._lm = SecondOrderLevenbergMarquardt(legacy[0], legacy[1], legacy[2], ndata=ndata, dtype=dtype)
        else:
            self._lm = SecondOrderLevenbergMarquardt(model_expr, None, ndata, dtype)
        self.nparam, self.ndata, self.dtype = self._lm.nparam, self._lm.ndata, self._lm.dtype

    def setup(self, consts_t, data_t, lower_bound_t, upper_bound_t):
        N = int(_as_tensor(data_t, "data_t").shape[1])
        dummy = torch.empty((self.nparam, N), dtype=self.dtype, device=_as_tensor(data_t, "data_t").device)
        self._lm.setup(dummy, consts_t, data_t, lower_bound_t, upper_bound_t)
        self.Nprobs = N

    def run(self, f, best_f, p, best_p):
        lm = self._lm
        with torch.cuda.device(lm.data_t.device):
            prog = lm.build()
            pv, plen = lm._proto_args()
            rc = _lib.lib().pcgb_search_step(prog.handle, _ptr(lm.consts_t), lm._cstride, _ptr(lm.data_t), _ptr(p),
                                             _ptr(f), _ptr(best_p), _ptr(best_f), self.Nprobs, pv, plen,
                                             ctypes.c_void_p(_stream_ptr()))
            _lib.check("pcgb_search_step", rc)


class RandomSearch:
    """Random search (reference ``RandomSearch``, lsqnonlin.py:1202-1242).

    ``setup(consts, data, lb, ub)`` then ``run(iters)``: ``iters`` draws per
    voxel uniform in [lb, ub], best point in ``best_pars_t`` / ``best_f_t``.
    All draws run in one launch with a counter-based generator (``seed``);
    each draw is compared by its own cost. (In the reference the cost buffer
    accumulates across draws, lsqnonlin.py:1230-1242 with the accumulating
    cost function, so in practice only its first draw is kept.) best_pars_t
    starts at the lower bounds instead of uninitialised memory.
    """

    lm_iters = 0

    def __init__(self, *args, solve_dtype=None, **kwargs):
        model_expr, _unused, legacy, ndata, dtype, write_to_file = _parse_ctor(
            args, kwargs, ("model_expr", "ndata", "dtype", "write_to_file"))
        if legacy is not None:
            self._lm = SecondOrderLevenbergMarquardt(legacy[0], legacy[1], legacy[2], ndata=ndata, dtype=dtype,
                                                     solve_dtype=solve_dtype)
        else:
            self._lm = SecondOrderLevenbergMarquardt(model_expr, None, ndata, dtype, solve_dtype=solve_dtype)
        self.nparam, self.ndata, self.dtype = self._lm.nparam, self._lm.ndata, self._lm.dtype
        self._seed = 0x5EED5EED

    def setup(self, consts_t, data_t, lower_bound_t, upper_bound_t):
        data_t = _as_tensor(data_t, "data_t")
        N = int(data_t.shape[1])
        self.Nprobs = N
        lm = self._lm
        lm.setup(torch.empty((self.nparam, N), dtype=self.dtype, device=data_t.device), consts_t, data_t,
                 lower_bound_t, upper_bound_t)
        if lm._bstride == 0:
            lbv = torch.tensor(lm._lb_host, dtype=self.dtype, device=data_t.device)
            self.best_pars_t = lbv[:, None].expand(self.nparam, N).contiguous()
        else:
            self.best_pars_t = lm.lower_bound_t.clone()
        self.best_f_t = torch.full((1, N), torch.finfo(self.dtype).max / 5, dtype=self.dtype, device=data_t.device)

    def run(self, iters: int, lm_iters: int | None = None, tol=1e-8, mu=0.25, eta=0.75, acc=0.2, dec=2.0,
            seed: int | None = None):
        lm = self._lm
        lm_iters = self.lm_iters if lm_iters is None else int(lm_iters)
        if seed is None:
            self._seed = (self._seed + 0x9E3779B97F4A7C15) & 0xFFFFFFFFFFFFFFFF
            seed = self._seed
        with torch.cuda.device(lm.data_t.device):
            prog = lm.build()
            pv, plen = lm._proto_args()
            lbh = (ctypes.c_double * self.nparam)(*(lm._lb_host or [0.0] * self.nparam))
            ubh = (ctypes.c_double * self.nparam)(*(lm._ub_host or [0.0] * self.nparam))
            rc = _lib.lib().pcgb_random_search(
                prog.handle, _ptr(lm.consts_t), lm._cstride, _ptr(lm.data_t), _ptr(lm.lower_bound_t),
                _ptr(lm.upper_bound_t), lm._bstride, _ptr(self.best_pars_t), _ptr(self.best_f_t), self.Nprobs,
                int(iters), lm_iters, float(tol), float(mu), float(eta), float(acc), float(dec),
                ctypes.c_uint64(int(seed)), pv, plen, lbh if lm._bstride == 0 else None,
                ubh if lm._bstride == 0 else None, ctypes.c_void_p(_stream_ptr()))
            _lib.check("pcgb_random_search", rc)


class SecondOrderRandomSearch(RandomSearch):
    """Multi-start LM (reference ``SecondOrderRandomSearch``, lsqnonlin.py:1245-1291).

    ``run(iters, lm_iters=20, tol=1e-8)``: every draw is refined by lm_iters LM
    iterations from lambda = 5 before its cost is compared, all in one launch.
    """

    def run(self, iters: int, lm_iters: int = 20, tol=1e-8, seed: int | None = None, **kw):
        return super().run(iters, lm_iters=lm_iters, tol=tol, seed=seed, **kw)
