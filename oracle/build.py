"""Build and load the CPU oracle (TEST INFRASTRUCTURE ONLY).

``OracleModel(expr, pars, consts)`` generates the model code with the package
codegen, compiles ``oracle_api.cpp`` against it with g++ (OpenMP,
``-ffp-contract=off`` so x86 and Arm hosts round alike) and wraps the C entry
points with numpy arrays. Builds are cached under ``oracle/_build/<key>/``.
"""
from __future__ import annotations

import ctypes
import hashlib
import os
import platform
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF_DIR = os.path.join(HERE, "_ref")
_lock = threading.Lock()

_CXXFLAGS = ["-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-w"]


def _codegen():
    from pycompute_gb300 import codegen

    return codegen


def _flags(contract: bool) -> list[str]:
    if not contract:
        return list(_CXXFLAGS)
    # same code with fused multiply-adds, as the GPU compiler contracts them:
    # a second legitimate rounding of the same algorithm (noise-floor twin)
    f = [x for x in _CXXFLAGS if x != "-ffp-contract=off"] + ["-ffp-contract=fast"]
    if platform.machine() in ("x86_64", "AMD64"):
        f.append("-mfma")
    return f


def _compile_model(gm, contract: bool = False) -> str:
    with open(os.path.join(HERE, "lm_oracle.hpp")) as f:
        hdr = f.read()
    with open(os.path.join(HERE, "oracle_api.cpp")) as f:
        api = f.read()
    flags = _flags(contract)
    key = hashlib.sha1((hdr + api + gm.source + " ".join(flags)).encode()).hexdigest()[:16]
    d = os.path.join(BUILD, key)
    so = os.path.join(d, "liboracle.so")
    with _lock:
        if os.path.exists(so):
            return so
        os.makedirs(d, exist_ok=True)
        mh = os.path.join(d, "model.h")
        with open(mh, "w") as f:
            f.write(gm.source)
        tmp = so + f".tmp{os.getpid()}"
        cmd = ["g++", *flags, f"-I{HERE}", f"-I{d}", f'-DPCGB_MODEL_FILE="model.h"',
               f"-DPCGB_MODEL_STRUCT={gm.struct_name}", os.path.join(HERE, "oracle_api.cpp"), "-o", tmp]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"oracle build failed:\n{' '.join(cmd)}\n{r.stderr}")
        os.replace(tmp, so)
    return so


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


MODES = {("float32", "float32"): 0, ("float32", "float64"): 1, ("float64", "float64"): 2}


class OracleModel:
    """CPU restatement of the reference LM for one model expression.

    ``contract=True`` builds the same code with fused multiply-adds: a second
    legitimate rounding of the algorithm, used to measure the noise floor that
    two correct implementations show against each other.
    """

    def __init__(self, expr: str, pars: list[str], consts: list[str], contract: bool = False):
        cg = _codegen()
        self.gm = cg.generate(expr, pars, consts)
        self.P, self.C, self.H = self.gm.P, self.gm.C, self.gm.H
        self.lib = ctypes.CDLL(_compile_model(self.gm, contract))
        L = self.lib
        L.oracle_lm_run.restype = ctypes.c_int
        L.oracle_lm_run.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_long, ctypes.c_long, ctypes.c_long] + \
            [ctypes.c_void_p] * 12 + [ctypes.c_int] + [ctypes.c_double] * 5
        L.oracle_cost.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_long, ctypes.c_long] + [ctypes.c_void_p] * 4
        L.oracle_gmw81_solve.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_long] + [ctypes.c_void_p] * 3
        L.oracle_set_threads.argtypes = [ctypes.c_int]
        L.oracle_search_step.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_long, ctypes.c_long] + [ctypes.c_void_p] * 6
        L.oracle_random_search.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_long, ctypes.c_long, ctypes.c_long] + \
            [ctypes.c_void_p] * 6 + [ctypes.c_int, ctypes.c_int, ctypes.c_ulonglong] + [ctypes.c_double] * 5

    def set_threads(self, n: int) -> int:
        return self.lib.oracle_set_threads(int(n))

    def lm_run(self, pars, consts, data, lb, ub, iters, tol=1e-8, mu=0.25, eta=0.75, acc=0.2, dec=2.0,
               lam=None, step_type=None, f=None, solve_dtype=None, want_step=False):
        """Run ``iters`` LM iterations on every voxel, like setup() + run().

        ``pars`` (P, N) is updated in place. ``consts`` is (C*M, N) per voxel or
        (C*M,) shared; ``lb``/``ub`` are (P, N) or (P,) shared. Returns a dict
        with pars, lam, step_type, f, first_f, last_f, iters (per voxel count)
        and optionally step.
        """
        dt = pars.dtype
        assert dt in (np.float32, np.float64)
        sdt = np.dtype(solve_dtype) if solve_dtype is not None else dt
        mode = MODES[(np.dtype(dt).name, sdt.name)]
        P, N = pars.shape
        assert P == self.P and pars.flags.c_contiguous
        M = data.shape[0]
        cstride = N if consts.ndim == 2 and consts.shape[1] == N and N != 1 else 0
        if consts.ndim == 2 and consts.shape[1] == 1:
            consts = consts[:, 0]
        bstride = N if lb.ndim == 2 and lb.shape[1] == N and N != 1 else 0
        if lb.ndim == 2 and lb.shape[1] == 1:
            lb, ub = lb[:, 0], ub[:, 0]
        consts = np.ascontiguousarray(consts, dtype=dt)
        data = np.ascontiguousarray(data, dtype=dt)
        lb = np.ascontiguousarray(lb, dtype=dt)
        ub = np.ascontiguousarray(ub, dtype=dt)
        lam = np.full(N, 5.0, dtype=dt) if lam is None else lam
        step_type = np.ones(N, dtype=np.int8) if step_type is None else step_type
        f = np.zeros(N, dtype=dt) if f is None else f
        first_f = np.zeros(N, dtype=dt)
        last_f = np.zeros(N, dtype=dt)
        nit = np.zeros(N, dtype=np.int32)
        step = np.zeros((P, N), dtype=dt) if want_step else None
        rc = self.lib.oracle_lm_run(mode, M, N, cstride, bstride, _p(pars), _p(consts), _p(data), _p(lb), _p(ub),
                                    _p(lam), _p(step_type), _p(f), _p(first_f), _p(last_f), _p(step), _p(nit),
                                    int(iters), tol, mu, eta, acc, dec)
        if rc != 0:
            raise RuntimeError(f"oracle_lm_run failed: {rc}")
        out = dict(pars=pars, lam=lam, step_type=step_type, f=f, first_f=first_f, last_f=last_f, iters=nit)
        if want_step:
            out["step"] = step
        return out

    def cost(self, pars, consts, data, f=None):
        """f += sum_i (m - d_i)^2 (the reference F accumulates into f)."""
        dt = pars.dtype
        P, N = pars.shape
        M = data.shape[0]
        cstride = N if consts.ndim == 2 and consts.shape[1] == N and N != 1 else 0
        consts = np.ascontiguousarray(consts.reshape(-1) if cstride == 0 else consts, dtype=dt)
        f = np.zeros(N, dtype=dt) if f is None else f
        rc = self.lib.oracle_cost(int(dt == np.float64), M, N, cstride, _p(np.ascontiguousarray(pars)), _p(consts),
                                  _p(np.ascontiguousarray(data, dtype=dt)), _p(f))
        if rc != 0:
            raise RuntimeError(f"oracle_cost failed: {rc}")
        return f

    def search_step(self, consts, data, p, f, best_p, best_f):
        """SearchStep.run: f += cost(p); best_p / best_f updated in place."""
        dt = p.dtype
        P, N = p.shape
        M = data.shape[0]
        cstride = N if consts.ndim == 2 and consts.shape[1] == N and N != 1 else 0
        consts = np.ascontiguousarray(consts.reshape(-1) if cstride == 0 else consts, dtype=dt)
        rc = self.lib.oracle_search_step(int(dt == np.float64), M, N, cstride, _p(consts),
                                         _p(np.ascontiguousarray(data, dtype=dt)), _p(np.ascontiguousarray(p)), _p(f),
                                         _p(best_p), _p(best_f))
        if rc != 0:
            raise RuntimeError(f"oracle_search_step failed: {rc}")

    def random_search(self, consts, data, lb, ub, best_p, best_f, draws, lm_iters=0, seed=0, tol=1e-8, mu=0.25,
                      eta=0.75, acc=0.2, dec=2.0, solve_dtype=None):
        """Random search (lm_iters = 0) or second-order random search; best_p / best_f in place."""
        dt = best_p.dtype
        sdt = np.dtype(solve_dtype) if solve_dtype is not None else dt
        mode = MODES[(np.dtype(dt).name, sdt.name)]
        P, N = best_p.shape
        M = data.shape[0]
        cstride = N if consts.ndim == 2 and consts.shape[1] == N and N != 1 else 0
        consts = np.ascontiguousarray(consts.reshape(-1) if cstride == 0 else consts, dtype=dt)
        bstride = N if lb.ndim == 2 and lb.shape[1] == N and N != 1 else 0
        lb = np.ascontiguousarray(lb.reshape(-1) if bstride == 0 else lb, dtype=dt)
        ub = np.ascontiguousarray(ub.reshape(-1) if bstride == 0 else ub, dtype=dt)
        rc = self.lib.oracle_random_search(mode, M, N, cstride, bstride, _p(consts),
                                           _p(np.ascontiguousarray(data, dtype=dt)), _p(lb), _p(ub), _p(best_p),
                                           _p(best_f), int(draws), int(lm_iters), int(seed), tol, mu, eta, acc, dec)
        if rc != 0:
            raise RuntimeError(f"oracle_random_search failed: {rc}")

    def gmw81_solve(self, mat_packed, rhs):
        n, N = rhs.shape
        sol = np.zeros_like(rhs)
        rc = self.lib.oracle_gmw81_solve(int(rhs.dtype == np.float64), n, N, _p(np.ascontiguousarray(mat_packed)),
                                         _p(np.ascontiguousarray(rhs)), _p(sol))
        if rc != 0:
            raise RuntimeError(f"oracle_gmw81_solve failed: {rc}")
        return sol


def ref_available(ndata: int = 21) -> bool:
    return os.path.exists(os.path.join(REF_DIR, f"libref_ivim{ndata}.so"))


def build_reference(ref_root: str) -> bool:
    """Build oracle/_ref from the reference tree at ref_root when it is present."""
    if not os.path.isdir(ref_root):
        return False
    r = subprocess.run(["make", "-s", "-C", HERE, f"REF={ref_root}"], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle/_ref build failed:\n{r.stdout}\n{r.stderr}")
    return True


class RefIVIM:
    """The reference's own generated IVIM LM kernel, run on the host.

    Same call surface as the reference: setup arrays (4, N), consts/data
    (ndata, N); ``lm_run`` repeats ``iters`` launches over all voxels.
    """

    def __init__(self, ndata: int = 21):
        path = os.path.join(REF_DIR, f"libref_ivim{ndata}.so")
        if not os.path.exists(path):
            raise FileNotFoundError(f"{path} missing: build it with build_reference() where the reference tree exists")
        self.ndata = ndata
        self.lib = ctypes.CDLL(path)
        self.lib.ref_lm_run.argtypes = [ctypes.c_int] + [ctypes.c_void_p] * 11 + [ctypes.c_int] + [ctypes.c_float] * 5
        self.lib.ref_search_step.argtypes = [ctypes.c_int] + [ctypes.c_void_p] * 8

    def lm_run(self, pars, consts, data, lb, ub, iters, tol=1e-8, mu=0.25, eta=0.75, acc=0.2, dec=2.0,
               lam=None, step_type=None, f=None, want_step=False):
        P, N = pars.shape
        assert P == 4 and pars.dtype == np.float32 and data.shape[0] == self.ndata
        if consts.ndim == 1 or consts.shape[1] != N:
            consts = np.ascontiguousarray(np.broadcast_to(consts.reshape(self.ndata, -1)[:, :1], (self.ndata, N)))
        if lb.ndim == 1 or lb.shape[1] != N:
            lb = np.ascontiguousarray(np.broadcast_to(lb.reshape(4, -1)[:, :1], (4, N)))
            ub = np.ascontiguousarray(np.broadcast_to(ub.reshape(4, -1)[:, :1], (4, N)))
        f32 = lambda a: np.ascontiguousarray(a, dtype=np.float32)  # noqa: E731
        consts, data, lb, ub = f32(consts), f32(data), f32(lb), f32(ub)
        lam = np.full(N, 5.0, dtype=np.float32) if lam is None else lam
        step_type = np.ones(N, dtype=np.int8) if step_type is None else step_type
        f = np.zeros(N, dtype=np.float32) if f is None else f
        first_f = np.zeros(N, dtype=np.float32)
        last_f = np.zeros(N, dtype=np.float32)
        step = np.zeros((4, N), dtype=np.float32) if want_step else None
        self.lib.ref_lm_run(N, _p(consts), _p(data), _p(lb), _p(ub), _p(pars), _p(lam), _p(step_type), _p(f),
                            _p(first_f), _p(last_f), _p(step), int(iters), tol, mu, eta, acc, dec)
        out = dict(pars=pars, lam=lam, step_type=step_type, f=f, first_f=first_f, last_f=last_f)
        if want_step:
            out["step"] = step
        return out

    def search_step(self, consts, data, lb, ub, best_p, p, best_f, f):
        N = p.shape[1]
        self.lib.ref_search_step(N, _p(consts), _p(data), _p(lb), _p(ub), _p(best_p), _p(p), _p(best_f), _p(f))
