"""The reference's own generated IVIM LM kernel on the GPU (TEST INFRASTRUCTURE
ONLY: parity tests and the reference arm of the benchmark).

oracle/_ref/ref_lm_ivim{10,16}_sm103a.cubin is built by oracle/Makefile from
the reference tree (test/ivim/second_order_levenberg_marquardt_4_1_21_f_f7def86f0a03.cu
with its out-of-range parameter loads bounded, its printf calls dropped and
its sample count set). This module launches it exactly as the reference's
SecondOrderLevenbergMarquardt.setup/run do (pycompute/cuda/lsqnonlin.py:1036-1073):
scratch arrays allocated once, lambda = 5, step_type = 1, then `iters` launches
of 32-thread blocks over all voxels, first_f / last_f copied after the first
and the last launch. Launches go through the CUDA driver API (ctypes) on
PyTorch's current context and stream; buffers are PyTorch CUDA tensors.
"""
from __future__ import annotations

import ctypes
import os

import torch

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
KERNEL = "k_second_order_levenberg_marquardt_4_1_21_f_f7def86f0a03"


def cubin_path(ndata: int) -> str:
    return os.path.join(REF_DIR, f"ref_lm_ivim{ndata}_sm103a.cubin")


def available(ndata: int) -> bool:
    return os.path.exists(cubin_path(ndata))


class RefGpuIVIM:
    """The reference LM kernel for IVIM with `ndata` samples, on the GPU."""

    _cuda = None

    def __init__(self, ndata: int):
        path = cubin_path(ndata)
        if not os.path.exists(path):
            raise FileNotFoundError(f"{path} missing: build it with oracle/Makefile where the reference tree exists")
        if RefGpuIVIM._cuda is None:
            cu = ctypes.CDLL("libcuda.so.1")
            vp, ui = ctypes.c_void_p, ctypes.c_uint
            cu.cuModuleLoad.argtypes = [ctypes.POINTER(vp), ctypes.c_char_p]
            cu.cuModuleGetFunction.argtypes = [ctypes.POINTER(vp), vp, ctypes.c_char_p]
            cu.cuLaunchKernel.argtypes = [vp, ui, ui, ui, ui, ui, ui, ui, vp, vp, vp]
            RefGpuIVIM._cuda = cu
        cu = RefGpuIVIM._cuda
        torch.cuda.init()
        torch.zeros(1, device="cuda")  # PyTorch's primary context is current on this thread
        self.ndata = ndata
        self.mod = ctypes.c_void_p()
        self._check(cu.cuModuleLoad(ctypes.byref(self.mod), path.encode()), "cuModuleLoad")
        self.fn = ctypes.c_void_p()
        self._check(cu.cuModuleGetFunction(ctypes.byref(self.fn), self.mod, KERNEL.encode()), "cuModuleGetFunction")

    @staticmethod
    def _check(rc, what):
        if rc != 0:
            raise RuntimeError(f"{what} failed with CUresult {rc}")

    def setup(self, pars, consts, data, lb, ub):
        """Reference setup(): pars (4, N) in place; consts (ndata, N) tiled per voxel;
        data (ndata, N); lb, ub (4, N); all float32 CUDA tensors."""
        N = int(pars.shape[1])
        dev = pars.device
        self.N = N
        self.pars, self.consts, self.data, self.lb, self.ub = pars, consts, data, lb, ub
        z = lambda *s: torch.zeros(s, dtype=torch.float32, device=dev)  # noqa: E731
        self.pars_tp, self.step, self.g = z(4, N), z(4, N), z(4, N)
        self.h, self.hl = z(10, N), z(10, N)
        self.lam = torch.full((1, N), 5.0, dtype=torch.float32, device=dev)
        self.step_type = torch.ones((1, N), dtype=torch.int8, device=dev)
        self.f, self.ftp = z(1, N), z(1, N)
        self.first_f, self.last_f = z(1, N), z(1, N)

    def run(self, iters: int, tol=1e-8, mu=0.25, eta=0.75, acc=0.2, dec=2.0):
        """Reference run(): `iters` launches of ceil(N/32) blocks of 32 threads."""
        p = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
        vals = [p(self.consts), p(self.data), p(self.lb), p(self.ub), ctypes.c_float(tol), ctypes.c_float(mu),
                ctypes.c_float(eta), ctypes.c_float(acc), ctypes.c_float(dec), p(self.pars), p(self.pars_tp),
                p(self.step), p(self.lam), p(self.step_type), p(self.f), p(self.ftp), p(self.g), p(self.h),
                p(self.hl), ctypes.c_int(self.N)]
        args = (ctypes.c_void_p * len(vals))(*[ctypes.cast(ctypes.pointer(v), ctypes.c_void_p) for v in vals])
        stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        grid = (self.N + 31) // 32
        for it in range(iters):
            self._check(RefGpuIVIM._cuda.cuLaunchKernel(self.fn, grid, 1, 1, 32, 1, 1, 0, stream, args, None),
                        "cuLaunchKernel")
            if it == 0:
                self.first_f.copy_(self.f)
            if it == iters - 1:
                self.last_f.copy_(self.f)
