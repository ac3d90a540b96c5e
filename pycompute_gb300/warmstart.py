"""Learned warm start for the LM fitter.

A 16 -> 128 -> 128 -> 128 -> P GELU (tanh form) network maps a voxel's signal curve to
initial parameters. Weights are bf16 on the tensor cores with fp32 master
copies and fp32 accumulation; training and inference run in libpcgb.so's
hand-written kernels (csrc/mlp.cu): GEMMs with fused bias/GELU/GELU'
epilogues and split-K weight gradients, a mean-squared-error gradient, Adam,
and a fused four-layer inference kernel. One training step (forward, backward,
Adam on all layers) is captured once as a CUDA graph and replayed per batch.

Inputs are the signals divided by their per-voxel maximum, or (``log_in``,
the default) the logarithm of that ratio, which turns exponential decays into
near-linear curves. Targets are the
parameters in a normalised space chosen per output ("kinds"): 0 = value
divided by the signal maximum (an amplitude such as S0), 1 = the value itself
(a fraction such as f), 2 = its logarithm (a rate or diffusivity), each then
standardised with the training set's mean and standard deviation.

The network is trained on signals of the package's own forward models with
Rician noise, with the plain LM's fits of those signals as labels (so it
learns where the fitter converges, not the noise-free truth).
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib

HID = 128


def _p(t):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def adam_step_constants(step0: int, total: int, b1: float = 0.9, b2: float = 0.999) -> torch.Tensor:
    """(total, 3) float32 rows for the training steps step0 + 1 .. step0 + total:
    Adam's bias corrections 1 - b1^s and 1 - b2^s and the cosine-decay scale
    (1 + cos(pi i / total)) / 2 of the i-th step of the run."""
    return torch.tensor([[1 - b1 ** (step0 + 1 + i), 1 - b2 ** (step0 + 1 + i), 0.5 * (1.0 + np.cos(np.pi * i / total))]
                         for i in range(total)], dtype=torch.float32)


@dataclass
class _Layer:
    fan_in: int
    rows: int       # outputs, padded to a multiple of 8
    rows_live: int
    master: torch.Tensor
    m: torch.Tensor
    v: torch.Tensor
    grad: torch.Tensor
    wbf: torch.Tensor

    @property
    def ld(self) -> int:
        return self.fan_in + 8


class WarmStartMLP:
    """Signal curve -> LM initial parameters (see module docstring)."""

    def __init__(self, nin: int, nout: int, kinds, lb, ub, device=None, seed: int = 0, log_in: bool = True):
        if nin != 16:
            raise ValueError("the fused inference kernel is built for 16 inputs")
        if not 1 <= nout <= 8:
            raise ValueError("nout must be 1..8")
        self.nin, self.nout = nin, nout
        self.log_in = bool(log_in)
        # training GEMMs: "tcgen05" (tensor memory accumulators) or "mma" (warp-level mma.sync)
        self.gemm_impl = "tcgen05"
        self.kinds = list(kinds)
        self.lb = [float(x) for x in lb]
        self.ub = [float(x) for x in ub]
        self.device = torch.device(device or "cuda")
        self.mean = np.zeros(nout, np.float32)
        self.std = np.ones(nout, np.float32)
        g = torch.Generator().manual_seed(seed)
        dims = [(nin, HID), (HID, HID), (HID, HID), (HID, nout)]
        self.layers: list[_Layer] = []
        for fan_in, fan_out in dims:
            rows = (fan_out + 7) // 8 * 8
            ld = fan_in + 8
            w = torch.zeros(rows, ld)
            bound = (6.0 / fan_in) ** 0.5 * (0.5 if fan_out == nout else 1.0)
            w[:fan_out, :fan_in] = (torch.rand(fan_out, fan_in, generator=g) * 2 - 1) * bound
            mk = lambda: torch.zeros(rows, ld, device=self.device)  # noqa: E731
            master = w.to(self.device)
            self.layers.append(_Layer(fan_in, rows, fan_out, master, mk(), mk(), mk(),
                                      master.to(torch.bfloat16).contiguous()))
        self.step = 0
        self._graph = None
        self.losses: list[float] = []

    # ---- persistence -----------------------------------------------------
    def state_dict(self) -> dict:
        d = {"nin": self.nin, "nout": self.nout, "log_in": int(self.log_in), "kinds": np.array(self.kinds),
             "lb": np.array(self.lb),
             "ub": np.array(self.ub), "mean": self.mean, "std": self.std, "step": self.step}
        for i, L in enumerate(self.layers):
            d[f"w{i}"] = L.master.cpu().numpy()
        return d

    def save(self, path: str):
        np.savez_compressed(path, **self.state_dict())

    @classmethod
    def load(cls, path: str, device=None) -> "WarmStartMLP":
        z = np.load(path)
        net = cls(int(z["nin"]), int(z["nout"]), list(z["kinds"]), list(z["lb"]), list(z["ub"]), device,
                  log_in=bool(int(z["log_in"])) if "log_in" in z.files else False)
        net.mean, net.std, net.step = z["mean"].astype(np.float32), z["std"].astype(np.float32), int(z["step"])
        for i, L in enumerate(net.layers):
            L.master.copy_(torch.from_numpy(z[f"w{i}"]))
            L.wbf.copy_(L.master.to(torch.bfloat16))
        return net

    # ---- data ---------------------------------------------------------------
    def _prepare(self, signals: torch.Tensor, params: torch.Tensor | None):
        n = signals.shape[1]
        ldx = self.nin + 8
        x = torch.empty((n, ldx), dtype=torch.bfloat16, device=self.device)
        snorm = torch.empty(n, dtype=torch.float32, device=self.device)
        t = None
        if params is not None:
            t = torch.empty((n, 8), dtype=torch.float32, device=self.device)
            kinds = torch.tensor(self.kinds, dtype=torch.int32, device=self.device)
            mean = torch.from_numpy(self.mean).to(self.device)
            std = torch.from_numpy(self.std).to(self.device)
        rc = _lib.lib().pcgb_mlp_prepare(_p(signals), n, self.nin, int(self.log_in), _p(x), ldx, _p(snorm),
                                         _p(params), self.nout,
                                         _p(kinds) if t is not None else None, _p(mean) if t is not None else None,
                                         _p(std) if t is not None else None, _p(t), 8, _stream())
        _lib.check("pcgb_mlp_prepare", rc)
        return x, snorm, t

    def fit_normalisation(self, signals: torch.Tensor, params: torch.Tensor):
        """Mean / std of the transformed targets over a training set."""
        smax = signals.max(dim=0).values.clamp_min(1e-20).double().cpu().numpy()
        p = params.double().cpu().numpy()
        for k, kind in enumerate(self.kinds):
            gk = p[k] / smax if kind == 0 else (np.log(np.maximum(p[k], 1e-30)) if kind == 2 else p[k])
            self.mean[k] = gk.mean()
            self.std[k] = max(gk.std(), 1e-6)

    # ---- training -----------------------------------------------------------
    def _alloc_batch(self, B: int):
        dev = self.device
        bf = torch.bfloat16
        self.B = B
        self.bx = torch.zeros((B, self.nin + 8), dtype=bf, device=dev)
        self.bt = torch.zeros((B, 8), dtype=torch.float32, device=dev)
        self.z = [torch.empty((B, HID), device=dev) for _ in range(3)]
        self.a = []
        for _ in range(3):
            a = torch.zeros((B, HID + 8), dtype=bf, device=dev)
            a[:, HID] = 1.0  # ones column: the weight-gradient GEMM then yields the bias gradient
            self.a.append(a)
        self.y = torch.empty((B, 8), device=dev)
        self.dy = torch.zeros((B, 8), dtype=bf, device=dev)
        self.dz = [torch.empty((B, HID), dtype=bf, device=dev) for _ in range(3)]
        self.loss_sum = torch.zeros(1, device=dev)
        self.corr = torch.zeros(3, device=dev)

    def _gemm(self, a_layout, b_layout, epi, A, lda, Bm, ldb, M, N, K, k_split=0, bias=None, bias_stride=0,
              out_f32=None, ldo=0, out_bf16=None, ldob=0, zin=None, ldz=0):
        if self.gemm_impl == "tcgen05":
            if getattr(self, "_gemm_status", None) is None:
                self._gemm_status = torch.zeros(1, dtype=torch.int32, device=self.device)
            rc = _lib.lib().pcgb_gemm_bf16_tc(a_layout, b_layout, epi, _p(A), lda, _p(Bm), ldb, M, N, K, k_split,
                                              bias, bias_stride, _p(out_f32), ldo, _p(out_bf16), ldob, _p(zin),
                                              ldz, _p(self._gemm_status), _stream())
            _lib.check("pcgb_gemm_bf16_tc", rc)
            return
        rc = _lib.lib().pcgb_gemm_bf16(a_layout, b_layout, epi, _p(A), lda, _p(Bm), ldb, M, N, K, k_split,
                                       bias, bias_stride, _p(out_f32), ldo, _p(out_bf16), ldob, _p(zin), ldz,
                                       _stream())
        _lib.check("pcgb_gemm_bf16", rc)

    def gemm_status(self) -> int:
        """Nonzero if a tcgen05 training GEMM gave up on a bounded wait (reads the device flag)."""
        st = getattr(self, "_gemm_status", None)
        return 0 if st is None else int(st.item())

    def _bias_ptr(self, L: _Layer):
        return ctypes.c_void_p(L.master.data_ptr() + 4 * L.fan_in)

    def _forward_train(self):
        B, L = self.B, self.layers
        self._gemm(0, 0, 0, self.bx, self.nin + 8, L[0].wbf, L[0].ld, B, HID, self.nin, bias=self._bias_ptr(L[0]),
                   bias_stride=L[0].ld, out_f32=self.z[0], ldo=HID, out_bf16=self.a[0], ldob=HID + 8)
        for i in (1, 2):
            self._gemm(0, 0, 0, self.a[i - 1], HID + 8, L[i].wbf, L[i].ld, B, HID, HID, bias=self._bias_ptr(L[i]),
                       bias_stride=L[i].ld, out_f32=self.z[i], ldo=HID, out_bf16=self.a[i], ldob=HID + 8)
        self._gemm(0, 0, 1, self.a[2], HID + 8, L[3].wbf, L[3].ld, B, 8, HID, bias=self._bias_ptr(L[3]),
                   bias_stride=L[3].ld, out_f32=self.y, ldo=8)

    def _backward(self, k_split: int):
        B, L = self.B, self.layers
        rc = _lib.lib().pcgb_mlp_mse_grad(_p(self.y), _p(self.bt), 8, B, self.nout, 8, _p(self.dy), 8,
                                          _p(self.loss_sum), _stream())
        _lib.check("pcgb_mlp_mse_grad", rc)
        # layer 4: dW4 = dy^T [a3, 1]; dz3 = (dy W4) * gelu'(z3)
        self._gemm(1, 1, 3, self.dy, 8, self.a[2], HID + 8, 8, HID + 8, B, k_split, out_f32=L[3].grad, ldo=L[3].ld)
        self._gemm(0, 1, 2, self.dy, 8, L[3].wbf, L[3].ld, B, HID, 8, out_bf16=self.dz[2], ldob=HID, zin=self.z[2],
                   ldz=HID)
        for i in (2, 1):
            self._gemm(1, 1, 3, self.dz[i], HID, self.a[i - 1], HID + 8, HID, HID + 8, B, k_split,
                       out_f32=L[i].grad, ldo=L[i].ld)
            self._gemm(0, 1, 2, self.dz[i], HID, L[i].wbf, L[i].ld, B, HID, HID, out_bf16=self.dz[i - 1], ldob=HID,
                       zin=self.z[i - 1], ldz=HID)
        self._gemm(1, 1, 3, self.dz[0], HID, self.bx, self.nin + 8, HID, self.nin + 8, B, k_split,
                   out_f32=L[0].grad, ldo=L[0].ld)

    def _adam(self, lr, b1=0.9, b2=0.999, eps=1e-8):
        for L in self.layers:
            rc = _lib.lib().pcgb_adam_step(_p(L.master), _p(L.m), _p(L.v), _p(L.grad), _p(L.wbf), L.rows, L.ld,
                                           L.rows_live, lr, b1, b2, eps, _p(self.corr), _stream())
            _lib.check("pcgb_adam_step", rc)

    def _train_step_launches(self, lr, k_split):
        self._forward_train()
        self._backward(k_split)
        self._adam(lr)

    def train(self, signals: torch.Tensor, params: torch.Tensor, epochs: int = 10, batch: int = 8192,
              lr: float = 2e-3, seed: int = 0, use_graph: bool = True, log_every: int = 0):
        """Train on signals (nin, n) and label parameters (nout, n), both fp32 on the device."""
        with torch.cuda.device(self.device):
            self.fit_normalisation(signals, params)
            x, snorm, t = self._prepare(signals, params)
            n = x.shape[0]
            rng = np.random.default_rng(seed)
            perm = torch.from_numpy(rng.permutation(n)).to(self.device)
            x, t = x[perm].contiguous(), t[perm].contiguous()
            nb = n // batch
            if nb < 1:
                raise ValueError("training set smaller than one batch")
            self._alloc_batch(batch)
            k_split = max(256, (batch // 32 + 31) // 32 * 32)
            b1, b2 = 0.9, 0.999
            graph = None
            total = epochs * nb
            # per step: Adam's two bias corrections and the cosine-decay scale,
            # made once and read from device memory (no host copy per step, so
            # the host queues steps ahead of the device)
            corr_tab = adam_step_constants(self.step, total, b1, b2).to(self.device)
            done = 0
            for ep in range(epochs):
                for b in range(nb):
                    self.bx.copy_(x[b * batch:(b + 1) * batch])
                    self.bt.copy_(t[b * batch:(b + 1) * batch])
                    self.step += 1
                    self.corr.copy_(corr_tab[done])
                    if not use_graph or done == 0:
                        # the first step runs eagerly so every kernel is loaded before capture
                        self._train_step_launches(lr, k_split)
                    else:
                        if graph is None:
                            torch.cuda.synchronize()
                            graph = torch.cuda.CUDAGraph()
                            s = torch.cuda.Stream()
                            s.wait_stream(torch.cuda.current_stream())
                            with torch.cuda.stream(s):
                                with torch.cuda.graph(graph, stream=s):
                                    self._train_step_launches(lr, k_split)
                            torch.cuda.current_stream().wait_stream(s)
                        graph.replay()
                    done += 1
                    if log_every and done % log_every == 0:
                        self.losses.append(float(self.loss_sum.item()) / log_every)
                        self.loss_sum.zero_()
            torch.cuda.synchronize()
        return self

    # ---- inference ------------------------------------------------------------
    def infer(self, signals: torch.Tensor, out: torch.Tensor | None = None, impl: str = "tcgen05") -> torch.Tensor:
        """Initial parameters (nout, n) for signals (nin, n).

        ``impl="tcgen05"`` (default) runs the tensor-memory kernel,
        ``impl="mma"`` the warp-level mma.sync kernel; both compute the same
        network with the same bf16 roundings.
        """
        n = signals.shape[1]
        if out is None:
            out = torch.empty((self.nout, n), dtype=torch.float32, device=signals.device)
        wb = (ctypes.c_void_p * 4)(*[L.wbf.data_ptr() for L in self.layers])
        wm = (ctypes.c_void_p * 4)(*[L.master.data_ptr() for L in self.layers])
        kinds = (ctypes.c_int * self.nout)(*self.kinds)
        fl = lambda v: (ctypes.c_float * self.nout)(*[float(x) for x in v])  # noqa: E731
        with torch.cuda.device(signals.device):
            if impl == "tcgen05":
                if getattr(self, "_status", None) is None or self._status.device != signals.device:
                    self._status = torch.zeros(1, dtype=torch.int32, device=signals.device)
                rc = _lib.lib().pcgb_mlp_forward_tc(_p(signals), n, self.nin, int(self.log_in), wb, wm, self.nout,
                                                    kinds, fl(self.mean), fl(self.std), fl(self.lb), fl(self.ub),
                                                    _p(out), _p(self._status), _stream())
                _lib.check("pcgb_mlp_forward_tc", rc)
            elif impl == "mma":
                rc = _lib.lib().pcgb_mlp_forward(_p(signals), n, self.nin, int(self.log_in), wb, wm, self.nout,
                                                 kinds, fl(self.mean), fl(self.std), fl(self.lb), fl(self.ub),
                                                 _p(out), _stream())
                _lib.check("pcgb_mlp_forward", rc)
            else:
                raise ValueError("impl must be 'tcgen05' or 'mma'")
        return out

    def tc_status(self) -> int:
        """Nonzero if a tcgen05 inference gave up on a bounded wait (reads the device flag)."""
        st = getattr(self, "_status", None)
        return 0 if st is None else int(st.item())

    def clear_tc_status(self):
        """Reset the device flag that tc_status() reads (it stays set once set)."""
        st = getattr(self, "_status", None)
        if st is not None:
            st.zero_()
