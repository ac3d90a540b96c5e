"""CPU oracle of the warm-start network (TEST INFRASTRUCTURE ONLY).

Forward and backward of the 16 -> 128 -> 128 -> 128 -> P GELU network in
float64 numpy, rounding to bfloat16 at exactly the points where the GPU recipe
stores bf16 (inputs, weights, post-GELU activations, the output gradient and
the pre-activation gradients), so GPU and oracle differ only by the order of
fp32 accumulation. Weight layout as on the GPU: W (rows x in+8) with the bias
in column `in`.
"""
from __future__ import annotations

import numpy as np


def bf16(x) -> np.ndarray:
    """Round float32 values to bfloat16 (round to nearest even), kept as float64."""
    u = np.ascontiguousarray(np.asarray(x, dtype=np.float32)).view(np.uint32)
    u = (u + (((u >> 16) & 1) + 0x7FFF)) & 0xFFFF0000
    return u.view(np.float32).astype(np.float64)


_C = np.sqrt(2.0 / np.pi)


def _tanh_arg(z):
    """u = z (c + c' z^2) rounded as the GPU evaluates it: z, z^2, the fused
    c' z^2 + c and the product each rounded to float16 (overflow -> +-Inf)."""
    with np.errstate(over="ignore", invalid="ignore"):
        h = lambda v: np.asarray(v, dtype=np.float64).astype(np.float16).astype(np.float64)  # noqa: E731
        zh = h(np.asarray(z, dtype=np.float32))
        q = h(h(zh * zh) * float(np.float16(0.044715 * _C)) + float(np.float16(_C)))
        return h(zh * q)


def gelu(z):
    """GELU, tanh form (Hendrycks & Gimpel 2016), with the tanh argument rounded
    to float16 as the GPU kernels compute it (tanh itself exact here)."""
    return 0.5 * z * (1.0 + np.tanh(_tanh_arg(z)))


def gelu_grad(z):
    t = np.tanh(_tanh_arg(z))
    return 0.5 * (1.0 + t) + 0.5 * z * (1.0 - t * t) * _C * (1.0 + 3 * 0.044715 * z * z)


def split(Wfull, fan_in, rows_live):
    W = np.asarray(Wfull, dtype=np.float64)
    return W[:rows_live, :fan_in], W[:rows_live, fan_in]


def forward(x_bf, weights, dims):
    """x_bf: (B, nin) bf16-rounded inputs; weights: list of (rows x in+8) fp32 masters.
    Returns (zs, acts, y) with acts bf16-rounded."""
    acts, zs = [x_bf], []
    a = x_bf
    for li, (fan_in, fan_out) in enumerate(dims):
        W, b = split(weights[li], fan_in, fan_out)
        z = a @ bf16(W).T + b
        if li < len(dims) - 1:
            zs.append(z)
            a = bf16(gelu(z))
            acts.append(a)
        else:
            y = z
    return zs, acts, y


def backward(x_bf, t, weights, dims, nout):
    """Gradients of the mean squared error (mean over batch and outputs) for
    every layer, in the GPU layout (rows x in+8, bias gradient in column in)."""
    B = x_bf.shape[0]
    zs, acts, y = forward(x_bf, weights, dims)
    dy = bf16(2.0 * (y - t[:, :nout]) / (B * nout))
    grads = [None] * len(dims)
    d = dy
    for li in range(len(dims) - 1, -1, -1):
        fan_in, fan_out = dims[li]
        a_prev = acts[li]
        G = np.zeros_like(np.asarray(weights[li], dtype=np.float64))
        G[:fan_out, :fan_in] = d.T @ a_prev
        G[:fan_out, fan_in] = d.sum(axis=0)
        grads[li] = G
        if li > 0:
            W, _ = split(weights[li], fan_in, fan_out)
            d = bf16((d @ bf16(W)) * gelu_grad(zs[li - 1]))
    loss = float(np.mean((y - t[:, :nout]) ** 2))
    return grads, y, loss
