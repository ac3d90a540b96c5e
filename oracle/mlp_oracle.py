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


def bf16_exact(x) -> np.ndarray:
    """Round float64 values to bfloat16 in one step (8 significant bits, round
    to nearest even), as a fused bf16 operation rounds its exact result."""
    x = np.asarray(x, dtype=np.float64)
    with np.errstate(over="ignore", invalid="ignore"):
        m, e = np.frexp(x)
        r = np.ldexp(np.rint(m * 256.0), e - 8)
        return np.where(np.abs(r) > 3.3895313892515355e38, np.sign(x) * np.inf, np.where(np.isfinite(x), r, x))


_CB = float(bf16([_C])[0])
_C3B = float(bf16([0.044715 * _C])[0])


def _trunc_bf16(v):
    """Truncate float64 values through float32 to bfloat16 (toward zero)."""
    u = np.ascontiguousarray(np.asarray(v, dtype=np.float32)).view(np.uint32) & np.uint32(0xFFFF0000)
    return u.view(np.float32).astype(np.float64)


def _tanh_bf16(z):
    """t = tanh(u) for the bf16-rounded z, with u = z (c + c' z^2) rounded as
    the GPU evaluates it in bf16x2 arithmetic (z^2, the fused c' z^2 + c and
    the product each rounded to bf16, overflow -> +-Inf); returns (z_bf16, t).
    tanh.approx.bf16x2 returns its fp32 approximation truncated toward zero
    (measured over all 65,536 bf16 inputs on sm_103a); the oracle truncates the
    exact tanh, which differs from it by one bf16 ulp on ~1.5 % of inputs."""
    zb = bf16(np.asarray(z, dtype=np.float32))
    with np.errstate(over="ignore", invalid="ignore"):
        q = bf16_exact(bf16_exact(zb * zb) * _C3B + _CB)
        u = bf16_exact(zb * q)
        return zb, _trunc_bf16(np.tanh(u))


def _gelu_tanh(z):
    """GELU, tanh form (Hendrycks & Gimpel 2016), as the GPU kernels compute it
    in bf16x2 arithmetic: half of bf16(z t + z) (one fused rounding)."""
    zb, t = _tanh_bf16(z)
    return 0.5 * bf16_exact(zb * t + zb)


def _gelu_tanh_grad(z):
    _, t = _tanh_bf16(z)
    return 0.5 * (1.0 + t) + 0.5 * z * (1.0 - t * t) * _C * (1.0 + 3 * 0.044715 * z * z)


# The polynomial recipe of the columns n with n % 16 < POLY_COLS (the GPU's
# FMA-pipe GELU): 2 gelu(z) ~ 2 relu(z) + (w e(w) - a), a = min(|z|, 3),
# w = a^2, e(w) = q1 + w (q2 + w (q3 + w q4)), every operation in bf16 with one
# rounding (products of bf16 values and the sums formed here are exact in
# float64 wherever the rounding to bf16 can depend on them, so rounding the
# float64 result once to bf16 is the fused operation's rounding).
POLY_COLS = 6
_Q = (0.7890625, -0.11572265625, 0.01116943359375, -0.0004405975341796875)


def _gelu_poly(z):
    B = bf16_exact
    zb = bf16(np.asarray(z, dtype=np.float32))
    with np.errstate(over="ignore", invalid="ignore"):
        a = np.fmin(np.abs(zb), 3.0)
        w = B(a * a)
        e = B(_Q[3] * w + _Q[2])
        e = B(e * w + _Q[1])
        e = B(e * w + _Q[0])
        t = B(e * w - a)
        r2 = np.maximum(B(2.0 * zb), 0.0)
        return 0.5 * B(r2 + t)


def _gelu_poly_grad(z):
    z = np.asarray(z, dtype=np.float64)
    w = z * z
    de = _Q[0] + 2 * _Q[1] * w + 3 * _Q[2] * w * w + 4 * _Q[3] * w ** 3
    inner = 0.5 * (1.0 + 2.0 * z * de)
    return np.where(np.abs(z) >= 3.0, np.where(z > 0, 1.0, 0.0), inner)


def _by_column(fp, ft, z, col):
    z = np.asarray(z)
    if col is None:
        cols = np.arange(z.shape[-1]) if z.ndim >= 1 else np.array(0)
    else:
        cols = np.asarray(col)
    poly = (cols % 16) < POLY_COLS
    return np.where(poly, fp(z), ft(z))


def gelu(z, col=None):
    """The network's activation of z; col: the network column of each entry
    (default: the position along the last axis, as in a (batch x units)
    array). Columns with col % 16 < POLY_COLS use the polynomial recipe, the
    others the tanh recipe."""
    return _by_column(_gelu_poly, _gelu_tanh, z, col)


def gelu_grad(z, col=None):
    return _by_column(_gelu_poly_grad, _gelu_tanh_grad, z, col)


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
