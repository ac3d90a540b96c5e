"""Warm-start network kernels against the numpy oracle (oracle/mlp_oracle.py).

The oracle rounds to bf16 at the same points as the GPU recipe, so the
remaining difference is fp32 accumulation order: GEMMs agree to 1e-5
relative, gradients to 1e-2 in relative Frobenius norm (a bf16 rounding of an
activation that lands on the other side of a tie changes single entries by
one bf16 ulp), fused inference to 1e-2 relative on the parameters.
"""
import ctypes

import numpy as np
import pytest
import torch

from oracle import mlp_oracle as mo
from pycompute_gb300 import _lib, synth
from pycompute_gb300.warmstart import HID, WarmStartMLP

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


@pytest.mark.parametrize("impl", ["tcgen05", "mma"])
@pytest.mark.parametrize("a_layout,b_layout", [(0, 0), (0, 1), (1, 0), (1, 1)])
@pytest.mark.parametrize("M,N,K", [(64, 64, 32), (200, 136, 128), (8, 136, 4096), (4096, 8, 16), (136, 24, 8)])
def test_gemm_layouts(a_layout, b_layout, M, N, K, impl):
    rng = np.random.default_rng(M + N + K)
    A = mo.bf16(rng.standard_normal((M, K)))
    Bm = mo.bf16(rng.standard_normal((K, N)))
    want = A @ Bm
    At = A if a_layout == 0 else A.T
    Bt = Bm.T if b_layout == 0 else Bm
    ta = torch.from_numpy(np.ascontiguousarray(At)).to(DEV, torch.bfloat16)
    tb = torch.from_numpy(np.ascontiguousarray(Bt)).to(DEV, torch.bfloat16)
    net = WarmStartMLP(16, 4, [0, 1, 2, 2], [0] * 4, [1] * 4, DEV)
    net.gemm_impl = impl
    for epi, ksplit in ((4, 0), (3, 256)):
        out = torch.zeros((M, N), device=DEV)
        net._gemm(a_layout, b_layout, epi, ta, ta.shape[1], tb, tb.shape[1], M, N, K, k_split=ksplit,
                  out_f32=out, ldo=N)
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        assert np.abs(got - want).max() <= 1e-5 * np.abs(want).max() + 1e-6
    assert net.gemm_status() == 0


@pytest.mark.parametrize("a_layout,b_layout", [(0, 0), (0, 1), (1, 1)])
@pytest.mark.parametrize("epi", [0, 1, 2])
def test_tcgen05_gemm_epilogues_match_mma(a_layout, b_layout, epi):
    """The fused epilogues of the training step (bias + GELU with the
    pre-activation and bf16 activation stored, bias only, GELU' times the
    gradient) on the tcgen05 GEMM equal the mma.sync GEMM's up to fp32
    summation order: fp32 outputs to 1e-5 of the largest, bf16 outputs
    within one bf16 ulp."""
    M, N, K = 1000, 136, 128
    rng = np.random.default_rng(epi * 7 + a_layout)
    A = mo.bf16(rng.standard_normal((M, K)) * 0.3)
    Bm = mo.bf16(rng.standard_normal((K, N)) * 0.3)
    At = A if a_layout == 0 else A.T
    Bt = Bm.T if b_layout == 0 else Bm
    ta = torch.from_numpy(np.ascontiguousarray(At)).to(DEV, torch.bfloat16)
    tb = torch.from_numpy(np.ascontiguousarray(Bt)).to(DEV, torch.bfloat16)
    bias = torch.from_numpy(rng.standard_normal(N).astype(np.float32)).to(DEV)
    zin = torch.from_numpy(rng.standard_normal((M, N)).astype(np.float32)).to(DEV)
    outs = []
    for impl in ("mma", "tcgen05"):
        net = WarmStartMLP(16, 4, [0, 1, 2, 2], [0] * 4, [1] * 4, DEV)
        net.gemm_impl = impl
        of = torch.zeros((M, N), device=DEV)
        ob = torch.zeros((M, N), dtype=torch.bfloat16, device=DEV)
        net._gemm(a_layout, b_layout, epi, ta, ta.shape[1], tb, tb.shape[1], M, N, K,
                  bias=ctypes.c_void_p(bias.data_ptr()), bias_stride=1, out_f32=of, ldo=N, out_bf16=ob, ldob=N,
                  zin=zin, ldz=N)
        torch.cuda.synchronize()
        assert net.gemm_status() == 0
        outs.append((of.cpu().numpy(), ob.float().cpu().numpy()))
    (f0, b0), (f1, b1) = outs
    assert np.abs(f1 - f0).max() <= 1e-5 * max(np.abs(f0).max(), 1e-30)
    ulp = np.maximum(np.abs(b0), 1e-30) * 2.0 ** -7
    assert np.all(np.abs(b1 - b0) <= ulp + 1e-6)


def _ivim16_batch(B, seed=0):
    w = synth.ivim(synth.ivim_b16(), name="ivim16")
    true, data, init, lb, ub, prot = w.generate(B, seed=seed)
    return w, data, true


def test_gradients_match_oracle():
    B = 512
    w, data, true = _ivim16_batch(B)
    net = WarmStartMLP(16, 4, [0, 1, 2, 2], w.lb, w.ub, DEV, seed=3)
    sig = torch.from_numpy(data).to(DEV)
    lab = torch.from_numpy(true).to(DEV)
    net.fit_normalisation(sig, lab)
    x, snorm, t = net._prepare(sig, lab)
    net._alloc_batch(B)
    net.bx.copy_(x)
    net.bt.copy_(t)
    net._forward_train()
    net._backward(k_split=128)
    torch.cuda.synchronize()
    dims = [(16, HID), (HID, HID), (HID, HID), (HID, 4)]
    x_np = x[:, :16].float().cpu().numpy().astype(np.float64)
    grads, y, loss = mo.backward(x_np, t.cpu().numpy().astype(np.float64),
                                 [L.master.cpu().numpy() for L in net.layers], dims, 4)
    np.testing.assert_allclose(net.y[:, :4].cpu().numpy(), y, rtol=2e-2, atol=2e-3)
    for li, L in enumerate(net.layers):
        g = L.grad.cpu().numpy().astype(np.float64)
        ref = grads[li]
        rel = np.linalg.norm(g - ref) / np.linalg.norm(ref)
        cos = (g * ref).sum() / (np.linalg.norm(g) * np.linalg.norm(ref))
        assert rel < 1e-2 and cos > 0.9999, (li, rel, cos)


@pytest.mark.parametrize("impl", ["mma", "tcgen05"])
@pytest.mark.parametrize("log_in", [False, True])
def test_fused_inference_matches_oracle(log_in, impl):
    B = 3000
    w, data, true = _ivim16_batch(B, seed=1)
    net = WarmStartMLP(16, 4, [0, 1, 2, 2], w.lb, w.ub, DEV, seed=4, log_in=log_in)
    sig = torch.from_numpy(data).to(DEV)
    net.fit_normalisation(sig, torch.from_numpy(true).to(DEV))
    out = net.infer(sig, impl=impl)
    torch.cuda.synchronize()
    assert net.tc_status() == 0
    smax = data.max(axis=0)
    x = data.T / smax[:, None]
    x = mo.bf16(np.log(np.maximum(x, 1e-6)) if log_in else x)
    dims = [(16, HID), (HID, HID), (HID, HID), (HID, 4)]
    _, _, y = mo.forward(x, [L.master.cpu().numpy() for L in net.layers], dims)
    t = y * net.std + net.mean
    p = np.stack([t[:, 0] * smax, t[:, 1], np.exp(t[:, 2]), np.exp(t[:, 3])])
    p = np.clip(p, np.array(w.lb)[:, None], np.array(w.ub)[:, None])
    np.testing.assert_allclose(out.cpu().numpy(), p, rtol=1e-2, atol=1e-6)


@pytest.mark.parametrize("n", [1, 127, 129, 1000, 65537])
def test_tcgen05_inference_matches_mma(n):
    """Both inference kernels round to bf16 at the same points; the tcgen05
    kernel adds each bias as two bf16 terms inside the MMA (b to 2^-16), so
    pre-activations differ in the last fp32 bits and an occasional bf16
    rounding of an activation flips."""
    w = synth.ivim(synth.ivim_b16(), name="ivim16")
    true, data, *_ = w.generate(max(n, 2), seed=9)
    data, true = data[:, :n], true[:, :n]
    net = WarmStartMLP(16, 4, [0, 1, 2, 2], w.lb, w.ub, DEV, seed=6, log_in=True)
    sig = torch.from_numpy(np.ascontiguousarray(data)).to(DEV)
    net.fit_normalisation(sig, torch.from_numpy(np.ascontiguousarray(true)).to(DEV))
    a = net.infer(sig, impl="mma")
    b = net.infer(sig, impl="tcgen05")
    torch.cuda.synchronize()
    assert net.tc_status() == 0
    np.testing.assert_allclose(b.cpu().numpy(), a.cpu().numpy(), rtol=1e-2, atol=1e-7)
    rel = ((a - b).abs() / a.abs().clamp_min(1e-30)).flatten()
    assert float(rel.median()) < 1e-3


def test_training_reduces_loss_and_graph_matches_eager():
    B = 2048
    w, data, true = _ivim16_batch(B * 8, seed=2)
    sig = torch.from_numpy(data).to(DEV)
    lab = torch.from_numpy(true).to(DEV)
    nets = []
    for use_graph in (True, False):
        net = WarmStartMLP(16, 4, [0, 1, 2, 2], w.lb, w.ub, DEV, seed=5)
        net.train(sig, lab, epochs=4, batch=B, lr=2e-3, use_graph=use_graph, log_every=8)
        nets.append(net)
    g, e = nets
    assert g.losses[-1] < 0.8 * g.losses[0] and all(np.diff(g.losses) < 0), g.losses
    # split-K weight gradients accumulate with atomics, so the two runs differ
    # in summation order only: same loss curve, nearly the same weights
    np.testing.assert_allclose(g.losses, e.losses, rtol=0.05)
    for a, b in zip(g.layers, e.layers):
        torch.testing.assert_close(a.master, b.master, rtol=0.05, atol=2e-2)


def test_gelu_recipe_matches_oracle():
    """The activation every network kernel computes (2 gelu in bf16x2
    arithmetic, tanh.approx.bf16x2) against the oracle's restatement of the
    recipe: bit-equal except where the hardware tanh's truncated fp32
    approximation and the truncated exact tanh fall on different bf16 values.
    One ulp of t (at most 2^-8) moves z t by |z| 2^-8, which can tip the bf16
    rounding of z t + z by one ulp of the result (up to 2 |z| 2^-8): at most
    1.5 |z| 2^-8 in gelu. The derivative (fp32 on the GPU) agrees to 1e-5 for
    most inputs and everywhere within what one ulp of t (at most |t| 2^-7)
    moves it: (1/2 + |z t| k(z)) |t| 2^-7, k(z) = sqrt(2/pi) (1 + 3 0.044715 z^2)."""
    rng = np.random.default_rng(5)
    z = np.concatenate([np.linspace(-12, 12, 240001), rng.standard_normal(100000) * 3,
                        [0.0, -0.0, 1e-30, -1e-30, 40.0, -40.0]]).astype(np.float32)
    zt = torch.from_numpy(z).to(DEV)
    g = torch.empty_like(zt)
    dg = torch.empty_like(zt)
    rc = _lib.lib().pcgb_mlp_gelu(ctypes.c_void_p(zt.data_ptr()), zt.numel(), 15, ctypes.c_void_p(g.data_ptr()),
                                  ctypes.c_void_p(dg.data_ptr()), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    _lib.check("pcgb_mlp_gelu", rc)
    torch.cuda.synchronize()
    g, dg = g.cpu().numpy().astype(np.float64), dg.cpu().numpy().astype(np.float64)
    want = mo.gelu(z, col=15)
    same = g == want
    assert same.mean() > 0.97, same.mean()
    zb = mo.bf16(z)
    assert np.all(np.abs(g - want) <= np.abs(zb) * 1.5 * 2.0 ** -8 + 1e-30), np.abs(g - want).max()
    zd = z.astype(np.float64)
    want_d = mo.gelu_grad(zd, col=15)
    _, t = mo._tanh_bf16(z)
    k = np.sqrt(2 / np.pi) * (1 + 3 * 0.044715 * zd * zd)
    tol = (0.5 + np.abs(zd * t) * k) * np.maximum(np.abs(t), 2.0 ** -126) * 2.0 ** -7 + 1e-6 + 1e-5 * np.abs(want_d)
    assert np.all(np.isfinite(want_d))
    assert np.isclose(dg, want_d, rtol=1e-5, atol=1e-6).mean() > 0.95
    assert np.all(np.abs(dg - want_d) <= tol), np.max(np.abs(dg - want_d) / tol)
    assert g[np.where(z == 40.0)[0][0]] == 40.0 and g[np.where(z == -40.0)[0][0]] == 0.0


def test_polynomial_gelu_matches_oracle_bit_for_bit():
    """The FMA-pipe GELU of columns n % 16 < 6 (bf16x2 polynomial, no MUFU
    operation) equals the oracle's restatement of its bf16 roundings bit for
    bit, column 0 through 5 alike and columns 6 to 15 not, from tiny to huge
    inputs; its fp32 derivative agrees with the oracle's float64 evaluation
    to 1e-5."""
    rng = np.random.default_rng(6)
    z = np.concatenate([np.linspace(-40, 40, 400001), rng.standard_normal(100000) * 3,
                        [0.0, -0.0, 1e-30, -1e-30, 1e-20, -1e-20, 3.0, -3.0, 2.9999, -2.9999, 65000.0, -65000.0,
                         1e30, -1e30]]).astype(np.float32)
    zt = torch.from_numpy(z).to(DEV)
    for col in (0, 5, 16 * 7 + 2):
        g = torch.empty_like(zt)
        dg = torch.empty_like(zt)
        rc = _lib.lib().pcgb_mlp_gelu(ctypes.c_void_p(zt.data_ptr()), zt.numel(), col, ctypes.c_void_p(g.data_ptr()),
                                      ctypes.c_void_p(dg.data_ptr()),
                                      ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
        _lib.check("pcgb_mlp_gelu", rc)
        torch.cuda.synchronize()
        g, dg = g.cpu().numpy().astype(np.float64), dg.cpu().numpy().astype(np.float64)
        want = mo.gelu(z, col=col)
        np.testing.assert_array_equal(g, want)
        np.testing.assert_allclose(dg, mo.gelu_grad(z.astype(np.float64), col=col), rtol=1e-5, atol=1e-6)
    assert not np.array_equal(mo.gelu(z, col=6), mo.gelu(z, col=0))


@pytest.mark.parametrize("K", [16, 64, 128])
def test_tcgen05_gemm_lost_wait_sets_status_frees_tmem_and_returns(K):
    """The failure path of the tcgen05 training GEMM, made to run without any
    fault: through pcgb_gemm_bf16_tc_ex, CTA 0 (output rows 0-127, columns
    0-31) never issues its MMAs nor their commits, so its first mbarrier wait
    - the buffer reuse at K step 2, or the final wait for one and two K steps
    (K = 16, 64) - never completes while none of its tensor-core work is in
    flight. With a short wait limit the wait runs out: the call returns
    normally, the status word reads 1, CTA 0's tile is not written and every
    other tile equals the mma.sync GEMM. A normal call right after it equals
    the mma.sync GEMM everywhere, which it could not if the failed CTA had
    not freed its tensor memory."""
    M, N = 1000, 136
    rng = np.random.default_rng(K)
    A = mo.bf16(rng.standard_normal((M, K)) * 0.3)
    Bm = mo.bf16(rng.standard_normal((K, N)) * 0.3)
    ta = torch.from_numpy(np.ascontiguousarray(A)).to(DEV, torch.bfloat16)
    tb = torch.from_numpy(np.ascontiguousarray(Bm.T)).to(DEV, torch.bfloat16)
    bias = torch.from_numpy(rng.standard_normal(N).astype(np.float32)).to(DEV)
    net = WarmStartMLP(16, 4, [0, 1, 2, 2], [0] * 4, [1] * 4, DEV)
    net.gemm_impl = "mma"
    want = torch.zeros((M, N), device=DEV)
    net._gemm(0, 0, 1, ta, K, tb, K, M, N, K, bias=ctypes.c_void_p(bias.data_ptr()), bias_stride=1, out_f32=want,
              ldo=N)
    p = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    out = torch.full((M, N), -7.0, device=DEV)
    status = torch.zeros(1, dtype=torch.int32, device=DEV)
    rc = _lib.lib().pcgb_gemm_bf16_tc_ex(0, 0, 1, p(ta), K, p(tb), K, M, N, K, 0, p(bias), 1, p(out), N, None, 0,
                                         None, 0, p(status), 1 << 10, 0, stream)
    _lib.check("pcgb_gemm_bf16_tc_ex", rc)
    torch.cuda.synchronize()
    assert int(status.item()) == 1
    got, ref = out.cpu().numpy(), want.cpu().numpy()
    assert np.all(got[:128, :32] == -7.0)
    mask = np.ones((M, N), bool)
    mask[:128, :32] = False
    assert np.abs(got - ref)[mask].max() <= 1e-5 * np.abs(ref).max()
    status.zero_()
    out.fill_(-7.0)
    rc = _lib.lib().pcgb_gemm_bf16_tc_ex(0, 0, 1, p(ta), K, p(tb), K, M, N, K, 0, p(bias), 1, p(out), N, None, 0,
                                         None, 0, p(status), 0, -1, stream)
    _lib.check("pcgb_gemm_bf16_tc_ex", rc)
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    assert np.abs(out.cpu().numpy() - ref).max() <= 1e-5 * np.abs(ref).max()


def test_tcgen05_lost_wait_sets_status_frees_tmem_and_returns():
    """The failure path of the tcgen05 network kernel, made to run without any
    fault: through pcgb_mlp_forward_tc_ex, the issuing thread of the warpgroup
    that owns tile 0 never issues that tile's first layer nor its commit, so
    the layer's mbarrier phase never completes while none of that warpgroup's
    tensor-core work is in flight. With a short wait limit the wait runs out:
    the call returns normally, the status word reads 1 and the other tiles
    are still computed. A normal inference right after it must succeed and
    equal the mma.sync kernel on every voxel, which it could not if the tensor
    memory of the failed launch had not been freed (every CTA allocates all
    512 columns of its SM)."""
    w = synth.ivim(synth.ivim_b16(), name="ivim16")
    n = 128 * 12 + 77  # 13 tiles on 4 CTAs (one tile per warpgroup), a ragged last tile
    true, data, *_ = w.generate(n, seed=13)
    net = WarmStartMLP(16, 4, [0, 1, 2, 2], w.lb, w.ub, DEV, seed=8, log_in=True)
    sig = torch.from_numpy(np.ascontiguousarray(data)).to(DEV)
    net.fit_normalisation(sig, torch.from_numpy(np.ascontiguousarray(true)).to(DEV))
    want = net.infer(sig, impl="mma")
    out = torch.full((4, n), -1.0, device=DEV)
    status = torch.zeros(1, dtype=torch.int32, device=DEV)
    wb = (ctypes.c_void_p * 4)(*[L.wbf.data_ptr() for L in net.layers])
    wm = (ctypes.c_void_p * 4)(*[L.master.data_ptr() for L in net.layers])
    kinds = (ctypes.c_int * 4)(*net.kinds)
    fl = lambda v: (ctypes.c_float * 4)(*[float(x) for x in v])  # noqa: E731
    p = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
    rc = _lib.lib().pcgb_mlp_forward_tc_ex(p(sig), n, 16, 1, wb, wm, 4, kinds, fl(net.mean), fl(net.std), fl(net.lb),
                                           fl(net.ub), p(out), p(status), 1 << 12, 0,
                                           ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    _lib.check("pcgb_mlp_forward_tc_ex", rc)
    torch.cuda.synchronize()
    assert int(status.item()) == 1
    # tile 0 was never computed; every other tile (other warpgroups and CTAs) was
    got, ref = out.cpu().numpy(), want.cpu().numpy()
    assert np.all(got[:, :128] == -1.0)
    np.testing.assert_allclose(got[:, 128:], ref[:, 128:], rtol=1e-2, atol=1e-7)
    net.clear_tc_status()
    again = net.infer(sig, impl="tcgen05")
    torch.cuda.synchronize()
    assert net.tc_status() == 0
    np.testing.assert_allclose(again.cpu().numpy(), ref, rtol=1e-2, atol=1e-7)
