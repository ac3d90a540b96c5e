"""Device arithmetic helpers of the FP64 solve checked against correctly
rounded results: the Newton-Raphson reciprocal must stay within 1 ulp of
1/x (IEEE division on the GPU) everywhere, and return exactly 1/x for the
inputs it hands to the hardware reciprocal (zero, infinities, NaN,
subnormals and exponents outside the float range); the integer-pipe
double -> float rounding must equal the hardware conversion bit for bit."""
import ctypes

import numpy as np
import pytest
import torch

from pycompute_gb300 import _lib

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


def _helpers(x: torch.Tensor):
    y = torch.empty_like(x)
    f = torch.empty(x.shape, dtype=torch.float32, device=x.device)
    rc = _lib.lib().pcgb_fp64_helpers(ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(y.data_ptr()),
                                      ctypes.c_void_p(f.data_ptr()), x.numel(),
                                      ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    _lib.check("pcgb_fp64_helpers", rc)
    torch.cuda.synchronize()
    return y, f


def _rcp64(x: torch.Tensor) -> torch.Tensor:
    return _helpers(x)[0]


def _same_bits(a: torch.Tensor, b: torch.Tensor) -> bool:
    return bool(((a.view(torch.int32) == b.view(torch.int32)) | (torch.isnan(a) & torch.isnan(b))).all())


def _ulps(a: torch.Tensor, b: torch.Tensor) -> torch.Tensor:
    """|a - b| in units in the last place, for finite doubles of equal sign."""
    ia, ib = a.view(torch.int64), b.view(torch.int64)
    return (ia - ib).abs()


def test_rcp64_random_within_one_ulp():
    rng = np.random.default_rng(11)
    n = 1 << 22
    mant = rng.uniform(1.0, 2.0, n)
    expo = rng.integers(-140, 140, n)
    sign = rng.choice([-1.0, 1.0], n)
    x = torch.from_numpy(sign * np.ldexp(mant, expo)).to(DEV)
    y = _rcp64(x)
    ref = 1.0 / x
    assert int(_ulps(y, ref).max()) <= 1
    # the solve feeds it pivots of a Jacobi-scaled matrix: values near 1 must be exact to 1 ulp too
    x2 = torch.from_numpy(rng.uniform(0.5, 2.0, n)).to(DEV)
    assert int(_ulps(_rcp64(x2), 1.0 / x2).max()) <= 1


def test_rcp64_mantissa_edges_and_range_boundaries():
    vals = []
    for e in list(range(-130, -120)) + list(range(-3, 4)) + list(range(120, 130)):
        for m in (1.0, np.nextafter(1.0, 2.0), 1.5, np.nextafter(2.0, 1.0), 1.0 + 2.0 ** -20, 2.0 - 2.0 ** -20):
            vals += [np.ldexp(m, e), -np.ldexp(m, e)]
    x = torch.tensor(vals, dtype=torch.float64, device=DEV)
    assert int(_ulps(_rcp64(x), 1.0 / x).max()) <= 1


def test_rcp64_special_values_take_exact_path():
    f64 = np.finfo(np.float64)
    vals = [0.0, -0.0, np.inf, -np.inf, f64.tiny, -f64.tiny, f64.tiny / 8, 5e-324, f64.max, -f64.max, 1e-300, 1e300,
            2.0 ** -127, 2.0 ** 127, 2.0 ** 200, 2.0 ** -200]
    x = torch.tensor(vals, dtype=torch.float64, device=DEV)
    y = _rcp64(x)
    ref = 1.0 / x
    assert torch.equal(y.view(torch.int64), ref.view(torch.int64))
    nan = _rcp64(torch.tensor([float("nan")], dtype=torch.float64, device=DEV))
    assert bool(torch.isnan(nan).all())


def test_narrow_equals_hardware_conversion():
    rng = np.random.default_rng(12)
    n = 1 << 22
    mant = rng.uniform(1.0, 2.0, n)
    expo = rng.integers(-160, 140, n)
    vals = np.ldexp(mant, expo) * rng.choice([-1.0, 1.0], n)
    # exact float midpoints (ties) and their neighbours, across the range
    f = rng.uniform(1.0, 2.0, 1 << 16).astype(np.float32)
    e = rng.integers(-125, 126, 1 << 16)
    base = np.ldexp(f.astype(np.float64), e)
    ulp = np.ldexp(2.0 ** -23, e)
    ties = np.concatenate([base + ulp / 2, base - ulp / 2, np.nextafter(base + ulp / 2, np.inf),
                           np.nextafter(base + ulp / 2, -np.inf)])
    fmax = float(np.finfo(np.float32).max)
    special = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 5e-324, 1e-40, -1e-40, 1.1754943508222875e-38,
                        fmax, -fmax, np.nextafter(fmax, np.inf), 3.4028235677973366e38, 1e39, 2.0 ** 127,
                        2.0 ** 128 - 2.0 ** 103, 1.0, -1.0])
    x = torch.from_numpy(np.concatenate([vals, ties, special])).to(DEV)
    _, got = _helpers(x)
    assert _same_bits(got, x.float())
