"""Device arithmetic helpers of the FP64 solve checked against correctly
rounded results: the Newton-Raphson reciprocal must stay within 1 ulp of
1/x (IEEE division on the GPU) everywhere, and return exactly 1/x for the
inputs it hands to the hardware reciprocal (zero, infinities, NaN,
subnormals and exponents outside the float range)."""
import ctypes

import numpy as np
import pytest
import torch

from pycompute_gb300 import _lib

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


def _rcp64(x: torch.Tensor) -> torch.Tensor:
    y = torch.empty_like(x)
    rc = _lib.lib().pcgb_rcp64(ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(y.data_ptr()), x.numel(),
                               ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    _lib.check("pcgb_rcp64", rc)
    torch.cuda.synchronize()
    return y


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
