"""Generated model code against an independent sympy.lambdify evaluation.

The generated struct is compiled on the host (through the oracle build, which
includes it verbatim) and its m, dm/dp and packed d2m/dp2 are compared with
numpy evaluations of the symbolic derivatives, which share none of the CSE or
printing. Derivative list and packing follow pycompute/sym/util.py:100-112.
"""
import ctypes
import os
import subprocess

import numpy as np
import pytest

from pycompute_gb300 import codegen, synth

HOST_MAIN = r'''
#include <cmath>
#include "lm_oracle.hpp"
#include "model.h"
extern "C" void eval_all(int P, int C, int n, const double* p, const double* c, double* out) {
  const int H = P * (P + 1) / 2;
  for (int v = 0; v < n; ++v) {
    double m, J[8], Hm[36];
    MODEL::all<double>(p + v * P, c + v * (C > 0 ? C : 1), m, J, Hm);
    double* o = out + v * (1 + P + H);
    o[0] = m;
    for (int k = 0; k < P; ++k) o[1 + k] = J[k];
    for (int k = 0; k < H; ++k) o[1 + P + k] = Hm[k];
    double mv = MODEL::value<double>(p + v * P, c + v * (C > 0 ? C : 1));
    o[0] = (mv == m || std::fabs(mv - m) <= 1e-12 * std::fabs(m)) ? m : NAN;
  }
}
'''

CASES = [
    (synth.IVIM_EXPR, synth.IVIM_PARS, ["b"], [(500, 1500), (0.05, 0.35), (5e-3, 5e-2), (5e-4, 2.5e-3)], [(0, 1000)]),
    ("S0*sin(a)*(1-exp(-15/T1))/(1-cos(a)*exp(-15/T1))", ["S0", "T1"], ["a"], [(500, 1500), (300, 3000)],
     [(0.03, 0.5)]),
    ("S0*exp(-TE*R2s/1000)+c", ["S0", "R2s", "c"], ["TE"], [(500, 1500), (10, 200), (0, 50)], [(2, 40)]),
    ("S0*(f*exp(-TE/T2s)+(1-f)*exp(-TE/T2l))+c", ["S0", "f", "T2s", "T2l", "c"], ["TE"],
     [(500, 1500), (0.1, 0.5), (10, 40), (60, 300), (0, 50)], [(10, 320)]),
    ("A*sqrt(x)*log(B+x) + A**3/(B*x) + tanh(B*x)**2 + x**(B/4)", ["A", "B"], ["x"], [(0.5, 2), (0.5, 2)], [(0.5, 3)]),
    ("a*x + b", ["a", "b"], ["x"], [(-2, 2), (-2, 2)], [(-3, 3)]),
]


def _compile(gm, tmp_path):
    from oracle.build import HERE as ORACLE
    d = tmp_path / gm.struct_name
    d.mkdir()
    (d / "model.h").write_text(gm.source)
    (d / "main.cpp").write_text(HOST_MAIN)
    so = d / "libm.so"
    r = subprocess.run(["g++", "-O1", "-std=c++17", "-shared", "-fPIC", f"-I{ORACLE}", f"-I{d}",
                        f"-DMODEL={gm.struct_name}", str(d / "main.cpp"), "-o", str(so)], capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stderr
    return ctypes.CDLL(str(so))


@pytest.mark.parametrize("case", CASES, ids=lambda c: c[0][:30])
def test_generated_derivatives_match_sympy(case, tmp_path):
    expr, pars, consts, prange, crange = case
    gm = codegen.generate(expr, pars, consts)
    lib = _compile(gm, tmp_path)
    rng = np.random.default_rng(3)
    n = 257
    P, C, H = gm.P, gm.C, gm.H
    p = np.stack([rng.uniform(lo, hi, n) for lo, hi in prange], 1)
    c = np.stack([rng.uniform(lo, hi, n) for lo, hi in crange], 1) if C else np.zeros((n, 1))
    out = np.zeros((n, 1 + P + H))
    lib.eval_all.argtypes = [ctypes.c_int] * 3 + [ctypes.c_void_p] * 3
    lib.eval_all(P, C, n, p.ctypes.data, c.ctypes.data, out.ctypes.data)
    assert np.all(np.isfinite(out[:, 0])), "value() and all() disagree on m"
    fns = codegen.numpy_functions(expr, pars, consts)
    args = [p[:, k] for k in range(P)] + [c[:, k] for k in range(C)]
    for j, fn in enumerate(fns):
        want = np.broadcast_to(np.asarray(fn(*args), dtype=np.float64), (n,))
        np.testing.assert_allclose(out[:, j], want, rtol=1e-11, atol=1e-11 * np.abs(want).max() + 1e-300)
    # structurally-zero masks agree with the symbolic derivatives
    for k, nz in enumerate(gm.hnz):
        if not nz:
            assert np.all(out[:, 1 + P + k] == 0)


def test_ivim_masks_and_hash():
    gm = codegen.generate(synth.IVIM_EXPR, synth.IVIM_PARS, ["b"])
    # d2m/dS0^2, d2m/dD*dS0... : the reference snapshot prints 0.0f*res at hes[0], hes[2], hes[8]
    assert gm.hnz == [False, True, False, True, True, True, True, True, False, True]
    assert gm.hash == "f7def86f0a03"  # id of the reference's generated IVIM kernels
    assert gm.nexp == 2


@pytest.mark.parametrize("bad", [
    ("S0*exp(-b*D)", ["S0", "D"], ["b", "D"]),      # duplicate name
    ("S0*exp(-b*D)*Q", ["S0", "D"], ["b"]),         # undeclared symbol
    ("S0*(", ["S0"], []),                          # syntax
    ("Max(S0, b)", ["S0"], ["b"]),                 # non-smooth
    ("x", ["a b"], []),                            # not an identifier
])
def test_codegen_rejects(bad):
    with pytest.raises(ValueError):
        codegen.generate(*bad)
