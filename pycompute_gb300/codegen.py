"""Symbolic model -> straight-line C++ model code.

The reference turns a model expression into CUDA C with symengine: it
differentiates ``[m, dm/dp_k, d2m/dp_i dp_j (j <= i)]``, runs a common
subexpression pass over the whole list and prints the result
(``pycompute/sym/util.py:100-112`` for the derivative list,
``pycompute/sym/util.py:37-55`` for the float printer,
``pycompute/cuda/lsqnonlin.py:280-339`` for the renaming and substitution into
``pars[k]`` / ``consts[...]``).

This module keeps that recipe (same derivative list, same packing order of the
second derivatives, a CSE pass over everything) but emits a single model
*struct* instead of a templated kernel string:

* ``value(p, c)``       -> m(p; c), CSE over m alone (reference ``res``,
  ``sym/util.py:64-67``), used for the trial cost;
* ``all(p, c, m, J, H)`` -> m, the P first derivatives and the P(P+1)/2
  packed second derivatives (row i, column j <= i), CSE over all of them;
* ``HNZ`` / ``JNZ`` -> compile-time masks of the entries that are not
  structurally zero, so the LM kernel drops ``0 * res`` terms at compile time.

The struct is templated on the arithmetic type ``T`` and uses the math
wrappers ``pcgb_exp`` etc., which the including translation unit defines for
its target (``__device__`` overloads in the CUDA kernel source, ``std::``
overloads in the host oracle). One generated text therefore serves the GPU
fitter and the CPU oracle in both float and double.
"""
from __future__ import annotations

import functools
import hashlib
import re
from dataclasses import dataclass, field

import sympy as sp

_FUNCS = {
    sp.exp: "pcgb_exp",
    sp.log: "pcgb_log",
    sp.sin: "pcgb_sin",
    sp.cos: "pcgb_cos",
    sp.tan: "pcgb_tan",
    sp.asin: "pcgb_asin",
    sp.acos: "pcgb_acos",
    sp.atan: "pcgb_atan",
    sp.sinh: "pcgb_sinh",
    sp.cosh: "pcgb_cosh",
    sp.tanh: "pcgb_tanh",
    sp.Abs: "pcgb_abs",
    sp.erf: "pcgb_erf",
}

_IDENT = re.compile(r"^[A-Za-z_][A-Za-z0-9_]*$")


def expr_hash(expr: str, length: int = 12) -> str:
    """12-character model id: md5 of the expression text, characters [1:13].

    Same recipe as the reference (``pycompute/sym/util.py:61-62``) so kernel
    ids read the same (``..._4_1_21_f_f7def86f0a03`` for the IVIM model).
    """
    return hashlib.md5(expr.encode()).hexdigest()[1 : length + 1]


class _Printer:
    """Prints a sympy expression as C++ over the template type ``T``."""

    def __init__(self, names: dict[sp.Symbol, str]):
        self.names = names

    def lit(self, v) -> str:
        if isinstance(v, sp.Integer) or (isinstance(v, int)):
            return f"T({int(v)})"
        if isinstance(v, sp.Rational):
            return f"T({int(v.p)}.0 / {int(v.q)}.0)"
        return f"T({float(v)!r})"

    def __call__(self, e) -> str:
        return self.p(e)

    def p(self, e) -> str:  # noqa: C901 - a printer is a switch
        if e.is_Symbol:
            return self.names[e]
        if e.is_Number:
            if e is sp.nan or e in (sp.oo, -sp.oo, sp.zoo):
                raise ValueError(f"model produced a non-finite constant: {e}")
            return self.lit(e)
        if e is sp.pi:
            return self.lit(sp.Float(sp.pi, 20))
        if e is sp.E:
            return self.lit(sp.Float(sp.E, 20))
        if e.is_Add:
            terms = list(e.as_ordered_terms())
            out = self.p(terms[0])
            for t in terms[1:]:
                coeff, rest = t.as_coeff_Mul()
                if coeff.is_Number and coeff < 0:
                    out += " - " + self._factor(-t)
                else:
                    out += " + " + self._factor(t)
            return "(" + out + ")"
        if e.is_Mul:
            coeff, rest = e.as_coeff_Mul()
            if coeff == -1:
                return "(-" + self._factor(rest) + ")"
            num, den = [], []
            for f in e.as_ordered_factors():
                if f.is_Pow and f.exp.is_Number and f.exp < 0:
                    den.append(sp.Pow(f.base, -f.exp))
                elif f.is_Rational and not f.is_Integer and f.p == 1:
                    den.append(sp.Integer(f.q))
                else:
                    num.append(f)
            s = "*".join(self._factor(f) for f in num) if num else "T(1)"
            if den:
                d = "*".join(self._factor(f) for f in den)
                s = f"({s}/({d}))" if len(den) > 1 else f"({s}/{d})"
            return s
        if e.is_Pow:
            b, x = e.base, e.exp
            if x.is_Integer:
                n = int(x)
                if n == 0:
                    return "T(1)"
                if 0 < n <= 8:
                    bb = self._factor(b)
                    return "(" + "*".join([bb] * n) + ")"
                if -8 <= n < 0:
                    bb = self._factor(b)
                    return "(T(1)/(" + "*".join([bb] * (-n)) + "))"
            if x == sp.Rational(1, 2):
                return f"pcgb_sqrt({self.p(b)})"
            if x == sp.Rational(-1, 2):
                return f"(T(1)/pcgb_sqrt({self.p(b)}))"
            if b is sp.E:
                return f"pcgb_exp({self.p(x)})"
            return f"pcgb_pow({self.p(b)}, {self.p(x)})"
        if e.func in _FUNCS:
            args = ", ".join(self.p(a) for a in e.args)
            return f"{_FUNCS[e.func]}({args})"
        if isinstance(e, sp.Piecewise) or e.func in (sp.Max, sp.Min, sp.sign, sp.Heaviside):
            raise ValueError(f"non-smooth function {e.func} is not supported in a fitted model")
        raise ValueError(f"cannot print {e.func} in a model")

    def _factor(self, e) -> str:
        s = self.p(e)
        return s


@dataclass
class GeneratedModel:
    """A model expression after differentiation, CSE and printing."""

    expr: str
    pars: list[str]
    consts: list[str]
    struct_name: str
    source: str
    jnz: list[bool]
    hnz: list[bool]
    nexp: int = 0
    meta: dict = field(default_factory=dict)

    @property
    def P(self) -> int:
        return len(self.pars)

    @property
    def C(self) -> int:
        return len(self.consts)

    @property
    def H(self) -> int:
        return self.P * (self.P + 1) // 2

    @property
    def hash(self) -> str:
        return expr_hash(self.expr, 12)


def _symbols_for(expr: str, pars: list[str], consts: list[str]):
    for n in list(pars) + list(consts):
        if not _IDENT.match(n):
            raise ValueError(f"parameter/constant name {n!r} is not an identifier")
    if len(set(pars) | set(consts)) != len(pars) + len(consts):
        raise ValueError("parameter and constant names must be distinct")
    local = {n: sp.Symbol(n, real=True) for n in list(pars) + list(consts)}
    try:
        e = sp.sympify(expr, locals=local)
    except (sp.SympifyError, SyntaxError, TypeError) as exc:
        raise ValueError(f"cannot parse model expression {expr!r}: {exc}") from exc
    free = {s.name for s in e.free_symbols}
    unknown = free - set(local)
    if unknown:
        raise ValueError(f"model expression uses undeclared symbols {sorted(unknown)}")
    psyms = [sp.Symbol(f"p__{k}", real=True) for k in range(len(pars))]
    csyms = [sp.Symbol(f"c__{k}", real=True) for k in range(len(consts))]
    sub = {local[n]: psyms[k] for k, n in enumerate(pars)}
    sub.update({local[n]: csyms[k] for k, n in enumerate(consts)})
    e = e.xreplace(sub)
    names = {s: f"p[{k}]" for k, s in enumerate(psyms)}
    names.update({s: f"c[{k}]" for k, s in enumerate(csyms)})
    return e, psyms, csyms, names


def derivative_list(e, psyms):
    """[m, dm/dp_0..dm/dp_{P-1}, d2m/dp_i dp_j for i in 0..P-1, j in 0..i].

    Same list and order as ``res_jac_hes`` (``pycompute/sym/util.py:100-112``).
    """
    exprs = [e]
    for s in psyms:
        exprs.append(sp.diff(e, s))
    for i in range(len(psyms)):
        for j in range(i + 1):
            exprs.append(sp.diff(e, psyms[i], psyms[j]))
    return exprs


def _emit_block(exprs, names, prefix, indent="    "):
    """CSE a list of expressions; return (lines, printed reduced exprs)."""
    syms = sp.numbered_symbols(prefix)
    repl, reduced = sp.cse(exprs, symbols=syms, optimizations="basic")
    names = dict(names)
    lines = []
    pr = _Printer(names)
    for s, v in repl:
        cname = s.name
        names[s] = cname
        pr = _Printer(names)
        lines.append(f"{indent}const T {cname} = {pr(v)};")
    return lines, [pr(r) for r in reduced], repl


def generate(expr: str, pars: list[str], consts: list[str], struct_name: str | None = None) -> GeneratedModel:
    """Differentiate, CSE and print one model expression (memoised: sympy
    differentiation and CSE take tens of milliseconds per model)."""
    return _generate_cached(expr, tuple(pars), tuple(consts), struct_name)


@functools.lru_cache(maxsize=256)
def _generate_cached(expr: str, pars: tuple, consts: tuple, struct_name: str | None) -> GeneratedModel:
    pars, consts = list(pars), list(consts)
    if not pars:
        raise ValueError("a model needs at least one parameter")
    if len(pars) > 8:
        raise ValueError("at most 8 parameters are supported")
    e, psyms, csyms, names = _symbols_for(expr, pars, consts)
    P = len(pars)
    H = P * (P + 1) // 2
    struct_name = struct_name or f"Model_{expr_hash(expr)}"
    dl = derivative_list(e, psyms)
    jnz = [not (sp.simplify(d) == 0) for d in dl[1 : 1 + P]]
    hnz = [not (sp.simplify(d) == 0) for d in dl[1 + P :]]

    vlines, (vexpr,), _ = _emit_block([e], names, "v")
    live = [dl[0]] + [d for d, nz in zip(dl[1 : 1 + P], jnz) if nz] + [d for d, nz in zip(dl[1 + P :], hnz) if nz]
    alines, aexprs, arepl = _emit_block(live, names, "x")
    it = iter(aexprs)
    m_s = next(it)
    jl, hl = [], []
    for k in range(P):
        jl.append(f"    J[{k}] = {next(it)};" if jnz[k] else f"    J[{k}] = T(0);")
    for k in range(H):
        hl.append(f"    H[{k}] = {next(it)};" if hnz[k] else f"    H[{k}] = T(0);")
    nexp = sum(1 for _, v in arepl for _f in sp.preorder_traversal(v) if isinstance(_f, sp.exp))

    def bools(v):
        return ", ".join("true" if b else "false" for b in v)

    src = f"""// model: {expr}
// parameters: {', '.join(pars)}; constants per sample: {', '.join(consts) if consts else '(none)'}
struct {struct_name} {{
  static constexpr int P = {P};
  static constexpr int C = {len(consts)};
  static constexpr int H = {H};
  PCGB_HD static constexpr bool jnz(int k) {{ constexpr bool v[{P}] = {{{bools(jnz)}}}; return v[k]; }}
  PCGB_HD static constexpr bool hnz(int k) {{ constexpr bool v[{H}] = {{{bools(hnz)}}}; return v[k]; }}

  template <typename T>
  PCGB_HD static T value(const T* p, const T* c) {{
    (void)c;
{chr(10).join(vlines)}
    return {vexpr};
  }}

  template <typename T>
  PCGB_HD static void all(const T* p, const T* c, T& m, T* J, T* H) {{
    (void)c;
{chr(10).join(alines)}
    m = {m_s};
{chr(10).join(jl)}
{chr(10).join(hl)}
  }}
}};
"""
    return GeneratedModel(expr=expr, pars=list(pars), consts=list(consts), struct_name=struct_name,
                          source=src, jnz=jnz, hnz=hnz, nexp=nexp)


def numpy_functions(expr: str, pars: list[str], consts: list[str]):
    """Independent numpy evaluators of m, J and packed H via ``sympy.lambdify``.

    Used to check the printed code: it shares the symbolic derivatives but none
    of the CSE or printing.
    """
    e, psyms, csyms, _ = _symbols_for(expr, pars, consts)
    dl = derivative_list(e, psyms)
    args = psyms + csyms
    return [sp.lambdify(args, d, modules="numpy") for d in dl]
