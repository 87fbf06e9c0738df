"""Generates csrc/rhs_algebra_gen.cuh from bssn_spec.py.

FP64 arithmetic, not memory, bounds the right-hand side on GB300, so the
pointwise algebra is emitted in a form with fewer FP64 instructions than the
reference's Maple-generated monomial sums:
  * every temporary of the spec is expanded to a polynomial in its inputs
    (1/r is an independent symbol), collected by powers of r and 1/r, and each
    coefficient is put in multivariate Horner form with the variables ordered
    by how many monomials they occur in (the cheapest of a few orderings under
    an FMA-aware cost model is kept);
  * common subexpressions across all temporaries are then shared;
  * the result is printed as straight-line CUDA with products written so
    that nvcc contracts the additions into FMAs.
Every rewritten temporary is checked to be algebraically identical to the
spec expression before it is emitted.

    python gen_rhs.py            # writes ../rhs_algebra_gen.cuh
"""
import os
import sys

import sympy as sp
from sympy.printing.c import C99CodePrinter

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import bssn_spec  # noqa: E402

sys.setrecursionlimit(100000)


def cost(e):
    """FP64 instructions of ``e`` with a*b+c contracted to one FMA."""
    if e.is_Symbol or e.is_Number:
        return 0
    if e.is_Pow:
        b, k = e.args
        k = int(k)
        return cost(b) + {1: 0, 2: 1, 3: 2, 4: 2, 5: 3, 6: 3, 7: 4, 8: 3}.get(k, 4)
    if e.is_Mul:
        nums = [a for a in e.args if a.is_Number]
        others = [a for a in e.args if not a.is_Number]
        c = sum(cost(a) for a in others) + max(len(others) - 1, 0)
        if nums and abs(nums[0]) != 1:
            c += 1
        return c
    if e.is_Add:
        c = sum(cost(a) for a in e.args) + len(e.args) - 1
        fus = sum(1 for a in e.args if a.is_Mul and (len(a.args) >= 2))
        return c - min(fus, len(e.args) - 1)
    return sum(cost(a) for a in e.args)


METRIC = ("gA", "gB", "gC", "gH", "r", "ir", "glam", "lam", "ipsi4")


def _horner(poly_expr, gens):
    try:
        return sp.polys.polyfuncs.horner(poly_expr, *gens)
    except Exception:
        return poly_expr


def horner_by_frequency(poly_expr, exclude=()):
    """Cheapest multivariate Horner form over a few variable orderings:
    by frequency, data (derivatives, curvature) first, metric first."""
    if not poly_expr.free_symbols:
        return poly_expr
    terms = sp.Add.make_args(poly_expr)
    freq = {}
    for t in terms:
        for s in t.free_symbols:
            freq[s] = freq.get(s, 0) + 1
    gens = sorted((s for s in freq if s not in exclude), key=lambda s: (-freq[s], s.name))
    if not gens:
        return poly_expr
    data = [g for g in gens if g.name not in METRIC]
    metric = [g for g in gens if g.name in METRIC]
    cands = [_horner(poly_expr, gens), _horner(poly_expr, data + metric), _horner(poly_expr, metric + data),
             _horner(poly_expr, list(reversed(gens)))]
    return min(cands, key=cost)


def optimise(expr, r, ir):
    """Pick the cheapest of a few exact rewritings of ``expr``."""
    cands = [expr]
    ex = sp.expand(expr)
    cands.append(ex)
    if len(sp.Add.make_args(ex)) > 2:
        cands.append(horner_by_frequency(ex))
        # collect by powers of r and 1/r, Horner inside each coefficient
        parts = sp.collect(ex, [r, ir], evaluate=False)
        acc = 0
        for k, v in parts.items():
            acc += k * horner_by_frequency(sp.expand(v))
        cands.append(acc)
        # Horner in r on the outside
        try:
            P = sp.Poly(ex, r)
            coeffs = [horner_by_frequency(sp.expand(c)) for c in P.all_coeffs()]
            h = 0
            for c in coeffs:
                h = h * r + c
            cands.append(h)
        except sp.PolynomialError:
            pass
    best = min(cands, key=cost)
    if sp.expand(best - expr) != 0:
        raise AssertionError("rewriting changed the value")
    return best


class CudaPrinter(C99CodePrinter):
    def _print_Pow(self, expr):
        b, k = expr.args
        k = int(k)
        base = self.parenthesize(b, 100)
        if k == 2:
            return "(%s * %s)" % (base, base)
        if k == 3:
            return "(%s * %s * %s)" % (base, base, base)
        if k == 4:
            return "((%s * %s) * (%s * %s))" % (base, base, base, base)
        raise ValueError("power %d" % k)

    def _print_Rational(self, expr):
        return "%s" % repr(float(expr.p) / float(expr.q)) if expr.q != 1 else "%d.0" % expr.p

    def _print_Integer(self, expr):
        return "%d.0" % int(expr)

    def _print_Float(self, expr):
        return repr(float(expr))


def generate(outputs, fname):
    syms = {n: sp.Symbol(n) for n in bssn_spec.INPUTS}

    class X:
        pass
    x = X()
    for n, s in syms.items():
        setattr(x, n, s)
    lets = []

    def let(name, expr):
        s = sp.Symbol("t_" + name)
        lets.append((s, expr))
        return s

    outs = bssn_spec.algebra(x, let)
    # dead-code elimination
    need = set()
    for o in outputs:
        need |= outs[o].free_symbols
    letmap = dict(lets)
    changed = True
    while changed:
        changed = False
        for s, e in lets:
            if s in need:
                new = e.free_symbols - need
                if new:
                    need |= new
                    changed = True
    stmts = [(s, e) for s, e in lets if s in need]
    r, ir = syms["r"], syms["ir"]
    before = sum(cost(e) for _, e in stmts) + sum(cost(outs[o]) for o in outputs)
    opt = [(s, optimise(e, r, ir)) for s, e in stmts]
    oexp = [optimise(outs[o], r, ir) for o in outputs]
    after = sum(cost(e) for _, e in opt) + sum(cost(e) for e in oexp)
    # common subexpressions across everything
    allexprs = [e for _, e in opt] + oexp
    repl, reduced = sp.cse(allexprs, symbols=sp.numbered_symbols("c"), optimizations="basic")
    after_cse = sum(cost(e) for _, e in repl) + sum(cost(e) for e in reduced)
    pr = CudaPrinter()
    # Emission order: depth-first from each output, every definition placed
    # just before its first use, so that temporaries live briefly (the
    # register pressure of the straight-line code follows the text order).
    defs = dict(list(repl) + [(s, e) for (s, _), e in zip(opt, reduced[:len(opt)])])
    inputs = set(syms.values())
    emitted = set()
    lines = []

    def emit(sym):
        if sym in emitted or sym in inputs:
            return
        e = defs[sym]
        for dep in sorted(e.free_symbols, key=lambda x: x.name):
            if dep in defs:
                emit(dep)
        lines.append("    const double %s = %s;" % (sym, pr.doprint(e)))
        emitted.add(sym)

    for o, e in zip(outputs, reduced[len(opt):]):
        for dep in sorted(e.free_symbols, key=lambda x: x.name):
            if dep in defs:
                emit(dep)
        lines.append("    o.%s = %s;" % (o, pr.doprint(e)))
    return lines, before, after, after_cse


HEADER = """// Generated by csrc/gen/gen_rhs.py from csrc/gen/bssn_spec.py -- do not edit.
//
// Pointwise BSSN algebra (lapse Laplacian, Ricci tensor and scalar,
// traceless-curvature contractions, divergence of KT, geometric sources and
// constraints) in an FP64-instruction-minimised form.  Estimated FP64
// instructions per point (FMA-contracted):
//   sources : %(src_before)d as written in the spec -> %(src_after)d
//   analysis: %(ana_before)d as written in the spec -> %(ana_after)d
#pragma once

namespace ollin {

struct AlgIn {
    double %(inputs)s;
};

struct SrcOut { double %(src_out)s; };
struct AnaOut { double %(ana_out)s; };

__device__ __forceinline__ void bssn_sources(const AlgIn& in, SrcOut& o) {
%(unpack)s
%(src_body)s
}

__device__ __forceinline__ void bssn_analysis(const AlgIn& in, AnaOut& o) {
%(unpack)s
%(ana_body)s
}

}  // namespace ollin
"""


def main():
    src_lines, sb, sa, sc = generate(bssn_spec.SOURCE_OUTPUTS, "sources")
    ana_lines, ab, aa, ac = generate(bssn_spec.ANALYSIS_OUTPUTS, "analysis")
    unpack = "\n".join("    const double %s = in.%s;" % (n, n) for n in bssn_spec.INPUTS)
    text = HEADER % dict(src_before=sb, src_after=sc, ana_before=ab, ana_after=ac,
                         inputs=", ".join(bssn_spec.INPUTS),
                         src_out=", ".join(bssn_spec.SOURCE_OUTPUTS),
                         ana_out=", ".join(bssn_spec.ANALYSIS_OUTPUTS),
                         unpack=unpack, src_body="\n".join(src_lines), ana_body="\n".join(ana_lines))
    out = os.path.join(os.path.dirname(HERE), "rhs_algebra_gen.cuh")
    with open(out, "w") as f:
        f.write(text)
    print("sources: %d -> %d (after horner) -> %d (after cse)" % (sb, sa, sc))
    print("analysis: %d -> %d -> %d" % (ab, aa, ac))
    print("wrote", out)


if __name__ == "__main__":
    main()
