"""Generate nl_gen.cuh: the pointwise u.grad(u) Galerkin coupling for K0 = 4 and 6.

The wall-normal basis of Model Waleffe Flow (free-slip walls at y = +-1, b = pi/2):
    u, w : phi_0 = 1, phi_k = sin(k b y) for odd k, cos(k b y) for even k
    v    : psi_k = cos(k b y) for odd k, sin(k b y) for even k          (k >= 1)
The coupling projects u.grad(u) onto these modes with the normalised inner product
<f, g> = int f g dy / int f^2 dy.  Every triple-product integral is a trigonometric
polynomial integral; this script evaluates them exactly with the product-to-sum rule
(each basis function as a sum of complex exponentials) in rational arithmetic and writes
straight-line CUDA code with the coefficients as exact constants.

Structure of the generated code (per physical point; p holds the KK y-coefficients of
(u, v, w) in the order u_0..u_{K0-1}, v_1..v_{K0-1}, w_0..w_{K0-1}):
    nl_y_<K0>(p, nl)             nl  = projection of v d/dy (u, v, w)
    nl_xz_<K0><J>(p, px, pz, nl)  nl += projection of u d/dx f_J + w d/dz f_J  for field J
so the z pass can form the term field by field.  p and nl are indexable accessors (register
arrays or shared-memory views); each nl entry is read once and written once per call.

Usage: python gen_nl.py > nl_gen.cuh   (the output is committed; nvcc does not run this).
"""
from fractions import Fraction
import sys


def basis(kind, k):
    """Basis function as {freq: (re, im)}: coefficients of e^{i freq b y} (Fractions)."""
    is_cos = (k % 2 == 0) if kind == "phi" else (k % 2 == 1)
    if k == 0:
        return {0: (Fraction(1), Fraction(0))}
    if is_cos:   # cos = (e^{ik} + e^{-ik})/2
        return {k: (Fraction(1, 2), Fraction(0)), -k: (Fraction(1, 2), Fraction(0))}
    # sin = (e^{ik} - e^{-ik})/(2i) = -i/2 e^{ik} + i/2 e^{-ik}
    return {k: (Fraction(0), Fraction(-1, 2)), -k: (Fraction(0), Fraction(1, 2))}


def deriv(kind, k):
    """d/dy of a basis function in units of b: d/dy e^{i f b y} = i f b e^{i f b y}."""
    return {f: (-im * f, re * f) for f, (re, im) in basis(kind, k).items()}


def mul(a, b):
    out = {}
    for fa, (ra, ia) in a.items():
        for fb, (rb, ib) in b.items():
            f = fa + fb
            r0, i0 = out.get(f, (Fraction(0), Fraction(0)))
            out[f] = (r0 + ra * rb - ia * ib, i0 + ra * ib + ia * rb)
    return {f: v for f, v in out.items() if v != (0, 0)}


def integral(prod):
    """int_{-1}^{1} sum_f c_f e^{i f b y} dy.

    Even nonzero frequencies integrate to zero.  Odd frequencies would give the
    irrational 4 sin(f pi/2)/(f pi); by the parity of the basis they only occur in odd
    functions, where the f and -f coefficients cancel -- the script checks that.
    """
    total = prod.get(0, (Fraction(0), Fraction(0)))
    for f, (re, im) in prod.items():
        if f % 2 != 0 and f > 0:
            re2, im2 = prod.get(-f, (Fraction(0), Fraction(0)))
            if re + re2 != 0 or im + im2 != 0:
                raise ValueError("odd-frequency term survives: not a polynomial coefficient")
    if total[1] != 0:
        raise ValueError("complex projection")
    return 2 * total[0]


def norm(kind, k):
    p = mul(basis(kind, k), basis(kind, k))
    return integral(p)


def proj(kind_k, k, f1, f2):
    """<basis_k, f1 f2> for expansions f1, f2 in the {freq: (re, im)} form."""
    val = integral(mul(basis(kind_k, k), mul(f1, f2)))
    return val / norm(kind_k, k)


def tensors(K0):
    U = range(K0)
    V = range(1, K0)
    Gp = {(k, i, j): proj("phi", k, basis("phi", i), basis("phi", j)) for k in U for i in U for j in U}
    Gv = {(k, i, j): proj("psi", k, basis("phi", i), basis("psi", j)) for k in V for i in U for j in V}
    # H terms carry one factor b from the derivative
    Hp = {(k, i, j): proj("phi", k, basis("psi", i), deriv("phi", j)) for k in U for i in V for j in U}
    Hv = {(k, i, j): proj("psi", k, basis("psi", i), deriv("psi", j)) for k in V for i in V for j in V}
    return Gp, Gv, Hp, Hv


def frac_c(fr, times_beta=False):
    s = f"{float(fr)!r}"
    if times_beta:
        return f"T({s} * MWF_BETA)"
    return f"T({s})"


def emit(K0, out):
    KK = 3 * K0 - 1
    Gp, Gv, Hp, Hv = tensors(K0)
    ui = lambda a: a                    # u_a index in p
    vi = lambda a: K0 + a - 1           # v_a (a >= 1)
    wi = lambda a: 2 * K0 - 1 + a       # w_a
    out.append(f"// ---- K0 = {K0} (KK = {KK}) ----")
    # y terms: nl = v d/dy (u, v, w).  p, nl: indexable accessors (register arrays or views).
    out.append(f"template <typename T, typename P, typename NL> __device__ __forceinline__ void nl_y_{K0}(const P& p, NL&& nl) {{")
    body = []
    used = set()
    for comp, idx, H, kr in (("u", ui, Hp, range(K0)), ("v", vi, Hv, range(1, K0)), ("w", wi, Hp, range(K0))):
        src = {"u": ui, "v": vi, "w": wi}[comp]
        for k in kr:
            terms = []
            for (kk, i, j), c in sorted(H.items()):
                if kk != k or c == 0:
                    continue
                terms.append((c, vi(i), src(j)))
                used.update((vi(i), src(j)))
            dst = idx(k)
            if not terms:
                body.append(f"  nl[{dst}] = T(0);")
                continue
            c0, a0, b0 = terms[0]
            body.append(f"  {{ T a = ({frac_c(c0, True)} * p{a0}) * p{b0};")
            for c, a, b in terms[1:]:
                body.append(f"    a = fma({frac_c(c, True)} * p{a}, p{b}, a);")
            body.append(f"    nl[{dst}] = a; }}")
    for i in sorted(used):
        out.append(f"  const T p{i} = p[{i}];")
    out.extend(body)
    out.append("}")
    # x/z terms per field J: nl += u d/dx f_J + w d/dz f_J
    out.append(f"template <int J, typename T, typename P, typename NL> __device__ __forceinline__ void nl_xz_{K0}(const P& p, T px, T pz, NL&& nl) {{")
    out.append("  const T hx = T(0.5) * px, hz = T(0.5) * pz;")
    first = True
    for J in range(KK):
        if J < K0:
            comp, b, G, kr, dst = "u", J, Gp, range(K0), ui
        elif J < 2 * K0 - 1:
            comp, b, G, kr, dst = "v", J - K0 + 1, Gv, range(1, K0), vi
        else:
            comp, b, G, kr, dst = "w", J - (2 * K0 - 1), Gp, range(K0), wi
        out.append(f"  {'if' if first else 'else if'} constexpr (J == {J}) {{  // {comp}_{b}")
        first = False
        body = []
        used = set()
        for k in kr:
            stmts = []
            for (kk, i, j), c in sorted(G.items()):
                if kk != k or j != b or c == 0:
                    continue
                a_u, a_w = ui(i), wi(i)
                used.update((a_u, a_w))
                if c == 1:
                    stmts.append(f"a = fma(p{a_u}, px, a); a = fma(p{a_w}, pz, a);")
                elif c == -1:
                    stmts.append(f"a = fma(-p{a_u}, px, a); a = fma(-p{a_w}, pz, a);")
                elif c == Fraction(1, 2):
                    stmts.append(f"a = fma(p{a_u}, hx, a); a = fma(p{a_w}, hz, a);")
                elif c == Fraction(-1, 2):
                    stmts.append(f"a = fma(-p{a_u}, hx, a); a = fma(-p{a_w}, hz, a);")
                else:
                    raise ValueError(f"unexpected x/z coupling coefficient {c}")
            if stmts:
                d = dst(k)
                body.append(f"    {{ T a = nl[{d}]; " + " ".join(stmts) + f" nl[{d}] = a; }}")
        for i in sorted(used):
            out.append(f"    const T p{i} = p[{i}];")
        out.extend(body)
        out.append("  }")
    out.append("}")


def main():
    out = ["// Generated by gen_nl.py -- do not edit.  Galerkin coupling of Model Waleffe Flow.",
           "#pragma once",
           "#define MWF_BETA 1.5707963267948966",
           ""]
    for K0 in (4, 6):
        emit(K0, out)
        out.append("")
    sys.stdout.write("\n".join(out) + "\n")


if __name__ == "__main__":
    main()
