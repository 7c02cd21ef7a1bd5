"""Generate golden vectors for the mode-coupling functions from the reference's own expressions.

Run in a container where the reference tree is mounted, giving the root of that tree as the
first argument or in the environment variable MWF_REFERENCE.  The script reads the Fortran function bodies of program/modes.M4.f90 and
program/modes.M6.f90 as text, evaluates their ``ans(i) = ...`` expressions with numpy on
seeded random inputs, and writes ``udotgradu_M4.npz`` / ``udotgradu_M6.npz`` beside itself.
Nothing in the tests reads the reference at run time; they read these fixtures.

Fixture contents (arrays of shape (P, KK) unless noted):
    v, vx, vz        inputs (physical-space y-coefficients of u, du/dx, du/dz)
    udotgradu        reference ``udotgradu`` (explicit form for M4, helper form for M6)
    udotgradu2       M4 only: the reference's helper form ``udotgradu2``
    epos             (P,) reference ``epos`` (program/velocity.f90:115-126) built from the
                     reference's ``nluw``/``nlvv``
"""
import os
import re
import sys

import numpy as np

BETA = 3.1415926535897931 / 2.0


def parse_functions(path):
    """Return {name: (args, bases, result_base, [(index, expr)], calls)} for each function."""
    src = open(path).read().split("\n")
    funcs = {}
    cur = None
    for line in src:
        s = line.strip()
        m = re.match(r"function\s+(\w+)\s*\(([^)]*)\)\s*result\s*\(\s*(\w+)\s*\)", s, re.I)
        if m:
            cur = {"name": m.group(1), "args": [a.strip() for a in m.group(2).split(",")],
                   "bases": {}, "body": []}
            funcs[cur["name"]] = cur
            continue
        if cur is None:
            continue
        if re.match(r"end\s+function", s, re.I):
            cur = None
            continue
        if s.lower().startswith("double precision"):
            for nm, lo in re.findall(r"(\w+)\((\w+)(?::\w+)?\)", s.split("::")[1]):
                cur["bases"][nm] = 0 if lo == "0" else 1
            continue
        if re.match(r"ans\s*\(", s):
            cur["body"].append(s)
    return funcs


def to_python(expr, bases):
    expr = expr.replace("d_beta", "BETA")

    def sub(m):
        nm, idx = m.group(1), m.group(2)
        if ":" in idx:
            lo, hi = idx.split(":")
            return f"{nm}[..., ({lo})-{bases[nm]}:({hi})-{bases[nm]}+1]"
        return f"{nm}[..., ({idx})-{bases[nm]}]"

    return re.sub(r"\b(\w+)\(([^()]*)\)", lambda m: sub(m) if m.group(1) in bases else m.group(0),
                  expr)


def build(funcs, K0):
    KK = 3 * K0 - 1
    env = {"np": np, "BETA": BETA, "i_K0": K0, "i_KK": KK, "i_K1": K0 - 1}
    for name, f in funcs.items():
        bases = dict(f["bases"])
        rbase = bases.get("ans", 1)
        size = {"udotgradu": KK, "udotgradu2": KK}.get(name, K0 if rbase == 0 else K0 - 1)
        lines = [f"def {name}({', '.join(f['args'])}):",
                 f"    _a = {{}}"]
        for st in f["body"]:
            lhs, rhs = st.split("=", 1)
            lhs_idx = re.match(r"ans\s*\((.*)\)\s*$", lhs.strip()).group(1)
            rhs_py = to_python(rhs, {k: v for k, v in bases.items() if k != "ans"})
            rhs_py = re.sub(r"\b(nluw|nluyv|nluv|nlvvy|nlvv)\b", r"_f['\1']", rhs_py)
            lines.append(f"    _a[{lhs_idx!r}] = {rhs_py}")
        lines.append(f"    return _a")
        env.setdefault("_f", {})
        code = "\n".join(lines)
        exec(code, env)
        raw = env[name]

        def wrap(*args, _raw=raw, _rbase=rbase, _size=size, _K0=K0, _KK=KK):
            a = _raw(*args)
            shape = np.broadcast(*[x[..., 0] for x in args]).shape
            out = np.zeros(shape + (_size,))
            for key, val in a.items():
                if ":" in key:
                    lo, hi = key.split(":")
                    lo = eval(lo, {"i_K0": _K0, "i_KK": _KK})
                    hi = eval(hi, {"i_K0": _K0, "i_KK": _KK})
                    out[..., lo - _rbase:hi - _rbase + 1] = val
                else:
                    out[..., eval(key) - _rbase] = val
            return out

        env["_f"][name] = wrap
    return env["_f"]


def epos(f, K0, u):
    e = f["nluw"](u[..., :K0], u[..., :K0])[..., 0]
    e = e + f["nlvv"](u[..., K0:2 * K0 - 1])[..., 0]
    e = e + f["nluw"](u[..., 2 * K0 - 1:], u[..., 2 * K0 - 1:])[..., 0]
    return e


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("MWF_REFERENCE")
    if not ref:
        raise SystemExit("usage: make_golden.py <reference tree> (or set MWF_REFERENCE)")
    here = os.path.dirname(os.path.abspath(__file__))
    for K0, fn in ((4, "modes.M4.f90"), (6, "modes.M6.f90")):
        funcs = parse_functions(os.path.join(ref, "program", fn))
        f = build(funcs, K0)
        KK = 3 * K0 - 1
        rng = np.random.default_rng(1234 + K0)
        P = 64
        v, vx, vz = (rng.standard_normal((P, KK)) for _ in range(3))
        out = {"v": v, "vx": vx, "vz": vz,
               "udotgradu": f["udotgradu"](v, vx, vz),
               "epos": epos(f, K0, v)}
        if "udotgradu2" in f:
            out["udotgradu2"] = f["udotgradu2"](v, vx, vz)
        np.savez(os.path.join(here, f"udotgradu_M{K0}.npz"), **out)
        print(f"M{K0}: wrote {P} points, functions {sorted(f)}")


if __name__ == "__main__":
    main()
