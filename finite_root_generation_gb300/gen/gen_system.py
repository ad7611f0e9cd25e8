"""Generate the CSE'd straight-line evaluation of the Stephenson II loop-closure
system, its Jacobian nonzeros and its t-derivative, for the CUDA tracker.

The system is FSYS of the reference (htpykinematics.cu:8-126): for each j = 1..7 three
equations (rows j-1, j+6, j+13) in the 22 homogeneous unknowns
Z = [A,B,C,D,F,G,H, Ac..Hc, U1..U7, Z0] and the 30 parameters
q = [P0..P7, Pc0..Pc7, Q1..Q7, Qc1..Qc7]. Equation j involves only U_j among the U's, so
one "group" evaluation per j yields F (3 values), dF/dZ (8 + 6 + 16 nonzeros, the
sparsity of JVAR, htpykinematics.cu:129-1129) and dF/dt = dF/dq . dq/dt (the t
column of JH, htpysupport.cu:113-121) in one pass.

The equations are restated here symbolically and differentiated by sympy; the
reciprocals 1/U, 1/(F-B), 1/(H-C), 1/(Fc-Bc), 1/(Hc-Cc) are carried as symbols with
their own chain rule so that the emitted code has no division. Quantities that do
not depend on j are hoisted into a per-point "shared" block.

Output: ../csrc/frg_system_gen.cuh (committed; regenerate with
``python finite_root_generation_gb300/gen/gen_system.py``). The script also prints
the operation counts used for the roofline's algorithmic FLOPs per evaluation.
"""
from __future__ import annotations

import os

import sympy as sp

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "..", "csrc", "frg_system_gen.cuh")

# ---- symbols -----------------------------------------------------------------
A, B, C, D, F, G, H = sp.symbols("A B C D F G H")
Ac, Bc, Cc, Dc, Fc, Gc, Hc = sp.symbols("Ac Bc Cc Dc Fc Gc Hc")
U, z = sp.symbols("U z")
P0, Pc0, Pj, Pcj, Qj, Qcj = sp.symbols("P0 Pc0 Pj Pcj Qj Qcj")
dP0, dPc0, dPj, dPcj, dQj, dQcj = sp.symbols("dP0 dPc0 dPj dPcj dQj dQcj")
# reciprocals carried as symbols
iU, e1, e2, ec1, ec2 = sp.symbols("iU e1 e2 ec1 ec2")

VARS = [A, B, C, D, F, G, H, Ac, Bc, Cc, Dc, Fc, Gc, Hc, U, z]
PARAMS = [(P0, dP0), (Pc0, dPc0), (Pj, dPj), (Pcj, dPcj), (Qj, dQj), (Qcj, dQcj)]
# d(reciprocal)/d(var) rules
RECIP = {
    iU: {U: -iU**2},
    e1: {F: -e1**2, B: e1**2},
    e2: {H: -e2**2, C: e2**2},
    ec1: {Fc: -ec1**2, Bc: ec1**2},
    ec2: {Hc: -ec2**2, Cc: ec2**2},
}


def total_diff(expr, v):
    d = sp.diff(expr, v)
    for r, rules in RECIP.items():
        if v in rules:
            d += sp.diff(expr, r) * rules[v]
    return sp.expand(d) if False else d


# ---- the three equation families (htpykinematics.cu:36-122) -------------------
p, pc, p0, pc0 = Pj * z, Pcj * z, P0 * z, Pc0 * z
a, ac = C - A, Cc - Ac
S = Pj * Pcj + P0 * Pc0
m = pc - Ac - ac * Qcj
n = p - A - a * Qj
fI = (-S * z**3 + ac * Qcj * z * (p - A) + Ac * z * (a + p) + Hc * z * (p0 - C) + a * Qj * z * (pc - Ac)
      + A * z * (ac + pc) + U * (p0 - H) * m + H * z * (pc0 - Cc) + z**2 * n * (pc0 - Hc) * iU)
fII = (z**2 * (Bc * Pj + B * Pcj) - S * z**3 + Fc * z * (p0 - B) + U * (p0 - F) * (pc - Bc)
       + F * z * (pc0 - Bc) + z**2 * (p - B) * (pc0 - Fc) * iU)
X = (A - B) + a * Qj - (D - B) * (p - B) * e1 + (G - C) * n * e2
Xc = (Ac - Bc) + ac * Qcj - (Dc - Bc) * (pc - Bc) * ec1 + (Gc - Cc) * m * ec2
W = -(D - B) * (p0 - F) * e1 + (G - C) * (p0 - H) * e2
Wc = -(Dc - Bc) * (pc0 - Fc) * ec1 + (Gc - Cc) * (pc0 - Hc) * ec2
fIII = (G - D) * (Gc - Dc) * z - z * X * Xc + U * W * Xc + z**2 * X * Wc * iU - z * W * Wc

FAMILIES = [
    ("I", fI, [A, C, H, Ac, Cc, Hc, U, z]),
    ("II", fII, [B, F, Bc, Fc, U, z]),
    ("III", fIII, [A, B, C, D, F, G, H, Ac, Bc, Cc, Dc, Fc, Gc, Hc, U, z]),
]
# column of each variable in Z (U -> 13 + j)
COL = {A: 0, B: 1, C: 2, D: 3, F: 4, G: 5, H: 6, Ac: 7, Bc: 8, Cc: 9, Dc: 10, Fc: 11, Gc: 12, Hc: 13,
       U: -1, z: 21}

# j-independent inputs the group code reads from the shared block
SHARED = {
    "z2": z**2, "z3": z**3, "p0": P0 * z, "pc0": Pc0 * z, "S0": P0 * Pc0,
    "k1": D - B, "k2": G - C, "kc1": Dc - Bc, "kc2": Gc - Cc,
    "GD": (G - D) * (Gc - Dc),
}


def outputs():
    outs = []
    names = []
    for fam, f, vars_ in FAMILIES:
        outs.append(f)
        names.append(("f", fam, None))
        for v in vars_:
            outs.append(total_diff(f, v))
            names.append(("j", fam, v))
        tcol = sum(total_diff(f, prm) * dprm for prm, dprm in PARAMS)
        outs.append(tcol)
        names.append(("t", fam, None))
    return names, outs


def count_ops(exprs):
    """(complex muls, complex adds, scalar*complex) of straight-line code."""
    cm = ca = sm = 0
    for e in exprs:
        for node in sp.preorder_traversal(e):
            if isinstance(node, sp.Mul):
                num = [a for a in node.args if a.is_Number]
                sym = [a for a in node.args if not a.is_Number]
                k = len(sym)
                cm += max(k - 1, 0)
                if num and num[0] not in (1, -1):
                    sm += 1
            elif isinstance(node, sp.Add):
                ca += len(node.args) - 1
            elif isinstance(node, sp.Pow):
                ex = int(node.exp)
                cm += abs(ex) - 1
    return cm, ca, sm


class Printer:
    def __init__(self):
        self.lines = []

    def expr(self, e) -> str:
        if e.is_Symbol:
            return e.name
        if e.is_Number:
            return f"cx<T>(T({float(e)!r}))"
        if isinstance(e, sp.Pow):
            base = self.expr(e.args[0])
            ex = int(e.args[1])
            assert ex >= 2, e
            return "(" + "*".join([base] * ex) + ")"
        if isinstance(e, sp.Mul):
            coeff, rest = e.as_coeff_Mul()
            factors = sp.Mul.make_args(rest)
            body = "*".join(self.expr(f) if not isinstance(f, sp.Add) else "(" + self.expr(f) + ")" for f in factors)
            if coeff == 1:
                return body
            if coeff == -1:
                return f"(-({body}))"
            return f"(T({float(coeff)!r})*({body}))"
        if isinstance(e, sp.Add):
            terms = list(sp.Add.make_args(e))
            out = ""
            for i, t in enumerate(terms):
                coeff, rest = t.as_coeff_Mul()
                if coeff.is_negative:
                    tt = self.expr(-t)
                    out += f" - {tt}" if i else f"(-{tt})"
                else:
                    tt = self.expr(t)
                    out += f" + {tt}" if i else tt
            return out
        raise TypeError(type(e), e)


def main():
    names, outs = outputs()
    # hoist shared quantities: substitute them by symbols
    shared_syms = {k: sp.Symbol(k) for k in SHARED}
    rep = []
    for k, v in SHARED.items():
        rep.append((v, shared_syms[k]))
    outs = [o.subs(z**3, shared_syms["z3"]).subs(z**2, shared_syms["z2"]) for o in outs]
    repl, reduced = sp.cse(outs, symbols=sp.numbered_symbols("x"), optimizations="basic")
    cm, ca, sm = count_ops([r for _, r in repl] + reduced)
    pr = Printer()

    lines = []
    lines.append("// GENERATED by finite_root_generation_gb300/gen/gen_system.py -- do not edit.")
    lines.append("//")
    lines.append("// One j-group of the Stephenson II loop-closure system (reference FSYS,")
    lines.append("// htpykinematics.cu:36-122): the three equations (rows j-1, j+6, j+13), their")
    lines.append("// nonzero partial derivatives over Z (JVAR's sparsity, htpykinematics.cu:129-1129)")
    lines.append("// and the t-derivative dF/dq . dq/dt (JH's last column, htpysupport.cu:113-121).")
    lines.append(f"// Straight-line cost per group: {cm} complex mul, {ca} complex add/sub,")
    lines.append(f"// {sm} real-scalar x complex.")
    lines.append("#pragma once")
    lines.append("")
    lines.append(f"#define FRG_GEN_CMUL {cm}")
    lines.append(f"#define FRG_GEN_CADD {ca}")
    lines.append(f"#define FRG_GEN_SMUL {sm}")
    lines.append("")
    lines.append("// Output slots: fI, dI[8] over {A,C,H,Ac,Cc,Hc,U_j,Z0}, tI;")
    lines.append("//               fII, dII[6] over {B,F,Bc,Fc,U_j,Z0}, tII;")
    lines.append("//               fIII, dIII[16] over {A..H,Ac..Hc,U_j,Z0}, tIII.")
    lines.append("template <typename T>")
    lines.append("struct FrgGroupOut {")
    lines.append("  cx<T> fI, dI[8], tI;")
    lines.append("  cx<T> fII, dII[6], tII;")
    lines.append("  cx<T> fIII, dIII[16], tIII;")
    lines.append("};")
    lines.append("")
    lines.append("// Column in Z of each derivative slot (U_j's column is 13 + j, marked -1).")
    for fam, _, vars_ in FAMILIES:
        cols = ", ".join(str(COL[v]) for v in vars_)
        lines.append(f"#define FRG_COLS_{fam} {{{cols}}}")
    lines.append("")
    lines.append("template <typename T>")
    lines.append("__device__ __forceinline__ void frg_group_eval(")
    lines.append("    const cx<T> A, const cx<T> B, const cx<T> C, const cx<T> D, const cx<T> F, const cx<T> G,")
    lines.append("    const cx<T> H, const cx<T> Ac, const cx<T> Bc, const cx<T> Cc, const cx<T> Dc, const cx<T> Fc,")
    lines.append("    const cx<T> Gc, const cx<T> Hc, const cx<T> z,")
    lines.append("    const cx<T> e1, const cx<T> e2, const cx<T> ec1, const cx<T> ec2,")
    lines.append("    const cx<T> z2, const cx<T> z3,")
    lines.append("    const cx<T> P0, const cx<T> Pc0, const cx<T> dP0, const cx<T> dPc0,")
    lines.append("    const cx<T> U, const cx<T> iU, const cx<T> Pj, const cx<T> Pcj, const cx<T> Qj, const cx<T> Qcj,")
    lines.append("    const cx<T> dPj, const cx<T> dPcj, const cx<T> dQj, const cx<T> dQcj,")
    lines.append("    FrgGroupOut<T>& o) {")
    for s_, e in repl:
        lines.append(f"  const cx<T> {s_} = {pr.expr(e)};")
    slot = {"I": 0, "II": 0, "III": 0}
    for (kind, fam, v), e in zip(names, reduced):
        if kind == "f":
            lines.append(f"  o.f{fam} = {pr.expr(e)};")
        elif kind == "t":
            lines.append(f"  o.t{fam} = {pr.expr(e)};")
        else:
            lines.append(f"  o.d{fam}[{slot[fam]}] = {pr.expr(e)};")
            slot[fam] += 1
    lines.append("}")
    # ---- F only (the three equations), for FP64 residuals next to FP32 Jacobians
    f_outs = [fI, fII, fIII]
    f_outs = [o.subs(z**3, shared_syms["z3"]).subs(z**2, shared_syms["z2"]) for o in f_outs]
    frepl, fred = sp.cse(f_outs, symbols=sp.numbered_symbols("y"), optimizations="basic")
    fcm, fca, fsm = count_ops([r for _, r in frepl] + fred)
    lines.append("")
    lines.append(f"// The three equations alone: {fcm} complex mul, {fca} complex add/sub, {fsm} real x complex.")
    lines.append(f"#define FRG_GENF_CMUL {fcm}")
    lines.append(f"#define FRG_GENF_CADD {fca}")
    lines.append("template <typename T>")
    lines.append("__device__ __forceinline__ void frg_group_f(")
    lines.append("    const cx<T> A, const cx<T> B, const cx<T> C, const cx<T> D, const cx<T> F, const cx<T> G,")
    lines.append("    const cx<T> H, const cx<T> Ac, const cx<T> Bc, const cx<T> Cc, const cx<T> Dc, const cx<T> Fc,")
    lines.append("    const cx<T> Gc, const cx<T> Hc, const cx<T> z,")
    lines.append("    const cx<T> e1, const cx<T> e2, const cx<T> ec1, const cx<T> ec2,")
    lines.append("    const cx<T> z2, const cx<T> z3, const cx<T> P0, const cx<T> Pc0,")
    lines.append("    const cx<T> U, const cx<T> iU, const cx<T> Pj, const cx<T> Pcj, const cx<T> Qj, const cx<T> Qcj,")
    lines.append("    cx<T>& fI, cx<T>& fII, cx<T>& fIII) {")
    for s_, e in frepl:
        lines.append(f"  const cx<T> {s_} = {pr.expr(e)};")
    lines.append(f"  fI = {pr.expr(fred[0])};")
    lines.append(f"  fII = {pr.expr(fred[1])};")
    lines.append(f"  fIII = {pr.expr(fred[2])};")
    lines.append("}")
    used = set()
    for _, e in repl:
        used |= {s.name for s in e.free_symbols}
    for e in reduced:
        used |= {s.name for s in e.free_symbols}
    with open(OUT, "w") as fh:
        fh.write("\n".join(lines) + "\n")
    print(f"wrote {OUT}: {len(repl)} temporaries; per group {cm} cmul, {ca} cadd, {sm} smul; "
          f"F only {fcm} cmul, {fca} cadd")
    print("free inputs used:", sorted(u for u in used if not u.startswith("x")))


if __name__ == "__main__":
    main()
