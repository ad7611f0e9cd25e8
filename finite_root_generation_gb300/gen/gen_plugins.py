"""Generate the tracker's code for the system plug-ins (finite_root_generation_gb300/systems).

For every plug-in module listed in systems.PLUGINS this emits

  * a CUDA struct (../csrc/frg_plugins_gen.cuh) with
      NV, NP, NS          unknowns, parameters, solved parameters
      rows<T, LD>(Y, q, dq, M, F)
                          rows 0..NV-1 of the homotopy Jacobian at the path state
                          Y = [Z (NV), Z0, t]: M[i*LD + c] = dF_i/dY_c for the NV + 1
                          homogeneous unknowns and M[i*LD + NV + 1] = dF_i/dq . dq/dt
                          (the t column, as JH's last column, htpysupport.cu:113-121);
                          F[i] = F_i(Z, Z0; q) when F is given
      start(rng, dist, range, z, q)
                          the start root and start parameters: the unknowns and the free
                          parameters drawn (re, im per value, in declaration order), then
                          the solved parameters from the square linear system
      canonical(root, fpm, out)
                          the root as reported (plug-ins have no cognate map: a copy)
  * a plain-C copy of rows and start for the oracle (../../oracle/frg_plugins_gen.h),
    included by oracle/frg_oracle.c.

The equations are homogenized (F_i^h(Z, Z0) = Z0^{deg F_i} F_i(Z / Z0)), differentiated
by sympy and CSE'd. Run ``python finite_root_generation_gb300/gen/gen_plugins.py``;
the outputs are committed, and tests/test_plugins_cpu.py checks they are current.
"""
from __future__ import annotations

import importlib
import os
import sys

import sympy as sp

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(HERE)
CUDA_OUT = os.path.join(PKG, "csrc", "frg_plugins_gen.cuh")
C_OUT = os.path.join(PKG, "..", "oracle", "frg_plugins_gen.h")


def load_plugins():
    sys.path.insert(0, os.path.dirname(PKG))
    try:
        systems = importlib.import_module("finite_root_generation_gb300.systems")
        return [importlib.import_module(f"finite_root_generation_gb300.systems.{n}") for n in systems.PLUGINS]
    finally:
        sys.path.pop(0)


class Printer:
    """Straight-line printer for the two dialects: 'cuda' (cx<T> with operators) and
    'c' (the oracle's cd struct with cadd/csub/cmul/cscal/mk)."""

    def __init__(self, dialect, names):
        self.d = dialect
        self.names = names

    def num(self, v):
        v = float(v)
        return f"cx<T>(T({v!r}))" if self.d == "cuda" else f"mk({v!r}, 0.0)"

    def scale(self, c, body):
        c = float(c)
        if self.d == "cuda":
            return f"(-({body}))" if c == -1.0 else f"(T({c!r}) * ({body}))"
        return f"cscal({c!r}, {body})"

    def mul(self, parts):
        if self.d == "cuda":
            return "(" + " * ".join(parts) + ")" if len(parts) > 1 else parts[0]
        out = parts[-1]
        for p in reversed(parts[:-1]):
            out = f"cmul({p}, {out})"
        return out

    def expr(self, e) -> str:
        if e.is_Symbol:
            return self.names[e]
        if e.is_Number:
            return self.num(e)
        if e.has(sp.I):
            raise ValueError("plug-in systems have real rational coefficients")
        if isinstance(e, sp.Pow):
            ex = int(e.exp)
            if ex < 2 or ex != e.exp:
                raise ValueError(f"not a polynomial term: {e}")
            return self.mul([self.expr(e.base)] * ex)
        if isinstance(e, sp.Mul):
            coeff, rest = e.as_coeff_Mul()
            body = self.mul([self.expr(f) for f in sp.Mul.make_args(rest)])
            return body if coeff == 1 else self.scale(coeff, body)
        if isinstance(e, sp.Add):
            terms = list(sp.Add.make_args(e))
            if self.d == "cuda":
                out = ""
                for i, t in enumerate(terms):
                    if t.as_coeff_Mul()[0].is_negative:
                        out += f" - {self.expr(-t)}" if i else f"(-{self.expr(-t)})"
                    else:
                        out += f" + {self.expr(t)}" if i else self.expr(t)
                return "(" + out + ")"
            out = self.expr(terms[0])
            for t in terms[1:]:
                if t.as_coeff_Mul()[0].is_negative:
                    out = f"csub({out}, {self.expr(-t)})"
                else:
                    out = f"cadd({out}, {self.expr(t)})"
            return out
        raise TypeError(type(e), e)


def analyse(mod):
    """Homogenized equations and the expressions the emitted code evaluates."""
    X, Q, S = list(mod.UNKNOWNS), list(mod.PARAMS), list(mod.SOLVED)
    nv, np_, ns = len(X), len(Q), len(S)
    if len(mod.EQUATIONS) != nv:
        raise ValueError(f"{mod.NAME}: need one equation per unknown")
    if ns != nv or any(s not in Q for s in S):
        raise ValueError(f"{mod.NAME}: SOLVED must name one parameter per equation")
    if nv > 21:
        raise ValueError(f"{mod.NAME}: at most 21 unknowns")
    z0 = sp.Symbol("__Z0")
    dq = [sp.Symbol("__d_" + q.name) for q in Q]
    Fh = []
    for f in mod.EQUATIONS:
        p = sp.Poly(sp.expand(f), *X)
        Fh.append(sp.expand(p.homogenize(z0).as_expr()))
    cols = X + [z0]
    jac = [[sp.diff(f, v) for v in cols] + [sum(sp.diff(f, q) * d for q, d in zip(Q, dq))] for f in Fh]
    # start system: F(x, q) = A(x, q_free) s + b(x, q_free), s = the solved parameters
    A = [[sp.expand(sp.diff(f, s)) for s in S] for f in mod.EQUATIONS]
    b = [sp.expand(f.subs({s: 0 for s in S})) for f in mod.EQUATIONS]
    for row in A:
        for a in row:
            if any(a.has(s) for s in S):
                raise ValueError(f"{mod.NAME}: the equations must be linear in SOLVED")
    return dict(X=X, Q=Q, S=S, z0=z0, dq=dq, Fh=Fh, jac=jac, A=A, b=b, nv=nv, np=np_, ns=ns)


def names_for(info):
    names = {x: f"u_{x.name}" for x in info["X"]}
    names[info["z0"]] = "u_Z0"
    names.update({q: f"p_{q.name}" for q in info["Q"]})
    names.update({d: f"dp_{q.name}" for q, d in zip(info["Q"], info["dq"])})
    return names


def cse_block(exprs, tmp_prefix):
    repl, reduced = sp.cse(exprs, symbols=sp.numbered_symbols(tmp_prefix), optimizations="basic")
    return repl, reduced


def count_ops(exprs):
    """(complex multiplications, complex additions, real-scalar multiplications) of the
    straight-line code for `exprs` (powers as repeated products)."""
    cm = ca = sm = 0
    for e in exprs:
        for node in sp.preorder_traversal(e):
            if isinstance(node, sp.Mul):
                coeff, rest = node.as_coeff_Mul()
                cm += max(len(sp.Mul.make_args(rest)) - 1, 0)
                sm += 1 if coeff not in (1, -1) else 0
            elif isinstance(node, sp.Add):
                ca += len(node.args) - 1
            elif isinstance(node, sp.Pow):
                cm += int(node.exp) - 1
    return cm, ca, sm


def rows_cost(info):
    """Operation counts of one rows() evaluation (Jacobian rows, t column and F)."""
    flat = [e for row in info["jac"] for e in row] + info["Fh"]
    repl, red = cse_block(flat, "r_")
    return count_ops([e for _, e in repl] + list(red))


def emit_rows(mod, info, dialect):
    """Body lines of rows(): loads, CSE temporaries, the row entries and F."""
    names = names_for(info)
    nv = info["nv"]
    flat = [e for row in info["jac"] for e in row] + info["Fh"]
    repl, red = cse_block(flat, "r_")
    for s_, _ in repl:
        names[s_] = s_.name
    pr = Printer(dialect, names)
    used = set()
    for _, e in repl:
        used |= e.free_symbols
    for e in red:
        used |= e.free_symbols
    T = "const cx<T>" if dialect == "cuda" else "const cd"
    lines = []
    for i, x in enumerate(info["X"] + [info["z0"]]):
        if x in used:
            lines.append(f"  {T} {names[x]} = Y[{i}];")
    for i, (q, d) in enumerate(zip(info["Q"], info["dq"])):
        if q in used:
            lines.append(f"  {T} {names[q]} = q[{i}];")
        if d in used:
            lines.append(f"  {T} {names[d]} = dq[{i}];")
    for s_, e in repl:
        lines.append(f"  {T} {s_.name} = {pr.expr(e)};")
    ld = "LD" if dialect == "cuda" else "ld"
    k = 0
    for i in range(nv):
        for c in range(nv + 2):
            e = red[k]
            k += 1
            val = pr.expr(e) if e != 0 else ("cx<T>(T(0))" if dialect == "cuda" else "mk(0.0, 0.0)")
            lines.append(f"  M[{i} * {ld} + {c}] = {val};")
    lines.append("  if (F) {")
    for i in range(nv):
        lines.append(f"    F[{i}] = {pr.expr(red[k])};")
        k += 1
    lines.append("  }")
    return lines


def emit_start(mod, info, dialect):
    """Body lines of start(): draws, the linear system for the solved parameters, its
    solution into q."""
    names = names_for(info)
    X, Q, S = info["X"], info["Q"], info["S"]
    ns = info["ns"]
    lines = []
    draw = "start_value(rng, dist, range)" if dialect == "cuda" else "start_draw(c, r)"
    mkc = "cd" if dialect == "cuda" else "mk"
    for i, x in enumerate(X):
        lines.append(f"  {{ const double re = {draw}; const double im = {draw}; z[{i}] = {mkc}(re, im); }}")
    for i, q in enumerate(Q):
        if q not in S:
            lines.append(f"  {{ const double re = {draw}; const double im = {draw}; q[{i}] = {mkc}(re, im); }}")
    flat = [a for row in info["A"] for a in row] + info["b"]
    repl, red = cse_block(flat, "s_")
    for s_, _ in repl:
        names[s_] = s_.name
    # the CUDA start code works in double (T = double inside start())
    pr = Printer(dialect, names)
    used = set()
    for _, e in repl:
        used |= e.free_symbols
    for e in red:
        used |= e.free_symbols
    T = "const cx<T>" if dialect == "cuda" else "const cd"
    for i, x in enumerate(X):
        if x in used:
            lines.append(f"  {T} {names[x]} = z[{i}];")
    for i, q in enumerate(Q):
        if q in used:
            lines.append(f"  {T} {names[q]} = q[{i}];")
    for s_, e in repl:
        lines.append(f"  {T} {s_.name} = {pr.expr(e)};")
    arr = "cx<T>" if dialect == "cuda" else "cd"
    lines.append(f"  {arr} A[{ns * ns}], b[{ns}], s[{ns}];")
    zero = "cx<T>(T(0))" if dialect == "cuda" else "mk(0.0, 0.0)"
    for k in range(ns * ns):
        e = red[k]
        lines.append(f"  A[{k}] = {pr.expr(e) if e != 0 else zero};")
    for k in range(ns):
        e = red[ns * ns + k]
        neg = pr.expr(-e) if e != 0 else zero
        lines.append(f"  b[{k}] = {neg};")
    if dialect == "cuda":
        lines.append(f"  small_solve<{ns}>(A, b, s);")
    else:
        lines.append(f"  small_solve({ns}, A, b, s);")
    for k, sv in enumerate(S):
        lines.append(f"  q[{Q.index(sv)}] = s[{k}];")
    return lines


def cuda_struct(mod, info, sid):
    cname = "Sys_" + mod.NAME
    cm, ca, sm = rows_cost(info)
    out = [f"// ---- system {sid}: {mod.NAME} ({info['nv']} unknowns, {info['np']} parameters)",
           f"// rows(): {cm} complex mul, {ca} complex add/sub, {sm} real x complex",
           f"struct {cname} {{",
           f"  static constexpr int ID = {sid};",
           f"  static constexpr int NV = {info['nv']};",
           f"  static constexpr int NP = {info['np']};",
           f"  static constexpr int NS = {info['ns']};",
           f"  static constexpr int ROWS_CMUL = {cm}, ROWS_CADD = {ca}, ROWS_SMUL = {sm};",
           "  template <typename T, int LD>",
           "  __device__ static void rows(const cx<T>* Y, const cx<T>* q, const cx<T>* dq, cx<T>* M, cx<T>* F) {"]
    out += ["  " + ln for ln in emit_rows(mod, info, "cuda")]
    out += ["  }",
            "  __device__ static void start(Rng& rng, int dist, double range, cd* z, cd* q) {",
            "    typedef double T;"]
    out += ["  " + ln for ln in emit_start(mod, info, "cuda")]
    out += ["  }",
            "  __device__ static void canonical(const cd* root, const cd*, cd* out) {",
            "    for (int i = 0; i < NV; ++i) out[i] = root[i];",
            "  }",
            "};",
            ""]
    return out


def c_funcs(mod, info, sid):
    n = mod.NAME
    out = [f"/* ---- system {sid}: {n} ({info['nv']} unknowns, {info['np']} parameters) */",
           f"static void plug_{n}_rows(const cd* Y, const cd* q, const cd* dq, cd* M, int ld, cd* F) {{"]
    out += emit_rows(mod, info, "c")
    out += ["}",
            f"static void plug_{n}_start(const or_config* c, rng_t* r, cd* z, cd* q) {{"]
    out += emit_start(mod, info, "c")
    out += ["}", ""]
    return out


def generate():
    mods = load_plugins()
    infos = [analyse(m) for m in mods]
    cu = ["// GENERATED by finite_root_generation_gb300/gen/gen_plugins.py from the modules in",
          "// finite_root_generation_gb300/systems -- do not edit.",
          "//",
          "// System plug-ins for the one-thread-per-path tracker: the homogenized equations'",
          "// rows of the homotopy Jacobian (columns Z, Z0, then the t column dF/dq . dq/dt) and",
          "// the finite-root-generation start (random unknowns and free parameters, then the",
          "// parameters that make the random point an exact root).",
          "#pragma once",
          "",
          "#include \"frg_device.cuh\"",
          "",
          "namespace frg {",
          ""]
    c = ["/* GENERATED by finite_root_generation_gb300/gen/gen_plugins.py from the modules in",
         " * finite_root_generation_gb300/systems -- do not edit.",
         " *",
         " * ORACLE TEST INFRASTRUCTURE: the plug-in systems' rows and starts for the oracle's",
         " * tracker (included by frg_oracle.c, which defines cd, mk, cadd, csub, cmul, cscal,",
         " * rng_t, start_draw and small_solve). */",
         ""]
    listing = []
    for k, (m, info) in enumerate(zip(mods, infos)):
        sid = k + 1
        cu += cuda_struct(m, info, sid)
        c += c_funcs(m, info, sid)
        listing.append((sid, m.NAME, info))
    cu.append("}  // namespace frg")
    cu.append("")
    cu.append("// X(id, name, struct) for every plug-in")
    cu.append("#define FRG_PLUGIN_LIST(X) \\")
    cu += [f"  X({sid}, \"{n}\", frg::Sys_{n}) \\" for sid, n, _ in listing]
    cu.append("")
    cu.append(f"#define FRG_NUM_PLUGINS {len(listing)}")
    c.append("static const or_plugin OR_PLUGINS[] = {")
    for sid, n, info in listing:
        c.append(f"  {{{sid}, \"{n}\", {info['nv']}, {info['np']}, plug_{n}_rows, plug_{n}_start}},")
    c.append("};")
    c.append(f"#define OR_NUM_PLUGINS {len(listing)}")
    return "\n".join(cu) + "\n", "\n".join(c) + "\n"


def main(check=False):
    cu, c = generate()
    if check:
        return open(CUDA_OUT).read() == cu and open(C_OUT).read() == c
    with open(CUDA_OUT, "w") as f:
        f.write(cu)
    with open(C_OUT, "w") as f:
        f.write(c)
    print(f"wrote {CUDA_OUT} and {C_OUT}")
    return True


if __name__ == "__main__":
    main()
