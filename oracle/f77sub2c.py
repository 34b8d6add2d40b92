#!/usr/bin/env python3
"""Mechanical translator for the small Fortran-77 subset used by the LNS3D
block-pentadiagonal line solvers (src/penta{1,2}{p,bc}.f, src/cpenta{1,2}{p,bc}.f).

No Fortran compiler exists on either build machine, so this script is the
recipe that turns the reference's *own* solver sources into C, which is then
compiled into ``oracle/_ref/libref_penta.so``.  That library is the pin for
the oracle restatement in ``oracle/penta_oracle.c``: both must agree
bit-for-bit on the same inputs.  The generated C is a build product, written
only under ``oracle/_ref/`` (git-ignored); no reference source is copied into
the repository.

Supported subset (exactly what the translated solver files use):
  subroutine header, ``implicit none``, ``integer``/``real``/``complex``
  declarations with explicit-shape (optionally ``lo:hi``) dimensions,
  ``parameter``, ``do v = a, b[, s]`` / ``end do``, ``if (...) then`` /
  ``else`` / ``end if``, assignment, ``return``, ``end``, and the
  ``!$omp parallel do`` directive (translated to ``#pragma omp parallel for``
  with every scalar assigned inside the loop made private).  Free-form
  sources (``.f90``: the block-tridiagonal solvers src/nsolve{1,2}{p,bc}.f90)
  add ``&`` continuation lines, ``type[, intent(...)|, parameter] :: list``
  declarations and array-section assignments (``a(:, 1:k, 1, iv) = b(1, :,
  1:k, 1, iv)``), expanded into loops over the section subscripts in order.

Semantics follow a gfortran build with ``-fdefault-real-8``: ``real`` is
double, ``complex`` is a pair of doubles, complex multiply is
``(ac-bd, ad+bc)`` and complex divide is Smith's (1962) range-reduced
algorithm (gfortran's ``-fcx-fortran-rules`` default).  Array accesses are
bounds-checked: an out-of-range element access is skipped (reads give 0) and
counted in ``ref_oob_count``, so that reference index faults are observable
instead of undefined behaviour.

Usage: f77sub2c.py OUT.c OUT.h SRC.f [SRC.f ...]
"""
import re
import sys

TOK = re.compile(r"\s*(?:(\d+\.\d*(?:[eEdD][+-]?\d+)?|\d*\.\d+(?:[eEdD][+-]?\d+)?)|(\d+)|"
                 r"(\.(?:eq|ne|lt|gt|le|ge|and|or|not)\.)|([A-Za-z_][A-Za-z_0-9]*)|(\*\*|[-+*/(),:=]))")


def tokenize(s):
    out, pos = [], 0
    s = s.rstrip()
    while pos < len(s):
        m = TOK.match(s, pos)
        if not m or m.end() == pos:
            raise SyntaxError("cannot tokenize: %r at %d" % (s, pos))
        pos = m.end()
        real, integer, rel, name, op = m.groups()
        if real is not None:
            out.append(("real", real.lower().replace("d", "e")))
        elif integer is not None:
            out.append(("int", integer))
        elif rel is not None:
            out.append(("rel", rel.lower()))
        elif name is not None:
            out.append(("name", name.lower()))
        else:
            out.append(("op", op))
    return out


class Parser:
    """Recursive-descent expression parser producing (ctext, type) pairs."""

    def __init__(self, toks, unit):
        self.t, self.i, self.u = toks, 0, unit

    def peek(self):
        return self.t[self.i] if self.i < len(self.t) else (None, None)

    def take(self, kind=None, val=None):
        tok = self.peek()
        if kind and tok[0] != kind or val and tok[1] != val:
            raise SyntaxError("expected %s %s got %s" % (kind, val, tok))
        self.i += 1
        return tok

    def expr(self):
        return self.or_()

    def or_(self):
        a = self.and_()
        while self.peek() == ("rel", ".or."):
            self.take()
            b = self.and_()
            a = ("(%s || %s)" % (a[0], b[0]), "int")
        return a

    def and_(self):
        a = self.rel()
        while self.peek() == ("rel", ".and."):
            self.take()
            b = self.rel()
            a = ("(%s && %s)" % (a[0], b[0]), "int")
        return a

    def rel(self):
        a = self.add()
        tok = self.peek()
        ops = {".eq.": "==", ".ne.": "!=", ".lt.": "<", ".gt.": ">", ".le.": "<=", ".ge.": ">="}
        if tok[0] == "rel" and tok[1] in ops:
            self.take()
            b = self.add()
            if "complex" in (a[1], b[1]):
                raise SyntaxError("complex comparison")
            return ("(%s %s %s)" % (a[0], ops[tok[1]], b[0]), "int")
        return a

    def add(self):
        tok = self.peek()
        if tok == ("op", "-") or tok == ("op", "+"):
            self.take()
            a = self.mul()
            if tok[1] == "-":
                a = binop("neg", a, None)
        else:
            a = self.mul()
        while self.peek() in (("op", "+"), ("op", "-")):
            op = self.take()[1]
            b = self.mul()
            a = binop(op, a, b)
        return a

    def mul(self):
        a = self.unary()
        while self.peek() in (("op", "*"), ("op", "/")):
            op = self.take()[1]
            b = self.unary()
            a = binop(op, a, b)
        return a

    def unary(self):
        tok = self.peek()
        if tok == ("op", "-"):
            self.take()
            return binop("neg", self.unary(), None)
        return self.primary()

    def primary(self):
        kind, val = self.take()
        if kind == "int":
            return (val, "int")
        if kind == "real":
            return ("%s" % val if ("." in val or "e" in val) else val + ".0", "real")
        if kind == "op" and val == "(":
            e = self.expr()
            self.take("op", ")")
            return ("(%s)" % e[0], e[1])
        if kind == "name":
            if self.peek() == ("op", "("):
                self.take()
                idx = [self.expr()]
                while self.peek() == ("op", ","):
                    self.take()
                    idx.append(self.expr())
                self.take("op", ")")
                return self.u.array_ref(val, [x[0] for x in idx])
            return self.u.scalar_ref(val)
        raise SyntaxError("unexpected token %s %s" % (kind, val))


def promote(e, to):
    if e[1] == to:
        return e[0]
    if to == "complex":
        return "cx_r(%s)" % ("(double)(%s)" % e[0] if e[1] == "int" else e[0])
    if to == "real":
        return "(double)(%s)" % e[0]
    raise TypeError(to)


def binop(op, a, b):
    if op == "neg":
        if a[1] == "complex":
            return ("cx_neg(%s)" % a[0], "complex")
        return ("(-%s)" % a[0], a[1])
    rank = {"int": 0, "real": 1, "complex": 2}
    t = a[1] if rank[a[1]] >= rank[b[1]] else b[1]
    if t == "complex":
        fn = {"+": "cx_add", "-": "cx_sub", "*": "cx_mul", "/": "cx_div"}[op]
        return ("%s(%s, %s)" % (fn, promote(a, t), promote(b, t)), t)
    return ("(%s %s %s)" % (promote(a, t), op, promote(b, t)), t)


class Unit:
    def __init__(self, name, args):
        self.name, self.args = name, args
        self.types, self.dims, self.params = {}, {}, {}

    def declare(self, typ, items):
        for nm, dims in items:
            self.types[nm] = typ
            if dims:
                self.dims[nm] = dims

    def array_ref(self, nm, idx):
        if nm not in self.dims:
            raise SyntaxError("unknown array " + nm)
        dims = self.dims[nm]
        if len(idx) != len(dims):
            raise SyntaxError("rank mismatch for %s" % nm)
        terms = []
        for k, (lo, _hi) in enumerate(dims):
            terms.append("((long)(%s) - (long)(%s)) * st_%s_%d" % (idx[k], lo, nm, k))
        off = " + ".join(terms)
        return ("(*REF_%s(%s))" % (nm, off), self.types[nm])

    def scalar_ref(self, nm):
        if nm in self.params:
            return (nm, self.types.get(nm, "real"))
        if nm not in self.types:
            raise SyntaxError("undeclared scalar " + nm)
        return (nm, self.types[nm])


def split_top(s, sep=","):
    out, depth, cur = [], 0, ""
    for ch in s:
        if ch == "(":
            depth += 1
        elif ch == ")":
            depth -= 1
        if ch == sep and depth == 0:
            out.append(cur)
            cur = ""
        else:
            cur += ch
    out.append(cur)
    return [x.strip() for x in out if x.strip()]


def parse_decl_items(rest):
    items = []
    for it in split_top(rest):
        m = re.match(r"([a-z_][a-z_0-9]*)\s*(?:\((.*)\))?$", it)
        nm, dimstr = m.group(1), m.group(2)
        dims = []
        if dimstr:
            for d in split_top(dimstr):
                if ":" in d:
                    lo, hi = d.split(":")
                    dims.append((lo.strip(), hi.strip()))
                else:
                    dims.append(("1", d.strip()))
        items.append((nm, dims))
    return items


CTYPE = {"int": "int", "real": "double", "complex": "cx"}


def expr_c(text, unit):
    p = Parser(tokenize(text), unit)
    e = p.expr()
    if p.i != len(p.t):
        raise SyntaxError("trailing tokens in %r" % text)
    return e


def section_loops(lhs_text, rhs_text, unit, pad):
    """Loops for an array-section assignment: the i-th section subscript of
    the left side pairs with the i-th of the right side."""
    def parts(text):
        m = re.match(r"([a-z_][a-z_0-9]*)\s*\((.*)\)$", text.strip())
        return m.group(1), split_top(m.group(2))
    ln, lsub = parts(lhs_text)
    rn, rsub = parts(rhs_text)
    def ranges(nm, subs):
        out = []
        for k, sb in enumerate(subs):
            if ":" in sb:
                lo, hi = sb.split(":")
                dlo, dhi = unit.dims[nm][k]
                out.append((k, lo.strip() or dlo, hi.strip() or dhi))
        return out
    lr, rr = ranges(ln, lsub), ranges(rn, rsub)
    if len(lr) != len(rr):
        raise SyntaxError("non-conforming sections: %s = %s" % (lhs_text, rhs_text))
    lines, lidx, ridx = [], list(lsub), list(rsub)
    for a, ((kl, lo, hi), (kr, rlo, _rhi)) in enumerate(zip(lr, rr)):
        v = "sec_%d" % a
        lines.append(pad + "  " * a + "for (long %s = 0; %s <= (long)(%s) - (long)(%s); ++%s) {" % (
            v, v, expr_c(hi, unit)[0], expr_c(lo, unit)[0], v))
        lidx[kl] = "__SEC%d_L__" % a
        ridx[kr] = "__SEC%d_R__" % a
    subs = {}
    for a, ((kl, lo, _), (kr, rlo, _)) in enumerate(zip(lr, rr)):
        subs["__sec%d_l__" % a] = "((long)(%s) + sec_%d)" % (expr_c(lo, unit)[0], a)
        subs["__sec%d_r__" % a] = "((long)(%s) + sec_%d)" % (expr_c(rlo, unit)[0], a)
    unit.params.update({k: "0" for k in subs})
    lhs = expr_c("%s(%s)" % (ln, ",".join(lidx)), unit)
    rhs = expr_c("%s(%s)" % (rn, ",".join(ridx)), unit)
    for k in subs:
        del unit.params[k]
    stmt = "%s = %s;" % (lhs[0], promote(rhs, lhs[1]))
    for k, v in subs.items():
        stmt = stmt.replace(k, v)
    lines.append(pad + "  " * len(lr) + stmt)
    lines.append(pad + "}" * len(lr))
    return lines


def translate(path):
    free = path.endswith(".f90")
    src = open(path).read().lower().splitlines()
    if free:  # join '&' continuation lines
        joined, cur = [], ""
        for raw in src:
            s = raw.split("!")[0].rstrip() if not raw.strip().startswith("!$omp") else raw.rstrip()
            if cur:
                s = cur + " " + s.strip().lstrip("&")
                cur = ""
            if s.endswith("&") and not s.strip().startswith("!"):
                cur = s[:-1]
                continue
            joined.append(s if s.strip() else raw)
        src = joined
    stmts = []  # (kind, payload)
    for raw in src:
        s = raw.strip()
        if not s:
            continue
        if s.startswith("!$omp"):
            stmts.append(("omp", s))
            continue
        if s.startswith("!") or (not free and raw[:1] in ("c", "*") and not raw.startswith(" ")):
            continue
        s = s.split("!")[0].strip()
        if s:
            stmts.append(("stmt", s))

    unit = None
    body = []
    indent = 1
    pending_omp = False
    loop_stack = []
    omp_regions = []  # (body index of the locals placeholder, scalars assigned inside)
    omp_assigned = set()
    for kind, s in stmts:
        if kind == "omp":
            if "parallel do" in s and not re.search(r"end\s+parallel", s):
                pending_omp = True
            continue
        m = re.match(r"subroutine\s+([a-z_0-9]+)\s*\((.*)\)$", s)
        if m:
            unit = Unit(m.group(1), [a.strip() for a in m.group(2).split(",")])
            continue
        if s == "implicit none":
            continue
        m = re.match(r"(integer|real|complex)\s*((?:,\s*[a-z]+(?:\([a-z]+\))?\s*)*)::\s*(.*)$", s)
        if m:  # free-form declaration: type[, intent(...)][, parameter] :: list
            typ = {"integer": "int", "real": "real", "complex": "complex"}[m.group(1)]
            if "parameter" in m.group(2):
                for it in split_top(m.group(3)):
                    nm, val = [x.strip() for x in it.split("=")]
                    unit.params[nm] = val
                    unit.types[nm] = typ
            else:
                unit.declare(typ, parse_decl_items(m.group(3)))
            continue
        m = re.match(r"(integer|real|complex)\s+(.*)$", s)
        if m:
            unit.declare({"integer": "int", "real": "real", "complex": "complex"}[m.group(1)],
                         parse_decl_items(m.group(2)))
            continue
        m = re.match(r"parameter\s*\((.*)\)$", s)
        if m:
            for it in split_top(m.group(1)):
                nm, val = [x.strip() for x in it.split("=")]
                unit.params[nm] = val
            continue
        m = re.match(r"do\s+([a-z_0-9]+)\s*=\s*(.*)$", s)
        if m:
            v = m.group(1)
            if any(k == "omp" for k, _ in loop_stack):
                omp_assigned.add(v)
            parts = split_top(m.group(2))
            lo = expr_c(parts[0], unit)[0]
            hi = expr_c(parts[1], unit)[0]
            st = expr_c(parts[2], unit)[0] if len(parts) > 2 else "1"
            pad = "    " * indent
            if pending_omp:
                body.append(pad + "{ const long trip_%s = ((long)(%s) - (long)(%s) + (long)(%s)) / (long)(%s);" % (v, hi, lo, st, st))
                body.append(pad + "#pragma omp parallel for schedule(static)")
                body.append(pad + "for (long it_%s = 0; it_%s < trip_%s; ++it_%s) {" % (v, v, v, v))
                body.append(pad + "  int %s = (int)((long)(%s) + it_%s * (long)(%s));" % (v, lo, v, st))
                body.append(pad + "  /*OMP_LOCALS*/")
                omp_assigned = set()
                omp_regions.append((len(body) - 1, omp_assigned))
                loop_stack.append(("omp", v))
                pending_omp = False
            else:
                body.append(pad + "{ const long trip_%s_%d = ((long)(%s) - (long)(%s) + (long)(%s)) / (long)(%s);" % (v, len(body), hi, lo, st, st))
                body.append(pad + "for (long it_%s_%d = 0; it_%s_%d < trip_%s_%d; ++it_%s_%d) {" % (v, len(body) - 1, v, len(body) - 1, v, len(body) - 1, v, len(body) - 1))
                body.append(pad + "  %s = (int)((long)(%s) + it_%s_%d * (long)(%s));" % (v, lo, v, len(body) - 2, st))
                loop_stack.append(("do", v))
            indent += 1
            continue
        if s in ("end do", "enddo"):
            indent -= 1
            kind_, v = loop_stack.pop()
            body.append("    " * indent + "}}")
            continue
        m = re.match(r"if\s*\((.*)\)\s*then$", s)
        if m:
            body.append("    " * indent + "if (%s) {" % expr_c(m.group(1), unit)[0])
            indent += 1
            continue
        if s == "else":
            body.append("    " * (indent - 1) + "} else {")
            continue
        if s in ("end if", "endif"):
            indent -= 1
            body.append("    " * indent + "}")
            continue
        if s == "return":
            body.append("    " * indent + "return;")
            continue
        if s == "end" or s.startswith("end subroutine"):
            continue
        m = re.match(r"(.*?)=(.*)$", s)
        if m and ":" in m.group(1):  # array-section assignment
            body.extend(section_loops(m.group(1).strip(), m.group(2).strip(), unit, "    " * indent))
            continue
        if m:
            lhs = expr_c(m.group(1).strip(), unit)
            rhs = expr_c(m.group(2).strip(), unit)
            tgt = m.group(1).strip()
            if any(k == "omp" for k, _ in loop_stack) and "(" not in tgt:
                omp_assigned.add(tgt)
            body.append("    " * indent + "%s = %s;" % (lhs[0], promote(rhs, lhs[1])))
            continue
        raise SyntaxError("unsupported statement: %r" % s)

    # scalars assigned or used as loop indices inside an OpenMP loop become private
    for k, assigned in omp_regions:
        privs = sorted(assigned)
        body[k] = body[k].replace(
            "/*OMP_LOCALS*/", " ".join("%s %s;" % (CTYPE[unit.types[nm]], nm) for nm in privs
                                       if nm != loop_iv(body, k)) +
            " /* private per system */")
    return unit, body, omp_regions


def loop_iv(body, k):
    m = re.search(r"int ([a-z_0-9]+) = ", body[k - 1])
    return m.group(1) if m else None


def emit(units):
    out = []
    out.append("/* Generated by oracle/f77sub2c.py from the reference solver sources. */")
    out.append("/* Build product: do not edit, do not commit. */")
    out.append("#include <math.h>\n#include <stddef.h>\n#include \"ref_penta.h\"")
    out.append("long ref_oob_count = 0;")
    out.append("static double ref_sink_r; static cx ref_sink_c;")
    out.append("static inline cx cx_r(double a) { cx z; z.re = a; z.im = 0.0; return z; }")
    out.append("static inline cx cx_neg(cx a) { cx z; z.re = -a.re; z.im = -a.im; return z; }")
    out.append("static inline cx cx_add(cx a, cx b) { cx z; z.re = a.re + b.re; z.im = a.im + b.im; return z; }")
    out.append("static inline cx cx_sub(cx a, cx b) { cx z; z.re = a.re - b.re; z.im = a.im - b.im; return z; }")
    out.append("static inline cx cx_mul(cx a, cx b) { cx z; z.re = a.re * b.re - a.im * b.im; z.im = a.re * b.im + a.im * b.re; return z; }")
    out.append("/* Smith (1962), Algorithm 116: range-reduced complex division. */")
    out.append("static inline cx cx_div(cx a, cx b) { cx z; double r, d;\n"
               "  if (fabs(b.re) < fabs(b.im)) { r = b.re / b.im; d = b.re * r + b.im;\n"
               "    z.re = (a.re * r + a.im) / d; z.im = (a.im * r - a.re) / d; }\n"
               "  else { r = b.im / b.re; d = b.im * r + b.re;\n"
               "    z.re = (a.im * r + a.re) / d; z.im = (a.im - a.re * r) / d; }\n"
               "  return z; }")
    for unit, body, _ in units:
        sig = []
        for a in unit.args:
            t = unit.types[a]
            if a in unit.dims:
                sig.append("%s* %s" % (CTYPE[t], a))
            else:
                sig.append("int %s" % a)
        out.append("void ref_%s(%s) {" % (unit.name, ", ".join(sig)))
        for nm, val in unit.params.items():
            out.append("    const %s %s = %s;" % (CTYPE[unit.types.get(nm, "real")], nm, expr_c(val, unit)[0]))
        for nm, t in unit.types.items():
            if nm in unit.args or nm in unit.params or nm in unit.dims:
                continue
            out.append("    %s %s; (void)%s;" % (CTYPE[t], nm, nm))
        for nm, dims in unit.dims.items():
            stride = "1L"
            for k, (lo, hi) in enumerate(dims):
                lo_c = expr_c(lo, unit)[0]
                hi_c = expr_c(hi, unit)[0]
                out.append("    const long st_%s_%d = %s;" % (nm, k, stride))
                stride = "(st_%s_%d * ((long)(%s) - (long)(%s) + 1L))" % (nm, k, hi_c, lo_c)
            out.append("    const long sz_%s = %s;" % (nm, stride))
            sink = "ref_sink_c" if unit.types[nm] == "complex" else "ref_sink_r"
            zero = "cx_r(0.0)" if unit.types[nm] == "complex" else "0.0"
            out.append("#define REF_%s(off) ref_at_%s_%s(%s, sz_%s, (off))" % (nm, unit.name, nm, nm, nm))
        out.extend(body)
        for nm in unit.dims:
            out.append("#undef REF_%s" % nm)
        out.append("}")
        # bounds-checked accessors are emitted before the function body
        acc = []
        for nm in unit.dims:
            ct = CTYPE[unit.types[nm]]
            sink = "ref_sink_c" if unit.types[nm] == "complex" else "ref_sink_r"
            zero = "cx_r(0.0)" if unit.types[nm] == "complex" else "0.0"
            acc.append("static inline %s* ref_at_%s_%s(%s* base, long sz, long off) {\n"
                       "  if (off < 0 || off >= sz) {\n"
                       "    _Pragma(\"omp atomic\")\n    ++ref_oob_count;\n"
                       "    %s = %s; return &%s; }\n"
                       "  return base + off; }" % (ct, unit.name, nm, ct, sink, zero, sink))
        idx = out.index("void ref_%s(%s) {" % (unit.name, ", ".join(sig)))
        out[idx:idx] = acc
    return "\n".join(out) + "\n"


def main():
    out_c, out_h, srcs = sys.argv[1], sys.argv[2], sys.argv[3:]
    units = [translate(s) for s in srcs]
    with open(out_c, "w") as f:
        f.write(emit(units))
    with open(out_h, "w") as f:
        f.write("/* Generated by oracle/f77sub2c.py; declarations of the translated solvers. */\n")
        f.write("#pragma once\ntypedef struct { double re, im; } cx;\nextern long ref_oob_count;\n")
        for unit, _, _ in units:
            sig = []
            for a in unit.args:
                t = unit.types[a]
                sig.append("%s* %s" % (CTYPE[t], a) if a in unit.dims else "int %s" % a)
            f.write("void ref_%s(%s);\n" % (unit.name, ", ".join(sig)))


if __name__ == "__main__":
    main()
