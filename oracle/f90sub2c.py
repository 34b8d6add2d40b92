#!/usr/bin/env python3
"""Translator for the Fortran 90 (and fixed-form 77) subset used by the LNS3D
implicit-step routines, into C: the recipe that builds the reference's own
step code (``oracle/_ref/libref_step.so``) where no Fortran compiler exists.

Test infrastructure only.  The generated C is a build product under
``oracle/_ref/`` (git-ignored); no reference source is copied into the
repository.  It pins the hand restatements of the step (``adi3d_oracle.c``,
``impdrv2d_oracle.c``) routine by routine, and through them the GPU kernels.

What it accepts (exactly what the translated files use):
  * program units: ``module`` (variables, parameters, ``contains``),
    ``subroutine``, typed ``function``, generic ``interface`` blocks;
    ``use`` (module association), ``implicit none`` or default implicit typing;
  * declarations: integer, real, real*4, complex, logical, character(len) with
    ``parameter``, ``allocatable``, ``save``, ``intent``, ``external``,
    ``dimension``; explicit-shape, assumed-shape (``:``), assumed-size (``*``)
    and deferred-shape arrays; initialised locals are SAVEd;
  * statements: assignment (scalar, array element, whole-array and section
    assignment lowered to loops), ``call``, ``if``/``else if``/``else``,
    logical ``if``, ``do`` (named, with step) and ``do while``, ``exit``,
    ``cycle``, ``goto``/labels, ``continue``, ``return``, ``stop``,
    ``allocate``/``deallocate``, ``where`` (statement form);
  * unformatted sequential ``read``/``write`` (items, implied-do lists,
    ``err=``/``end=``) and ``open``/``close`` become calls of I/O hooks the
    harness provides; formatted writes pass their numeric scalar items to a
    hook (full precision) and are otherwise dropped;
  * expressions: ``**`` (integer powers expanded as gcc's powi does), complex
    arithmetic (multiply ``(ac-bd, ad+bc)``, Smith's (1962) division, real
    operands lowered component-wise as gcc's complex lowering does),
    intrinsics (abs, sqrt, exp, log, log10, sin, cos, tan, tanh, atan, atan2,
    max, min, mod, sign, int, nint, real, float, dble, cmplx, conjg, aimag,
    maxval, minval, maxloc, sum, size, allocated, char, ...).

Semantics are those of a gfortran build with ``-fdefault-real-8`` (REAL and
default COMPLEX are 8-byte per part), serial: OpenMP directives are dropped.
Array accesses can be bounds-checked (``-DREF_BOUNDS``): an out-of-range
element is counted in ``ref_oob_count`` and redirected to a scratch cell.

Usage: f90sub2c.py [-D NAME]... [-P FILE:LINE OLD NEW]... OUT.c OUT.h SRC...
  -P replaces the text OLD by NEW on one line of one source file before
  translation (the recipe uses it for the one documented reference fault
  that the drop-in corrects).
"""
import re
import sys

# --------------------------------------------------------------------------
# source reading
# --------------------------------------------------------------------------


class Stmt:
    __slots__ = ("text", "label", "file", "line")

    def __init__(self, text, label, file, line):
        self.text, self.label, self.file, self.line = text, label, file, line

    def __repr__(self):
        return "%s:%d: %s" % (self.file, self.line, self.text)


def preprocess(lines, defines):
    """cpp-style conditionals (#define, #undef, #if[n]def, #if, #else, #endif)."""
    out, stack = [], []
    active = True
    defs = dict(defines)
    for n, raw in enumerate(lines):
        s = raw.strip()
        if s.startswith("#"):
            d = s[1:].strip()
            if d.startswith("ifdef"):
                stack.append(active)
                active = active and d.split()[1] in defs
            elif d.startswith("ifndef"):
                stack.append(active)
                active = active and d.split()[1] not in defs
            elif d.startswith("if"):
                stack.append(active)
                cond = d[2:].strip()
                m = re.match(r"defined\s*\(?\s*(\w+)\s*\)?$", cond)
                if m:
                    val = m.group(1) in defs
                elif re.match(r"^\d+$", cond):
                    val = int(cond) != 0
                else:
                    val = bool(defs.get(cond, 0))
                active = active and val
            elif d.startswith("else"):
                parent = stack[-1] if stack else True
                active = parent and not active
            elif d.startswith("endif"):
                active = stack.pop()
            elif d.startswith("define") and active:
                parts = d.split()
                defs[parts[1]] = parts[2] if len(parts) > 2 else "1"
            elif d.startswith("undef") and active:
                defs.pop(d.split()[1], None)
            out.append((n + 1, ""))
            continue
        out.append((n + 1, raw if active else ""))
    return out


def strip_comment(s):
    """Remove a trailing ! comment outside string literals."""
    q = None
    for i, ch in enumerate(s):
        if q:
            if ch == q:
                q = None
        elif ch in "'\"":
            q = ch
        elif ch == "!":
            return s[:i]
    return s


def split_semicolons(s):
    out, q, cur = [], None, ""
    for ch in s:
        if q:
            if ch == q:
                q = None
        elif ch in "'\"":
            q = ch
        elif ch == ";":
            out.append(cur)
            cur = ""
            continue
        cur += ch
    out.append(cur)
    return [x for x in out if x.strip()]


def lower_outside_strings(s):
    out, q = [], None
    for ch in s:
        if q:
            out.append(ch)
            if ch == q:
                q = None
        elif ch in "'\"":
            q = ch
            out.append(ch)
        else:
            out.append(ch.lower())
    return "".join(out)


PATCHES = []   # (file basename, line number, old text, new text)


def read_source(path, defines):
    fixed = not path.endswith(".f90")
    lines = open(path, errors="replace").read().expandtabs(8).splitlines()
    base = path.split("/")[-1]
    for pf, pl, old, new in PATCHES:
        if pf == base:
            if old not in lines[pl - 1]:
                raise SyntaxError("patch %s:%d does not match: %r" % (pf, pl, lines[pl - 1]))
            lines[pl - 1] = lines[pl - 1].replace(old, new)
    pre = preprocess(lines, defines)
    stmts = []
    if fixed:
        cur, cur_label, cur_line = None, None, 0
        for n, raw in pre:
            if not raw.strip() or raw[:1] in "cC*!":
                continue
            raw = raw[:120]
            body = strip_comment(raw[6:]) if len(raw) > 6 else ""
            if len(raw) > 5 and raw[5] not in " 0":
                if cur is not None:
                    cur += " " + body.strip()
                continue
            if cur is not None and cur.strip():
                stmts.append((cur, cur_label, cur_line))
            lab = raw[:5].strip()
            cur, cur_label, cur_line = body, (lab or None), n
        if cur is not None and cur.strip():
            stmts.append((cur, cur_label, cur_line))
    else:
        cur, cur_line = None, 0
        for n, raw in pre:
            s = raw.strip()
            if s.startswith("!"):
                continue
            s = strip_comment(raw).strip()
            if not s:
                continue
            if cur is not None:
                s = s[1:] if s.startswith("&") else s
                s = cur + " " + s
            else:
                cur_line = n
            if s.rstrip().endswith("&"):
                cur = s.rstrip()[:-1]
                continue
            cur = None
            m = re.match(r"^(\d+)\s+(.*)$", s)
            lab = None
            if m:
                lab, s = m.group(1), m.group(2)
            stmts.append((s, lab, cur_line))
    out = []
    for s, lab, n in stmts:
        for part in split_semicolons(s):
            out.append(Stmt(lower_outside_strings(part.strip()), lab, path, n))
            lab = None
    return out


# --------------------------------------------------------------------------
# expressions
# --------------------------------------------------------------------------

OPWORDS = ("eq", "ne", "lt", "gt", "le", "ge", "and", "or", "not", "eqv", "neqv", "true", "false")
TOKRE = re.compile(r"""
   (?P<ws>\s+)
 | (?P<str>'(?:[^']|'')*'|"(?:[^"]|"")*")
 | (?P<dot>\.(?:eq|ne|lt|gt|le|ge|and|or|not|eqv|neqv|true|false)\.)
 | (?P<num>(?:\d+\.\d*|\.\d+|\d+)(?:[eEdD][+-]?\d+)?(?:_\w+)?)
 | (?P<name>[A-Za-z_][A-Za-z_0-9]*)
 | (?P<op>\*\*|//|==|/=|<=|>=|=>|::|[-+*/(),:=<>%])
""", re.X)


def tokenize(s):
    toks, pos = [], 0
    while pos < len(s):
        m = TOKRE.match(s, pos)
        if not m:
            raise SyntaxError("cannot tokenize %r at %d" % (s, pos))
        kind = m.lastgroup
        val = m.group(kind)
        if kind == "num":
            # "1.eq.2": an integer followed by a dotted operator
            mm = re.match(r"(\d+)\.(eq|ne|lt|gt|le|ge|and|or|not|eqv|neqv)\.", s[pos:])
            if mm:
                toks.append(("int", mm.group(1)))
                pos += len(mm.group(1))
                continue
        pos = m.end()
        if kind == "ws":
            continue
        if kind == "num":
            v = re.sub(r"_\w+$", "", val)
            if re.match(r"^\d+$", v):
                toks.append(("int", v))
            else:
                toks.append(("real", v))
        else:
            toks.append((kind, val))
    return toks


class N:
    """Expression node: kind in num, str, log, name, ref, bin, un, cplx, sec, kw."""
    __slots__ = ("k", "a", "b", "c")

    def __init__(self, k, a=None, b=None, c=None):
        self.k, self.a, self.b, self.c = k, a, b, c

    def __repr__(self):
        return "N(%s,%r,%r,%r)" % (self.k, self.a, self.b, self.c)


class EParser:
    def __init__(self, text):
        self.t = tokenize(text)
        self.i = 0
        self.text = text

    def peek(self, k=0):
        j = self.i + k
        return self.t[j] if j < len(self.t) else (None, None)

    def take(self, kind=None, val=None):
        tok = self.peek()
        if (kind and tok[0] != kind) or (val is not None and tok[1] != val):
            raise SyntaxError("expected %s %s, got %s in %r" % (kind, val, tok, self.text))
        self.i += 1
        return tok

    def at_op(self, *vals):
        tok = self.peek()
        return tok[0] in ("op", "dot") and tok[1] in vals

    def done(self):
        return self.i >= len(self.t)

    def expr(self):
        return self.eqv()

    def eqv(self):
        a = self.lor()
        while self.at_op(".eqv.", ".neqv."):
            op = self.take()[1]
            a = N("bin", op, a, self.lor())
        return a

    def lor(self):
        a = self.land()
        while self.at_op(".or."):
            self.take()
            a = N("bin", ".or.", a, self.land())
        return a

    def land(self):
        a = self.lnot()
        while self.at_op(".and."):
            self.take()
            a = N("bin", ".and.", a, self.lnot())
        return a

    def lnot(self):
        if self.at_op(".not."):
            self.take()
            return N("un", ".not.", self.lnot())
        return self.rel()

    RELS = {".eq.": "==", ".ne.": "/=", ".lt.": "<", ".gt.": ">", ".le.": "<=", ".ge.": ">=",
            "==": "==", "/=": "/=", "<": "<", ">": ">", "<=": "<=", ">=": ">="}

    def rel(self):
        a = self.concat()
        tok = self.peek()
        if tok[0] in ("op", "dot") and tok[1] in self.RELS:
            self.take()
            return N("bin", self.RELS[tok[1]], a, self.concat())
        return a

    def concat(self):
        a = self.add()
        while self.at_op("//"):
            self.take()
            a = N("bin", "//", a, self.add())
        return a

    def add(self):
        if self.at_op("-", "+"):
            op = self.take()[1]
            a = self.mul()
            if op == "-":
                a = N("un", "-", a)
        else:
            a = self.mul()
        while self.at_op("+", "-"):
            op = self.take()[1]
            a = N("bin", op, a, self.mul())
        return a

    def mul(self):
        a = self.power()
        while self.at_op("*", "/"):
            op = self.take()[1]
            a = N("bin", op, a, self.power())
        return a

    def power(self):
        a = self.primary()
        if self.at_op("**"):
            self.take()
            if self.at_op("-", "+"):  # x**-1
                op = self.take()[1]
                b = self.power()
                b = N("un", "-", b) if op == "-" else b
            else:
                b = self.power()
            return N("bin", "**", a, b)
        return a

    def arglist(self):
        """Inside parentheses: expressions, sections (lo:hi[:st]) and keyword=expr."""
        args = []
        if self.at_op(")"):
            return args
        while True:
            if self.peek()[0] == "name" and self.peek(1) == ("op", "="):
                kw = self.take()[1]
                self.take("op", "=")
                args.append(N("kw", kw, self.expr()))
            else:
                args.append(self.section_or_expr())
            if self.at_op(","):
                self.take()
                continue
            break
        return args

    def section_or_expr(self):
        lo = hi = st = None
        if not self.at_op(":"):
            lo = self.expr()
            if not self.at_op(":"):
                return lo
        self.take("op", ":")
        if not self.at_op(",", ")", ":"):
            hi = self.expr()
        if self.at_op(":"):
            self.take()
            st = self.expr()
        return N("sec", lo, hi, st)

    def primary(self):
        kind, val = self.take()
        if kind == "int":
            return N("num", val, "int")
        if kind == "real":
            return N("num", val, "real")
        if kind == "str":
            q = val[0]
            return N("str", val[1:-1].replace(q + q, q))
        if kind == "dot" and val in (".true.", ".false."):
            return N("log", val == ".true.")
        if kind == "op" and val == "(":
            e = self.expr()
            if self.at_op(","):  # complex constant (re, im)
                self.take()
                e2 = self.expr()
                self.take("op", ")")
                return N("cplx", e, e2)
            self.take("op", ")")
            return N("paren", e)
        if kind == "name":
            if self.at_op("("):
                self.take()
                args = self.arglist()
                self.take("op", ")")
                node = N("ref", val, args)
                if self.at_op("("):  # substring of an array element: a(i)(1:3)
                    self.take()
                    sub = self.arglist()
                    self.take("op", ")")
                    node = N("ref", val, args, sub)
                return node
            return N("name", val)
        raise SyntaxError("unexpected %s %r in %r" % (kind, val, self.text))


def parse_expr(text):
    p = EParser(text)
    e = p.expr()
    if not p.done():
        raise SyntaxError("trailing tokens in %r: %r" % (text, p.t[p.i:]))
    return e


def split_top(s, sep=","):
    out, depth, cur, q = [], 0, "", None
    for ch in s:
        if q:
            cur += ch
            if ch == q:
                q = None
            continue
        if ch in "'\"":
            q = ch
        elif ch == "(":
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


def find_top(s, ch):
    """Index of the first ch outside parentheses and strings, or -1."""
    depth, q = 0, None
    for i, c in enumerate(s):
        if q:
            if c == q:
                q = None
            continue
        if c in "'\"":
            q = c
        elif c == "(":
            depth += 1
        elif c == ")":
            depth -= 1
        elif c == ch and depth == 0:
            return i
    return -1


def match_paren(s, start):
    """Index of the ')' closing the '(' at s[start]."""
    depth, q = 0, None
    for i in range(start, len(s)):
        c = s[i]
        if q:
            if c == q:
                q = None
            continue
        if c in "'\"":
            q = c
        elif c == "(":
            depth += 1
        elif c == ")":
            depth -= 1
            if depth == 0:
                return i
    raise SyntaxError("unbalanced parentheses in %r" % s)


# --------------------------------------------------------------------------
# symbols and program units
# --------------------------------------------------------------------------

CT = {"int": "int", "real": "double", "complex": "cx", "logical": "int", "char": "char", "real4": "float"}


class Sym:
    def __init__(self, name, typ):
        self.name, self.type = name, typ
        self.dims = None          # list of (lo, hi) nodes; hi None => '*', ('def',) => ':'
        self.deferred = False     # allocatable / assumed-shape: bounds at run time
        self.assumed_shape = False
        self.param = None         # parameter value node
        self.init = None
        self.save = False
        self.allocatable = False
        self.external = False
        self.dummy = False
        self.charlen = None
        self.module = None        # owning module name for module variables
        self.kind = "var"         # var | proc

    @property
    def rank(self):
        return len(self.dims) if self.dims else 0


class Unit:
    def __init__(self, kind, name, args=(), host=None):
        self.kind, self.name, self.args = kind, name, list(args)
        self.host = host
        self.module = None
        self.uses = []
        self.syms = {}
        self.implicit_none = False
        self.body_stmts = []
        self.contains = []
        self.result = None
        self.rtype = None
        self.generics = {}        # generic interface name -> [specific names]
        self.iface_units = {}     # specific name -> Unit (interface body)


TYPE_RE = re.compile(r"^(integer|real\s*\*\s*8|real\s*\*\s*4|real|double\s+precision|complex\s*\*\s*16|"
                     r"complex|logical|character(?:\s*\*\s*\(?\s*\w+\s*\)?|\s*\([^)]*\))?)(?![a-z0-9_])(.*)$")


def base_type(t):
    t = t.replace(" ", "")
    if t.startswith("integer"):
        return "int", None
    if t in ("real*4",):
        return "real4", None
    if t.startswith("real") or t.startswith("doubleprecision"):
        return "real", None
    if t.startswith("complex"):
        return "complex", None
    if t.startswith("logical"):
        return "logical", None
    if t.startswith("character"):
        m = re.search(r"(\d+)", t)
        return "char", int(m.group(1)) if m else 1
    raise SyntaxError(t)


def parse_dims(text):
    dims = []
    for d in split_top(text):
        if d == ":":
            dims.append(("def",))
        elif d == "*":
            dims.append((N("num", "1", "int"), None))
        else:
            k = find_top(d, ":")
            if k >= 0:
                lo, hi = d[:k].strip(), d[k + 1:].strip()
                dims.append((parse_expr(lo), None if hi == "*" else parse_expr(hi)))
            else:
                dims.append((N("num", "1", "int"), parse_expr(d)))
    return dims


def parse_decl(unit, typ_text, rest):
    typ, clen = base_type(typ_text)
    attrs, items_text = [], rest
    k = rest.find("::")
    if k >= 0:
        attrs = split_top(rest[:k].lstrip(","))
        items_text = rest[k + 2:]
    elif rest.strip().startswith(","):
        raise SyntaxError("attributes without :: in %r" % rest)
    is_param = any(a == "parameter" for a in attrs)
    dim_attr = None
    for a in attrs:
        m = re.match(r"dimension\s*\((.*)\)$", a)
        if m:
            dim_attr = parse_dims(m.group(1))
    for it in split_top(items_text):
        m = re.match(r"^([a-z_][a-z_0-9]*)\s*(\((.*)\))?\s*(\*\s*\d+)?\s*(=(.*))?$", it, re.S)
        if not m:
            raise SyntaxError("declaration item %r" % it)
        nm = m.group(1)
        s = unit.syms.get(nm) or Sym(nm, typ)
        s.type, s.charlen = typ, clen
        if m.group(4) and typ == "char":
            s.charlen = int(m.group(4).strip("* "))
        if m.group(2):
            s.dims = parse_dims(m.group(3))
        elif dim_attr:
            s.dims = list(dim_attr)
        if s.dims and any(d == ("def",) for d in s.dims):
            s.deferred = True
        if "allocatable" in attrs:
            s.allocatable = True
            s.deferred = True
        if "save" in attrs:
            s.save = True
        if "external" in attrs:
            s.external = True
            s.kind = "proc"
        if m.group(5):
            val = parse_expr(m.group(6).strip())
            if is_param:
                s.param = val
            else:
                s.init = val
                s.save = True
        elif is_param:
            raise SyntaxError("parameter without value %r" % it)
        unit.syms[nm] = s


def implicit_type(name):
    return "int" if name[0] in "ijklmn" else "real"


# --------------------------------------------------------------------------
# unit structure: split statements into program units
# --------------------------------------------------------------------------

class Program:
    def __init__(self):
        self.modules = {}
        self.procs = {}     # external + module procedures by name
        self.order = []     # units in definition order


def build_units(stmts, prog):
    i = 0
    stack = []

    def cur():
        return stack[-1] if stack else None

    while i < len(stmts):
        st = stmts[i]
        s = st.text
        i += 1
        m = re.match(r"^module\s+([a-z_0-9]+)$", s)
        if m and not s.startswith("module procedure"):
            u = Unit("module", m.group(1))
            prog.modules[u.name] = u
            prog.order.append(u)
            stack.append(u)
            continue
        m = re.match(r"^(?:recursive\s+)?subroutine\s+([a-z_0-9]+)\s*(?:\((.*)\))?$", s)
        if m:
            args = [a.strip() for a in (m.group(2) or "").split(",") if a.strip()]
            host = cur()
            u = Unit("subroutine", m.group(1), args, host if host and host.kind != "module" else None)
            u.module = host.name if host and host.kind == "module" else (host.module if host else None)
            if host:
                host.contains.append(u)
            prog.order.append(u)
            if host is None or host.kind == "module":
                prog.procs[u.name] = u
            stack.append(u)
            continue
        m = re.match(r"^(?:(integer|real|complex|logical|double\s+precision)\s+)?function\s+([a-z_0-9]+)"
                     r"\s*\((.*?)\)\s*(?:result\s*\(\s*([a-z_0-9]+)\s*\))?$", s)
        if m:
            args = [a.strip() for a in m.group(3).split(",") if a.strip()]
            host = cur()
            u = Unit("function", m.group(2), args, host if host and host.kind != "module" else None)
            u.module = host.name if host and host.kind == "module" else (host.module if host else None)
            u.result = m.group(4) or m.group(2)
            if m.group(1):
                u.rtype = base_type(m.group(1))[0]
            if host:
                host.contains.append(u)
            prog.order.append(u)
            if host is None or host.kind == "module":
                prog.procs[u.name] = u
            stack.append(u)
            continue
        if re.match(r"^program\b", s):
            # the main program becomes a procedure without arguments
            u = Unit("subroutine", s.split()[1] if len(s.split()) > 1 else "main")
            prog.order.append(u)
            prog.procs[u.name] = u
            stack.append(u)
            continue
        m = re.match(r"^interface(?:\s+([a-z_0-9]+))?$", s)
        if m:
            # interface block: record generic name -> specifics and the bodies
            gname = m.group(1)
            u = cur()
            specifics = []
            while True:
                st2 = stmts[i]
                i += 1
                if re.match(r"^end\s*interface", st2.text):
                    break
                mm = re.match(r"^(?:subroutine|(?:\w+\s+)?function)\s+([a-z_0-9]+)\s*(?:\((.*)\))?", st2.text)
                if mm:
                    args = [a.strip() for a in (mm.group(2) or "").split(",") if a.strip()]
                    iu = Unit("subroutine", mm.group(1), args)
                    specifics.append(mm.group(1))
                    while True:
                        st3 = stmts[i]
                        i += 1
                        if re.match(r"^end\b", st3.text):
                            break
                        tm = TYPE_RE.match(st3.text)
                        if tm:
                            parse_decl(iu, tm.group(1), tm.group(2))
                    u.iface_units[mm.group(1)] = iu
            if gname:
                u.generics[gname] = specifics
            continue
        if s == "contains":
            continue
        if re.match(r"^end(\s*(module|subroutine|function|program)\b.*)?$", s) and \
                not re.match(r"^end\s*(if|do|where|select|interface)\b", s):
            stack.pop()
            continue
        u = cur()
        if u is None:
            raise SyntaxError("statement outside a unit: %r" % st)
        u.body_stmts.append(st)
    return prog


# --------------------------------------------------------------------------
# statements of a unit body: declarations, then an executable tree
# --------------------------------------------------------------------------

def classify_decls(u, prog):
    exec_stmts = []
    for st in u.body_stmts:
        s = st.text
        m = re.match(r"^use\s+([a-z_0-9]+)", s)
        if m:
            u.uses.append(m.group(1))
            continue
        if s == "implicit none":
            u.implicit_none = True
            continue
        if s.startswith("implicit "):
            continue
        tm = TYPE_RE.match(s)
        if tm and not re.match(r"^(real|integer|complex|logical)\s*\(", s) and \
                not re.match(r"^\w+\s+function\b", s):
            rest = tm.group(2)
            if rest.strip().startswith("(") and tm.group(1).startswith("character") is False:
                pass
            parse_decl(u, tm.group(1), rest)
            continue
        if tm and re.match(r"^(real|integer|complex|logical)\s*\(\s*(kind\s*=\s*)?\d+\s*\)", s):
            mm = re.match(r"^(real|integer|complex|logical)\s*\(\s*(?:kind\s*=\s*)?(\d+)\s*\)(.*)$", s)
            parse_decl(u, mm.group(1), mm.group(3))
            continue
        m = re.match(r"^external\s+(.*)$", s)
        if m:
            for nm in split_top(m.group(1).replace("::", "")):
                sy = u.syms.get(nm) or Sym(nm, implicit_type(nm))
                sy.external, sy.kind = True, "proc"
                u.syms[nm] = sy
            continue
        m = re.match(r"^save\b(.*)$", s)
        if m:
            names = split_top(m.group(1).replace("::", ""))
            if not names:
                u.save_all = True
            for nm in names:
                sy = u.syms.get(nm.strip("/ ")) or Sym(nm, implicit_type(nm))
                sy.save = True
                u.syms[nm] = sy
            continue
        m = re.match(r"^parameter\s*\((.*)\)$", s)
        if m:
            for it in split_top(m.group(1)):
                nm, val = [x.strip() for x in it.split("=", 1)]
                sy = u.syms.get(nm) or Sym(nm, implicit_type(nm))
                sy.param = parse_expr(val)
                u.syms[nm] = sy
            continue
        m = re.match(r"^dimension\s+(.*)$", s)
        if m:
            for it in split_top(m.group(1).replace("::", "")):
                mm = re.match(r"([a-z_0-9]+)\s*\((.*)\)$", it)
                sy = u.syms.get(mm.group(1)) or Sym(mm.group(1), implicit_type(mm.group(1)))
                sy.dims = parse_dims(mm.group(2))
                u.syms[mm.group(1)] = sy
            continue
        if re.match(r"^(namelist|intent|intrinsic|format|data|sequence|private|public|!\$)", s) or \
                re.match(r"^\d*\s*format\s*\(", s):
            if s.startswith("data"):
                raise SyntaxError("data statements are not supported: %r" % st)
            continue
        if re.match(r"^format\s*\(", s):
            continue
        exec_stmts.append(st)
    return exec_stmts


class Node:
    def __init__(self, kind, **kw):
        self.kind = kind
        self.label = None
        self.__dict__.update(kw)


def parse_exec(stmts):
    """Build the statement tree (if/do/where blocks) from the flat list."""
    pos = [0]

    def block(terms):
        out = []
        while pos[0] < len(stmts):
            st = stmts[pos[0]]
            s = st.text
            for t in terms:
                if re.match(t, s):
                    return out, st
            pos[0] += 1
            node = one(st)
            if node is not None:
                node.label = st.label
                node.src = st
                out.append(node)
        return out, None

    def one(st):
        s = st.text
        # construct name prefix  name: do ...
        cname = None
        m = re.match(r"^([a-z_][a-z_0-9]*)\s*:\s*(do\b.*|if\s*\(.*)$", s)
        if m:
            cname, s = m.group(1), m.group(2)
        m = re.match(r"^if\s*\((.*)$", s)
        if m:
            k = match_paren(s, s.index("("))
            cond = s[s.index("(") + 1:k]
            rest = s[k + 1:].strip()
            if rest == "then":
                arms = []
                c = parse_expr(cond)
                while True:
                    body, term = block([r"^else\s*if\s*\(", r"^else$", r"^end\s*if\b"])
                    arms.append((c, body))
                    pos[0] += 1
                    if term is None:
                        raise SyntaxError("unterminated if at %r" % st)
                    t = term.text
                    if re.match(r"^else\s*if", t):
                        kk = match_paren(t, t.index("("))
                        c = parse_expr(t[t.index("(") + 1:kk])
                        continue
                    if t == "else":
                        ebody, term2 = block([r"^end\s*if\b"])
                        pos[0] += 1
                        return Node("if", arms=arms, orelse=ebody)
                    return Node("if", arms=arms, orelse=[])
            inner = one(Stmt(rest, None, st.file, st.line))
            inner.src = st
            return Node("if", arms=[(parse_expr(cond), [inner])], orelse=[])
        m = re.match(r"^do\s+while\s*\((.*)\)$", s)
        if m:
            body, term = block([r"^end\s*do\b", r"^enddo\b"])
            pos[0] += 1
            return Node("dowhile", cond=parse_expr(m.group(1)), body=body, name=cname)
        m = re.match(r"^do\s+(\d+\s+)?([a-z_][a-z_0-9]*)\s*=\s*(.*)$", s)
        if m:
            if m.group(1):
                raise SyntaxError("labelled DO not supported: %r" % st)
            parts = split_top(m.group(3))
            body, term = block([r"^end\s*do\b", r"^enddo\b"])
            pos[0] += 1
            return Node("do", var=m.group(2), lo=parse_expr(parts[0]), hi=parse_expr(parts[1]),
                        step=parse_expr(parts[2]) if len(parts) > 2 else None, body=body, name=cname)
        if s == "do":
            body, term = block([r"^end\s*do\b", r"^enddo\b"])
            pos[0] += 1
            return Node("dowhile", cond=N("log", True), body=body, name=cname)
        m = re.match(r"^where\s*\((.*)$", s)
        if m:
            k = match_paren(s, s.index("("))
            mask = parse_expr(s[s.index("(") + 1:k])
            rest = s[k + 1:].strip()
            if not rest:
                raise SyntaxError("block where not supported: %r" % st)
            a = assignment(rest, st)
            return Node("where", mask=mask, lhs=a.lhs, rhs=a.rhs)
        m = re.match(r"^call\s+([a-z_][a-z_0-9]*)\s*(\((.*)\))?$", s)
        if m:
            args = EParser(m.group(3)).arglist() if m.group(2) else []
            if m.group(2):
                p = EParser(m.group(3))
                args = p.arglist()
                if not p.done():
                    raise SyntaxError("call args %r" % s)
            return Node("call", name=m.group(1), args=args)
        if s in ("return",):
            return Node("return")
        if re.match(r"^stop\b", s):
            return Node("stop")
        if s == "continue":
            return Node("nop")
        m = re.match(r"^exit(?:\s+([a-z_0-9]+))?$", s)
        if m:
            return Node("exit", name=m.group(1))
        m = re.match(r"^cycle(?:\s+([a-z_0-9]+))?$", s)
        if m:
            return Node("cycle", name=m.group(1))
        m = re.match(r"^go\s*to\s+(\d+)$", s)
        if m:
            return Node("goto", target=m.group(1))
        m = re.match(r"^(allocate|deallocate)\s*\((.*)\)$", s)
        if m:
            p = EParser(m.group(2))
            items = p.arglist()
            return Node(m.group(1), items=items)
        m = re.match(r"^(read|write)\s*\((.*)$", s)
        if m:
            k = match_paren(s, s.index("("))
            ctl = io_control(s[s.index("(") + 1:k])
            items = s[k + 1:].strip()
            return Node(m.group(1), ctl=ctl, items=io_items(items))
        m = re.match(r"^print\b", s)
        if m:
            return Node("nop")
        m = re.match(r"^(open|close|inquire|rewind|backspace|flush)\s*\((.*)\)$", s)
        if m:
            return Node(m.group(1), ctl=EParser(m.group(2)).arglist())
        if re.match(r"^(end\s*if|end\s*do|enddo|endif|else)\b", s):
            raise SyntaxError("unbalanced block statement %r" % st)
        return assignment(s, st)

    def assignment(s, st):
        k = find_top(s, "=")
        if k < 0 or s[k + 1:k + 2] == "=" or s[k - 1:k] in "<>/=":
            raise SyntaxError("unsupported statement: %r" % st)
        return Node("assign", lhs=parse_expr(s[:k].strip()), rhs=parse_expr(s[k + 1:].strip()))

    body, term = block([])
    return body


def io_control(text):
    """An I/O control list: unit, format, keyword items; '*' stands for the default unit or format."""
    out = []
    for it in split_top(text):
        m = re.match(r"^([a-z]+)\s*=\s*(.*)$", it)
        if m and not it.startswith(("'", '"')):
            val = m.group(2).strip()
            out.append(N("kw", m.group(1), N("star") if val == "*" else parse_expr(val)))
        elif it == "*":
            out.append(N("star"))
        else:
            out.append(parse_expr(it))
    return out


def io_items(text):
    """An I/O list: expressions and implied-do groups (list, var, lo, hi[, st])."""
    out = []
    for it in split_top(text):
        out.append(io_item(it))
    return out


def io_item(it):
    it = it.strip()
    if it.startswith("(") and match_paren(it, 0) == len(it) - 1:
        inner = it[1:-1]
        parts = split_top(inner)
        # implied do: the last parts are  v = lo, hi[, st]
        for j in range(len(parts) - 1, 0, -1):
            m = re.match(r"^([a-z_][a-z_0-9]*)\s*=\s*(.*)$", parts[j])
            if m and find_top(parts[j], "=") >= 0 and "==" not in parts[j]:
                bounds = [m.group(2)] + parts[j + 1:]
                return ("do", [io_item(p) for p in parts[:j]], m.group(1),
                        parse_expr(bounds[0]), parse_expr(bounds[1]),
                        parse_expr(bounds[2]) if len(bounds) > 2 else None)
    return ("e", parse_expr(it))


# --------------------------------------------------------------------------
# code generation
# --------------------------------------------------------------------------

INTRINSIC_ELEMENTAL = {"abs", "sqrt", "exp", "log", "log10", "sin", "cos", "tan", "tanh", "sinh",
                       "cosh", "atan", "asin", "acos", "atan2", "max", "min", "mod", "sign", "int",
                       "nint", "real", "float", "dble", "cmplx", "dcmplx", "conjg", "aimag", "dimag",
                       "dreal", "amax1", "amin1", "dmax1", "dmin1", "dsqrt", "dexp", "dabs", "iabs",
                       "ifix", "idint", "sngl", "dfloat", "cabs", "csqrt", "cexp", "char", "ichar",
                       "dsin", "dcos", "dtanh", "datan", "datan2", "dlog", "alog", "dsign", "isign",
                       "max0", "min0"}
INTRINSIC_OTHER = {"maxval", "minval", "sum", "maxloc", "minloc", "size", "allocated", "present",
                   "huge", "tiny", "epsilon", "trim", "len", "len_trim", "index", "adjustl",
                   "product", "any", "all", "count", "lbound", "ubound", "dot_product"}
C_RESERVED = set()


class GenError(Exception):
    pass


class Ctx:
    """Per-unit generation state."""

    def __init__(self, gen, unit):
        self.g, self.u = gen, unit
        self.tmp = 0
        self.pre = []          # statements hoisted before the current one
        self.labels_used = set()
        self.loops = []        # (fortran name or None, cycle label, exit label)
        self.frees = []

    def newtmp(self, prefix="t"):
        self.tmp += 1
        return "_%s%d" % (prefix, self.tmp)


class Gen:
    def __init__(self, prog):
        self.p = prog
        self.out = []
        self.externals = {}
        self.unresolved = set()
        self.resolve_units()

    # ---- symbol resolution ------------------------------------------------

    def resolve_units(self):
        for u in self.p.order:
            u.exec_stmts = classify_decls(u, self.p)
        for u in self.p.order:
            if u.kind == "module":
                for s in u.syms.values():
                    s.module = u.name
        for u in self.p.order:
            if u.kind in ("subroutine", "function"):
                for a in u.args:
                    if a not in u.syms:
                        if u.implicit_none and not self.module_has(u, a):
                            raise SyntaxError("undeclared dummy %s in %s" % (a, u.name))
                        u.syms[a] = Sym(a, implicit_type(a))
                    u.syms[a].dummy = True
                    if u.syms[a].dims and any(d == ("def",) for d in u.syms[a].dims) and \
                            not u.syms[a].allocatable:
                        u.syms[a].assumed_shape = True
                if u.kind == "function":
                    rs = u.syms.get(u.result) or Sym(u.result, u.rtype or implicit_type(u.name))
                    if u.rtype:
                        rs.type = u.rtype
                    u.syms[u.result] = rs
                    u.rtype = rs.type
        for u in self.p.order:
            if u.kind in ("subroutine", "function"):
                u.tree = parse_exec(u.exec_stmts)

    def module_has(self, u, name):
        return self.lookup_module(u, name) is not None

    def lookup_module(self, u, name, seen=None):
        seen = seen or set()
        chain = []
        x = u
        while x is not None:
            chain.append(x)
            x = x.host
        mods = []
        for x in chain:
            mods.extend(x.uses)
            if x.module:
                mods.append(x.module)
        for mn in mods:
            if mn in seen:
                continue
            seen.add(mn)
            mod = self.p.modules.get(mn)
            if mod is None:
                continue
            if name in mod.syms:
                return mod.syms[name]
            r = self.lookup_module(mod, name, seen)
            if r is not None:
                return r
        return None

    def lookup(self, u, name):
        x = u
        while x is not None:
            if name in x.syms:
                return x.syms[name], x
            x = x.host
        s = self.lookup_module(u, name)
        if s is not None:
            return s, None
        return None, None

    def generic_specifics(self, u, name):
        x = u
        mods = []
        while x is not None:
            if name in x.generics:
                return x.generics[name], x
            mods.extend(x.uses)
            if x.module:
                mods.append(x.module)
            x = x.host
        seen = set()
        while mods:
            mn = mods.pop()
            if mn in seen or mn not in self.p.modules:
                continue
            seen.add(mn)
            m = self.p.modules[mn]
            if name in m.generics:
                return m.generics[name], m
            mods.extend(m.uses)
        return None, None

    def cname_var(self, sym, owner):
        if sym.module:
            return "m_%s" % sym.name
        if sym.dummy and not sym.dims and sym.type != "char" and not (owner and owner.kind == "function"
                                                                       and sym.name == owner.result):
            return "(*a_%s)" % sym.name
        if sym.dummy and sym.type == "char":
            return "a_%s" % sym.name
        return "v_%s" % sym.name

    # ---- expression typing ------------------------------------------------

    def var_sym(self, c, name):
        s, owner = self.lookup(c.u, name)
        if s is None:
            if c.u.implicit_none and not self.implicit_ok(c.u):
                raise GenError("undeclared %s in %s" % (name, c.u.name))
            s = Sym(name, implicit_type(name))
            c.u.syms[name] = s
            owner = c.u
        return s, owner

    def implicit_ok(self, u):
        return False

    def is_array(self, c, name):
        s, _ = self.lookup(c.u, name)
        return s is not None and s.dims is not None and s.kind == "var" and s.param is None

    def rank_of(self, c, e):
        """Rank of an expression (0 for scalars)."""
        k = e.k
        if k in ("num", "str", "log", "cplx"):
            return 0
        if k == "paren":
            return self.rank_of(c, e.a)
        if k == "name":
            s, _ = self.lookup(c.u, e.a)
            if s is not None and s.dims and s.param is None and s.kind == "var":
                return len(s.dims)
            return 0
        if k == "ref":
            if self.is_array(c, e.a):
                return sum(1 for x in e.b if x.k == "sec")
            fn = e.a
            if fn in INTRINSIC_ELEMENTAL and not self.user_proc(c, fn):
                return max([self.rank_of(c, x) for x in e.b if x.k != "kw"] or [0])
            if fn in ("maxloc", "minloc"):
                return 1
            return 0
        if k == "bin":
            return max(self.rank_of(c, e.b), self.rank_of(c, e.c))
        if k == "un":
            return self.rank_of(c, e.b)
        if k == "sec":
            return 1
        raise GenError("rank of %r" % e)

    def user_proc(self, c, name):
        s, _ = self.lookup(c.u, name)
        if s is not None and (s.kind == "proc" or s.external):
            return True
        if name in self.p.procs:
            return True
        return False

    def type_of(self, c, e):
        k = e.k
        if k == "num":
            return e.b
        if k == "str":
            return "char"
        if k == "log":
            return "logical"
        if k == "cplx":
            return "complex"
        if k == "paren":
            return self.type_of(c, e.a)
        if k == "name":
            s, _ = self.var_sym(c, e.a)
            return s.type if s.type != "real4" else "real"
        if k == "ref":
            if self.is_array(c, e.a):
                s, _ = self.lookup(c.u, e.a)
                if e.c is not None:
                    return "char"
                return s.type if s.type != "real4" else "real"
            s, _ = self.lookup(c.u, e.a)
            if s is not None and s.type == "char" and not s.dims:
                return "char"  # substring
            return self.func_type(c, e)
        if k == "bin":
            op = e.a
            if op in ("==", "/=", "<", ">", "<=", ">=", ".and.", ".or.", ".eqv.", ".neqv."):
                return "logical"
            if op == "//":
                return "char"
            return self.promote_t(self.type_of(c, e.b), self.type_of(c, e.c), op)
        if k == "un":
            if e.a == ".not.":
                return "logical"
            return self.type_of(c, e.b)
        raise GenError("type of %r" % e)

    @staticmethod
    def promote_t(a, b, op=None):
        rank = {"logical": 0, "int": 0, "real": 1, "real4": 1, "complex": 2}
        if op == "**" and a == "int" and b == "int":
            return "int"
        return a if rank[a] >= rank[b] else b if rank[b] > rank[a] else a

    def func_type(self, c, e):
        fn = e.a
        args = [x for x in e.b if x.k != "kw"]
        s, owner = self.lookup(c.u, fn)
        if self.user_proc(c, fn):
            if fn in self.p.procs and self.p.procs[fn].kind == "function":
                return self.p.procs[fn].rtype
            if s is not None:
                return s.type
            return implicit_type(fn)
        at = [self.type_of(c, x) for x in args]
        if fn in ("abs", "dabs", "cabs"):
            return "real" if at[0] == "complex" else at[0]
        if fn in ("sqrt", "exp", "log", "sin", "cos", "tanh", "tan", "sinh", "cosh", "csqrt", "cexp",
                  "dsqrt", "dexp", "dlog", "dsin", "dcos", "dtanh"):
            return at[0] if at[0] != "int" else "real"
        if fn in ("log10", "atan", "asin", "acos", "atan2", "datan", "datan2", "alog"):
            return "real"
        if fn in ("max", "min", "amax1", "amin1", "dmax1", "dmin1", "max0", "min0"):
            t = "int"
            for x in at:
                t = self.promote_t(t, x)
            return t
        if fn in ("mod", "sign", "dsign", "isign"):
            t = at[0]
            for x in at[1:]:
                t = self.promote_t(t, x)
            return t
        if fn in ("int", "nint", "ifix", "idint", "iabs", "ichar", "size", "len", "len_trim", "index",
                  "lbound", "ubound", "count"):
            return "int"
        if fn in ("real", "float", "dble", "aimag", "dimag", "dreal", "sngl", "dfloat", "huge", "tiny",
                  "epsilon"):
            return "real"
        if fn in ("cmplx", "dcmplx", "conjg"):
            return "complex"
        if fn in ("maxval", "minval", "sum", "product", "dot_product"):
            return at[0]
        if fn in ("maxloc", "minloc"):
            return "int"
        if fn in ("allocated", "present", "any", "all"):
            return "logical"
        if fn in ("char", "trim", "adjustl"):
            return "char"
        if s is not None:
            return s.type
        self.unresolved.add(fn)
        return implicit_type(fn)

    # ---- C expressions ----------------------------------------------------

    def conv(self, code, frm, to):
        if frm == to or to is None:
            return code
        if to in ("real", "real4"):
            if frm == "complex":
                return "(%s).re" % code
            return "(double)(%s)" % code
        if to == "complex":
            if frm == "complex":
                return code
            return "cx_r((double)(%s))" % code
        if to in ("int", "logical"):
            if frm == "complex":
                return "(int)((%s).re)" % code
            if frm in ("real", "real4"):
                return "(int)(%s)" % code
            return code
        if to == "char":
            return code
        raise GenError("conversion %s -> %s" % (frm, to))

    def ex(self, c, e, idx=None):
        """C code and type of expression e.  idx: zero-based loop index names
        for the section dimensions of an array-valued expression (element
        of the result at those indices)."""
        k = e.k
        if k == "num":
            if e.b == "int":
                return e.a, "int"
            v = e.a.lower().replace("d", "e")
            if v.startswith("."):
                v = "0" + v
            if "." not in v and "e" not in v:
                v += ".0"
            v = re.sub(r"\.e", ".0e", v)
            if v.endswith("."):
                v += "0"
            return v, "real"
        if k == "str":
            return '"%s"' % e.a.replace("\\", "\\\\").replace('"', '\\"'), "char"
        if k == "log":
            return ("1" if e.a else "0"), "logical"
        if k == "cplx":
            a, ta = self.ex(c, e.a, idx)
            b, tb = self.ex(c, e.b, idx)
            return "cx_mk((double)(%s), (double)(%s))" % (a, b), "complex"
        if k == "paren":
            a, t = self.ex(c, e.a, idx)
            return "(%s)" % a, t
        if k == "name":
            return self.ex_name(c, e, idx)
        if k == "ref":
            return self.ex_ref(c, e, idx)
        if k == "un":
            a, t = self.ex(c, e.b, idx)
            if e.a == ".not.":
                return "(!%s)" % a, "logical"
            if t == "complex":
                return "cx_neg(%s)" % a, t
            return "(-%s)" % a, t
        if k == "bin":
            return self.ex_bin(c, e, idx)
        raise GenError("expression %r" % e)

    def ex_bin(self, c, e, idx):
        op = e.a
        a, ta = self.ex(c, e.b, idx)
        b, tb = self.ex(c, e.c, idx)
        ta = "real" if ta == "real4" else ta
        tb = "real" if tb == "real4" else tb
        if op in (".and.", ".or."):
            return "(%s %s %s)" % (a, "&&" if op == ".and." else "||", b), "logical"
        if op in (".eqv.", ".neqv."):
            return "((!!%s) %s (!!%s))" % (a, "==" if op == ".eqv." else "!=", b), "logical"
        if op == "//":
            return "fstr_cat(%s, %s)" % (a, b), "char"
        if op in ("==", "/=", "<", ">", "<=", ">="):
            cop = {"==": "==", "/=": "!=", "<": "<", ">": ">", "<=": "<=", ">=": ">="}[op]
            if ta == "char" or tb == "char":
                return "(fstr_cmp(%s, %s) %s 0)" % (a, b, cop), "logical"
            if "complex" in (ta, tb):
                t = "complex"
                a2, b2 = self.conv(a, ta, t), self.conv(b, tb, t)
                if cop == "==":
                    return "cx_eq(%s, %s)" % (a2, b2), "logical"
                if cop == "!=":
                    return "(!cx_eq(%s, %s))" % (a2, b2), "logical"
                raise GenError("complex ordering")
            t = self.promote_t(ta, tb)
            return "(%s %s %s)" % (self.conv(a, ta, t), cop, self.conv(b, tb, t)), "logical"
        if op == "**":
            return self.ex_pow(e, a, ta, b, tb)
        t = self.promote_t(ta, tb)
        if t == "complex":
            if ta == "complex" and tb == "complex":
                fn = {"+": "cx_add", "-": "cx_sub", "*": "cx_mul", "/": "cx_div"}[op]
                return "%s(%s, %s)" % (fn, a, b), t
            if ta != "complex":  # real op complex
                ra = self.conv(a, ta, "real")
                fn = {"+": "cx_radd", "-": "cx_rsub", "*": "cx_rmul", "/": "cx_rdiv"}[op]
                return "%s(%s, %s)" % (fn, ra, b), t
            rb = self.conv(b, tb, "real")
            fn = {"+": "cx_addr", "-": "cx_subr", "*": "cx_mulr", "/": "cx_divr"}[op]
            return "%s(%s, %s)" % (fn, a, rb), t
        if t == "int" and op == "/":
            return "(%s / %s)" % (a, b), "int"
        return "(%s %s %s)" % (self.conv(a, ta, t), op, self.conv(b, tb, t)), t

    def ex_pow(self, e, a, ta, b, tb):
        if tb == "int":
            if e.c.k == "num" or (e.c.k == "un" and e.c.b.k == "num"):
                n = int(e.c.a) if e.c.k == "num" else -int(e.c.b.a)
                if ta == "int":
                    return "ipow(%s, %d)" % (a, n), "int"
                if ta == "complex":
                    return "cx_powi(%s, %d)" % (a, n), "complex"
                return "powi_%s(%s)" % (("m%d" % -n) if n < 0 else n, a) if -8 <= n <= 8 \
                    else "powi_n(%s, %d)" % (a, n), "real"
            if ta == "int":
                return "ipow(%s, %s)" % (a, b), "int"
            if ta == "complex":
                return "cx_powi(%s, %s)" % (a, b), "complex"
            return "powi_n(%s, %s)" % (a, b), "real"
        if ta == "complex" or tb == "complex":
            return "cx_pow(%s, %s)" % (self.conv(a, ta, "complex"), self.conv(b, tb, "complex")), "complex"
        return "pow(%s, %s)" % (self.conv(a, ta, "real"), self.conv(b, tb, "real")), "real"

    def param_code(self, c, s, owner):
        code, t = self.ex(c, s.param)
        want = s.type if s.type != "real4" else "real"
        return "(%s)" % self.conv(code, t, want), want

    def ex_name(self, c, e, idx):
        s, owner = self.var_sym(c, e.a)
        if s.param is not None:
            return self.param_code(c, s, owner)
        t = s.type if s.type != "real4" else "real"
        if s.kind == "proc" and not s.dims:
            raise GenError("procedure name used as value: %s" % e.a)
        if s.dims:
            if idx is None:
                raise GenError("array %s used as scalar in %s" % (e.a, c.u.name))
            d = self.desc(c, s, owner)
            subs = ["%s.lb[%d] + %s" % (d, j, idx[j]) for j in range(len(s.dims))]
            return self.elem(d, s, subs), t
        if owner is not None and owner.kind == "function" and e.a == owner.name and owner is not c.u \
                and False:
            pass
        return self.cname_var(s, owner), t

    def desc(self, c, s, owner):
        if s.module:
            return "m_%s" % s.name
        return "v_%s" % s.name

    def elem(self, d, s, subs):
        ct = CT[s.type]
        return "(*(%s*)FAT%d(&%s, sizeof(%s), %s))" % (ct, len(subs), d, ct, ", ".join("(long)(%s)" % x for x in subs))

    def ex_ref(self, c, e, idx):
        name = e.a
        s, owner = self.lookup(c.u, name)
        if s is not None and s.dims and s.kind == "var" and s.param is None:
            return self.ex_arrayref(c, e, s, owner, idx)
        if s is not None and s.type == "char" and not s.dims and s.kind == "var" and s.param is None:
            # substring
            base = self.cname_var(s, owner)
            lo = self.ex(c, e.b[0].a)[0] if e.b[0].a is not None else "1"
            hi = self.ex(c, e.b[0].b)[0] if e.b[0].b is not None else "-1"
            return "fstr_sub(%s, %s, %s)" % (base, lo, hi), "char"
        return self.ex_call(c, e, idx)

    def ex_arrayref(self, c, e, s, owner, idx):
        d = self.desc(c, s, owner)
        subs, q = [], 0
        if len(e.b) != len(s.dims):
            raise GenError("rank mismatch for %s in %s" % (s.name, c.u.name))
        for j, x in enumerate(e.b):
            if x.k == "sec":
                if idx is None:
                    raise GenError("section of %s used as scalar" % s.name)
                lo = self.ex(c, x.a)[0] if x.a is not None else "%s.lb[%d]" % (d, j)
                st = self.ex(c, x.c)[0] if x.c is not None else None
                subs.append("(%s) + %s%s" % (lo, idx[q], (" * (%s)" % st) if st else ""))
                q += 1
            else:
                code, t = self.ex(c, x)
                if self.rank_of(c, x) > 0:
                    raise GenError("vector subscript in %s" % s.name)
                subs.append(self.conv(code, t, "int"))
        t = s.type if s.type != "real4" else "real"
        return self.elem(d, s, subs), t

    def section_shape(self, c, e):
        """Extents (C code) of an array-valued expression, or None if scalar."""
        k = e.k
        if k == "paren":
            return self.section_shape(c, e.a)
        if k == "name":
            s, owner = self.lookup(c.u, e.a)
            if s is not None and s.dims and s.param is None and s.kind == "var":
                d = self.desc(c, s, owner)
                return ["%s.n[%d]" % (d, j) for j in range(len(s.dims))]
            return None
        if k == "ref":
            s, owner = self.lookup(c.u, e.a)
            if s is not None and s.dims and s.param is None and s.kind == "var":
                d = self.desc(c, s, owner)
                out = []
                for j, x in enumerate(e.b):
                    if x.k == "sec":
                        lo = self.ex(c, x.a)[0] if x.a is not None else "%s.lb[%d]" % (d, j)
                        hi = self.ex(c, x.b)[0] if x.b is not None else "(%s.lb[%d] + %s.n[%d] - 1)" % (d, j, d, j)
                        st = self.ex(c, x.c)[0] if x.c is not None else "1"
                        out.append("fext((long)(%s), (long)(%s), (long)(%s))" % (lo, hi, st))
                return out or None
            if e.a in INTRINSIC_ELEMENTAL:
                for x in e.b:
                    if x.k != "kw":
                        sh = self.section_shape(c, x)
                        if sh:
                            return sh
            return None
        if k == "bin":
            return self.section_shape(c, e.b) or self.section_shape(c, e.c)
        if k == "un":
            return self.section_shape(c, e.b)
        return None

    def intr_args(self, c, e, idx):
        return [self.ex(c, x, idx) for x in e.b if x.k != "kw"]

    def ex_call(self, c, e, idx):
        fn = e.a
        if self.user_proc(c, fn) or (fn not in INTRINSIC_ELEMENTAL and fn not in INTRINSIC_OTHER):
            return self.ex_userfunc(c, e, idx)
        kw = {x.a: x.b for x in e.b if x.k == "kw"}
        if fn in ("maxval", "minval", "sum", "maxloc", "minloc", "product"):
            return self.ex_reduction(c, e, idx)
        if fn == "size":
            arr = e.b[0]
            s, owner = self.lookup(c.u, arr.a)
            d = self.desc(c, s, owner)
            if len(e.b) > 1:
                dim = self.ex(c, e.b[1] if e.b[1].k != "kw" else e.b[1].b)[0]
                return "(int)%s.n[(%s) - 1]" % (d, dim), "int"
            return "(int)fsize(&%s)" % d, "int"
        if fn in ("lbound", "ubound"):
            s, owner = self.lookup(c.u, e.b[0].a)
            d = self.desc(c, s, owner)
            dim = self.ex(c, e.b[1] if e.b[1].k != "kw" else e.b[1].b)[0]
            if fn == "lbound":
                return "(int)%s.lb[(%s) - 1]" % (d, dim), "int"
            return "(int)(%s.lb[(%s) - 1] + %s.n[(%s) - 1] - 1)" % (d, dim, d, dim), "int"
        if fn == "allocated":
            s, owner = self.lookup(c.u, e.b[0].a)
            return "(%s.p != 0)" % self.desc(c, s, owner), "logical"
        if fn == "present":
            return "(a_%s != 0)" % e.b[0].a, "logical"
        if fn in ("huge",):
            t = self.type_of(c, e.b[0])
            return ("2147483647" if t == "int" else "DBL_MAX"), ("int" if t == "int" else "real")
        if fn == "tiny":
            return "DBL_MIN", "real"
        if fn == "epsilon":
            return "DBL_EPSILON", "real"
        args = self.intr_args(c, e, idx)
        codes = [a for a, _ in args]
        types = [("real" if t == "real4" else t) for _, t in args]
        t0 = types[0] if types else None
        if fn in ("abs", "dabs", "iabs", "cabs"):
            if t0 == "complex":
                return "cx_abs(%s)" % codes[0], "real"
            if t0 == "int":
                return "iabs_(%s)" % codes[0], "int"
            return "fabs(%s)" % codes[0], "real"
        if fn in ("sqrt", "dsqrt", "csqrt", "exp", "dexp", "cexp", "log", "dlog", "alog", "sin", "dsin",
                  "cos", "dcos", "tanh", "dtanh", "tan", "sinh", "cosh"):
            base = fn.lstrip("dc") if fn not in ("cos", "cosh", "dcos") else fn[1:] if fn == "dcos" else fn
            base = {"dsqrt": "sqrt", "csqrt": "sqrt", "dexp": "exp", "cexp": "exp", "dlog": "log",
                    "alog": "log", "dsin": "sin", "dcos": "cos", "dtanh": "tanh"}.get(fn, fn)
            if t0 == "complex":
                return "cx_%s(%s)" % (base, codes[0]), "complex"
            return "%s(%s)" % (base, self.conv(codes[0], t0, "real")), "real"
        if fn in ("log10", "atan", "datan", "asin", "acos"):
            base = {"datan": "atan"}.get(fn, fn)
            return "%s(%s)" % (base, self.conv(codes[0], t0, "real")), "real"
        if fn in ("atan2", "datan2"):
            return "atan2(%s, %s)" % (self.conv(codes[0], t0, "real"), self.conv(codes[1], types[1], "real")), "real"
        if fn in ("max", "min", "amax1", "amin1", "dmax1", "dmin1", "max0", "min0"):
            t = "int"
            for x in types:
                t = self.promote_t(t, x)
            f = "fmax_" if fn in ("max", "amax1", "dmax1", "max0") else "fmin_"
            f = ("i" + f) if t == "int" else f
            acc = self.conv(codes[0], types[0], t)
            for cc, tt in zip(codes[1:], types[1:]):
                acc = "%s(%s, %s)" % (f, acc, self.conv(cc, tt, t))
            return acc, t
        if fn == "mod":
            t = self.promote_t(types[0], types[1])
            if t == "int":
                return "(%s %% %s)" % (codes[0], codes[1]), "int"
            return "fmod(%s, %s)" % (self.conv(codes[0], types[0], "real"), self.conv(codes[1], types[1], "real")), "real"
        if fn in ("sign", "dsign", "isign"):
            t = self.promote_t(types[0], types[1])
            if t == "int":
                return "isign_(%s, %s)" % (codes[0], codes[1]), "int"
            return "fsign_(%s, %s)" % (self.conv(codes[0], types[0], "real"), self.conv(codes[1], types[1], "real")), "real"
        if fn in ("int", "ifix", "idint"):
            if t0 == "complex":
                return "(int)((%s).re)" % codes[0], "int"
            return "(int)(%s)" % codes[0], "int"
        if fn == "nint":
            return "(int)lround(%s)" % codes[0], "int"
        if fn in ("real", "float", "dble", "dreal", "sngl", "dfloat"):
            if t0 == "complex":
                return "(%s).re" % codes[0], "real"
            return "(double)(%s)" % codes[0], "real"
        if fn in ("aimag", "dimag"):
            return "(%s).im" % codes[0], "real"
        if fn == "conjg":
            return "cx_conj(%s)" % codes[0], "complex"
        if fn in ("cmplx", "dcmplx"):
            if len(codes) == 1:
                return self.conv(codes[0], t0, "complex"), "complex"
            return "cx_mk((double)(%s), (double)(%s))" % (self.conv(codes[0], t0, "real"),
                                                           self.conv(codes[1], types[1], "real")), "complex"
        if fn == "char":
            return "fstr_char(%s)" % codes[0], "char"
        if fn == "ichar":
            return "(int)(unsigned char)(%s)[0]" % codes[0], "int"
        if fn == "trim":
            return "fstr_trim(%s)" % codes[0], "char"
        if fn == "adjustl":
            return "fstr_adjustl(%s)" % codes[0], "char"
        if fn in ("len",):
            return "(int)strlen(%s)" % codes[0], "int"
        if fn in ("len_trim",):
            return "(int)strlen(fstr_trim(%s))" % codes[0], "int"
        if fn == "index":
            return "fstr_index(%s, %s)" % (codes[0], codes[1]), "int"
        raise GenError("intrinsic %s not supported" % fn)

    def ex_reduction(self, c, e, idx):
        fn = e.a
        args = [x for x in e.b if x.k != "kw"]
        if any(x.k == "kw" for x in e.b):
            raise GenError("%s with keyword arguments not supported" % fn)
        src = args[0]
        sh = self.section_shape(c, src)
        if sh is None:
            raise GenError("%s of a scalar" % fn)
        r = len(sh)
        t = self.type_of(c, src)
        t = "real" if t == "real4" else t
        lv = [c.newtmp("i") for _ in range(r)]
        ext = [c.newtmp("n") for _ in range(r)]
        acc = c.newtmp("r")
        pre = c.pre
        for j in range(r):
            pre.append("long %s = %s;" % (ext[j], sh[j]))
        el_code, el_t = self.ex(c, src, lv)
        if fn in ("maxval", "minval", "sum", "product"):
            if fn == "sum":
                pre.append("%s %s = %s;" % (CT[t], acc, "cx_r(0.0)" if t == "complex" else "0"))
            elif fn == "product":
                pre.append("%s %s = 1;" % (CT[t], acc))
            else:
                init = {"maxval": ("-DBL_MAX", "-2147483647-1"), "minval": ("DBL_MAX", "2147483647")}[fn]
                pre.append("%s %s = %s;" % (CT[t], acc, init[0] if t == "real" else init[1]))
            loops, close = self.loop_nest(lv, ext)
            pre.extend(loops)
            if fn == "sum":
                if t == "complex":
                    pre.append("%s = cx_add(%s, %s);" % (acc, acc, el_code))
                else:
                    pre.append("%s = %s + %s;" % (acc, acc, el_code))
            elif fn == "product":
                pre.append("%s = %s * %s;" % (acc, acc, el_code))
            elif fn == "maxval":
                pre.append("{ %s _x = %s; if (_x > %s) %s = _x; }" % (CT[t], el_code, acc, acc))
            else:
                pre.append("{ %s _x = %s; if (_x < %s) %s = _x; }" % (CT[t], el_code, acc, acc))
            pre.extend(close)
            return acc, t
        # maxloc / minloc: an integer vector of rank r (first location in array element order)
        best = c.newtmp("b")
        pre.append("int %s[%d] = {%s};" % (acc, r, ", ".join("0" for _ in range(r))))
        pre.append("%s %s = %s; int %s_set = 0;" % (CT[t], best, "0", best))
        loops, close = self.loop_nest(lv, ext)
        pre.extend(loops)
        cmp = ">" if fn == "maxloc" else "<"
        pre.append("{ %s _x = %s; if (!%s_set || _x %s %s) { %s = _x; %s_set = 1; %s } }" % (
            CT[t], el_code, best, cmp, best, best, best,
            " ".join("%s[%d] = (int)(%s + 1);" % (acc, j, lv[j]) for j in range(r))))
        pre.extend(close)
        if idx is None:
            raise GenError("maxloc used as scalar")
        return "%s[%s]" % (acc, idx[0]), "int"

    @staticmethod
    def loop_nest(lv, ext):
        """Column-major loop nest: the first index varies fastest."""
        loops, close = [], []
        for j in reversed(range(len(lv))):
            loops.append("for (long %s = 0; %s < %s; ++%s) {" % (lv[j], lv[j], ext[j], lv[j]))
            close.append("}")
        return loops, close

    # ---- calls ----------------------------------------------------------

    def resolve_proc(self, c, name, args):
        specs, owner = self.generic_specifics(c.u, name)
        if specs:
            # pick the specific whose first dummy's rank matches the actual's
            r0 = self.rank_of(c, args[0]) if args else 0
            whole = args and args[0].k == "name" and self.is_array(c, args[0].a)
            for sp in specs:
                iu = owner.iface_units.get(sp)
                target = self.p.procs.get(sp)
                dummy0 = (target or iu).args[0] if (target or iu) and (target or iu).args else None
                ds = (target or iu).syms.get(dummy0) if dummy0 else None
                drank = ds.rank if ds else 0
                if (drank > 0) == (r0 > 0 or bool(whole)):
                    return sp
            return specs[0]
        return name

    def proc_unit(self, name):
        return self.p.procs.get(name)

    def ex_userfunc(self, c, e, idx):
        name = self.resolve_proc(c, e.a, [x for x in e.b if x.k != "kw"])
        pu = self.proc_unit(name)
        if pu is None:
            s, _ = self.lookup(c.u, e.a)
            t = s.type if s is not None else implicit_type(e.a)
            t = "real" if t == "real4" else t
            self.externals.setdefault(name, ("func", t, len(e.b)))
            args = self.actual_args(c, None, e.b)
            return "f_%s(%s)" % (name, ", ".join(args)), t
        if pu.kind != "function":
            raise GenError("%s is not a function" % name)
        args = self.actual_args(c, pu, e.b)
        return "f_%s(%s)" % (name, ", ".join(args)), pu.rtype

    def actual_args(self, c, pu, args):
        out = []
        for j, a in enumerate(args):
            if a.k == "kw":
                raise GenError("keyword arguments to user procedures not supported")
            dummy = pu.syms.get(pu.args[j]) if pu is not None and j < len(pu.args) else None
            out.append(self.actual(c, a, dummy))
        return out

    def actual(self, c, a, dummy):
        """Pass by reference: a pointer to the actual's storage, or to a temporary."""
        t = self.type_of(c, a)
        if t == "char":
            code, _ = self.ex(c, a)
            return "(char*)(%s)" % code
        if dummy is not None and dummy.assumed_shape:
            # assumed-shape dummy: pass a descriptor
            if a.k == "name" and self.is_array(c, a.a):
                s, owner = self.lookup(c.u, a.a)
                return "&%s" % self.desc(c, s, owner)
            raise GenError("section passed to an assumed-shape dummy")
        r = self.rank_of(c, a)
        if a.k == "name":
            s, owner = self.var_sym(c, a.a)
            if s.param is not None:
                code, ct = self.param_code(c, s, owner)
                tmp = c.newtmp("a")
                c.pre.append("%s %s = %s;" % (CT[ct], tmp, code))
                return "&%s" % tmp
            if s.dims:
                return "%s.p" % self.desc(c, s, owner)
            if s.kind == "proc":
                return "(void*)f_%s" % s.name
            cv = self.cname_var(s, owner)
            if cv.startswith("(*a_"):
                return "a_%s" % s.name
            return "&%s" % cv
        if a.k == "ref" and self.is_array(c, a.a) and r == 0:
            code, _ = self.ex(c, a)
            return "&%s" % code
        if a.k == "ref" and self.is_array(c, a.a) and r > 0:
            # a section: contiguous leading-dimension sections pass the address of the first element
            s, owner = self.lookup(c.u, a.a)
            d = self.desc(c, s, owner)
            secs = [x.k == "sec" for x in a.b]
            nsec = sum(secs)
            if secs[:nsec] == [True] * nsec and all(x.a is None and x.b is None for x in a.b[:nsec - 1]):
                lo = []
                for j, x in enumerate(a.b):
                    if x.k == "sec":
                        lo.append(self.ex(c, x.a)[0] if x.a is not None else "%s.lb[%d]" % (d, j))
                    else:
                        lo.append(self.conv(*self.ex(c, x), "int"))
                return "&%s" % self.elem(d, s, lo)
            # non-contiguous section: copy in to a temporary, copy back after the call
            sh = self.section_shape(c, a)
            tmp = c.newtmp("sec")
            ct = CT[s.type]
            lv = [c.newtmp("i") for _ in sh]
            ext = [c.newtmp("n") for _ in sh]
            for j in range(len(sh)):
                c.pre.append("long %s = %s;" % (ext[j], sh[j]))
            n = " * ".join(ext)
            c.pre.append("%s* %s = (%s*)malloc(sizeof(%s) * (size_t)(%s));" % (ct, tmp, ct, ct, n))
            off = lv[0]
            stride = ext[0]
            for j in range(1, len(sh)):
                off = "%s + %s * %s" % (off, stride, lv[j])
                stride = "%s * %s" % (stride, ext[j])
            loops, close = self.loop_nest(lv, ext)
            el, _ = self.ex(c, a, lv)
            c.pre.extend(loops)
            c.pre.append("%s[%s] = %s;" % (tmp, off, el))
            c.pre.extend(close)
            c.post.extend(loops)
            c.post.append("%s = %s[%s];" % (el, tmp, off))
            c.post.extend(close)
            c.post_free.append(tmp)
            return tmp
        if r > 0:
            # array expression: evaluate into a temporary array
            sh = self.section_shape(c, a)
            tmp = c.newtmp("x")
            ct = CT[t if t != "real4" else "real"]
            n = " * ".join("(%s)" % x for x in sh)
            c.pre.append("%s* %s = (%s*)malloc(sizeof(%s) * (size_t)(%s));" % (ct, tmp, ct, ct, n))
            lv = [c.newtmp("i") for _ in sh]
            ext = [c.newtmp("n") for _ in sh]
            for j in range(len(sh)):
                c.pre.append("long %s = %s;" % (ext[j], sh[j]))
            loops, close = self.loop_nest(lv, ext)
            c.pre.extend(loops)
            code, _ = self.ex(c, a, lv)
            off = lv[0]
            stride = ext[0]
            for j in range(1, len(sh)):
                off = "%s + %s * %s" % (off, stride, lv[j])
                stride = "%s * %s" % (stride, ext[j])
            c.pre.append("%s[%s] = %s;" % (tmp, off, code))
            c.pre.extend(close)
            c.post_free.append(tmp)
            return tmp
        code, et = self.ex(c, a)
        want = dummy.type if dummy is not None else et
        want = "real" if want == "real4" else want
        tmp = c.newtmp("a")
        c.pre.append("%s %s = %s;" % (CT[want], tmp, self.conv(code, et, want)))
        return "&%s" % tmp

    # ---- statements -----------------------------------------------------

    def flush_pre(self, c, ind, lines):
        if c.pre:
            lines.append(ind + "{")
            for p in c.pre:
                lines.append(ind + "  " + p)
            c.pre = []
            return True
        return False

    def emit_stmt(self, c, st, ind, lines):
        c.pre = []
        c.post = []
        c.post_free = []
        if st.label:
            lines.append("L%s:;" % st.label)
        body = []
        try:
            self.emit_core(c, st, ind + "  ", body)
        except (GenError, SyntaxError, KeyError) as ex:
            src = getattr(st, "src", None)
            raise GenError("%s: %s" % (src, ex))
        if c.pre or c.post_free or c.post:
            lines.append(ind + "{")
            for p in c.pre:
                lines.append(ind + "  " + p)
            lines.extend(body)
            for p in c.post:
                lines.append(ind + "  " + p)
            for f in c.post_free:
                lines.append(ind + "  free(%s);" % f)
            lines.append(ind + "}")
        else:
            lines.extend([ln[2:] if ln.startswith("  ") else ln for ln in body])
        c.pre = []
        c.post = []
        c.post_free = []

    def emit_block(self, c, stmts, ind, lines):
        for st in stmts:
            self.emit_stmt(c, st, ind, lines)

    def emit_core(self, c, st, ind, lines):
        k = st.kind
        if k == "assign":
            self.emit_assign(c, st.lhs, st.rhs, ind, lines)
        elif k == "call":
            self.emit_call(c, st, ind, lines)
        elif k == "if":
            first = True
            for cond, body in st.arms:
                code, t = self.ex(c, cond)
                lines.append(ind + ("if (%s) {" if first else "} else if (%s) {") % code)
                inner = []
                saved = c.pre
                c.pre = []
                self.emit_block(c, body, ind + "  ", inner)
                c.pre = saved
                lines.extend(inner)
                first = False
            if st.orelse:
                lines.append(ind + "} else {")
                inner = []
                saved = c.pre
                c.pre = []
                self.emit_block(c, st.orelse, ind + "  ", inner)
                c.pre = saved
                lines.extend(inner)
            lines.append(ind + "}")
            # a condition in an else-if arm that needed hoisted statements is not supported
        elif k == "do":
            self.emit_do(c, st, ind, lines)
        elif k == "dowhile":
            cl, xl = c.newtmp("cyc"), c.newtmp("ext")
            c.loops.append((st.name, cl, xl))
            saved = c.pre
            c.pre = []
            code, _ = self.ex(c, st.cond)
            if c.pre:
                raise GenError("do while condition needs temporaries")
            c.pre = saved
            lines.append(ind + "while (%s) {" % code)
            inner = []
            self.emit_block(c, st.body, ind + "  ", inner)
            lines.extend(inner)
            lines.append(ind + "  %s:;" % cl)
            lines.append(ind + "}")
            lines.append(ind + "%s:;" % xl)
            c.loops.pop()
        elif k == "exit":
            lines.append(ind + "goto %s;" % self.find_loop(c, st.name)[2])
        elif k == "cycle":
            lines.append(ind + "goto %s;" % self.find_loop(c, st.name)[1])
        elif k == "goto":
            lines.append(ind + "goto L%s;" % st.target)
            c.labels_used.add(st.target)
        elif k == "return":
            lines.append(ind + "goto _exit;")
        elif k == "stop":
            lines.append(ind + "f_stop_();")
        elif k == "nop":
            lines.append(ind + ";")
        elif k == "where":
            sh = self.section_shape(c, st.lhs)
            lv = [c.newtmp("i") for _ in sh]
            ext = [c.newtmp("n") for _ in sh]
            for j in range(len(sh)):
                lines.append(ind + "long %s = %s;" % (ext[j], sh[j]))
            loops, close = self.loop_nest(lv, ext)
            lines.extend(ind + x for x in loops)
            m, _ = self.ex(c, st.mask, lv)
            lhs, lt = self.ex(c, st.lhs, lv)
            rhs, rt = self.ex(c, st.rhs, lv)
            lines.append(ind + "if (%s) %s = %s;" % (m, lhs, self.conv(rhs, rt, lt)))
            lines.extend(ind + x for x in close)
        elif k in ("allocate", "deallocate"):
            self.emit_alloc(c, st, ind, lines)
        elif k == "read":
            self.emit_io(c, st, ind, lines, read=True)
        elif k == "write":
            self.emit_io(c, st, ind, lines, read=False)
        elif k == "open":
            kw = {}
            for j, x in enumerate(st.ctl):
                if x.k == "kw":
                    kw[x.a] = x.b
                elif j == 0:
                    kw["unit"] = x
            unit = self.conv(*self.ex(c, kw["unit"]), "int")
            fname = self.ex(c, kw["file"])[0] if "file" in kw else '""'
            form = self.ex(c, kw["form"])[0] if "form" in kw else '"formatted"'
            status = self.ex(c, kw["status"])[0] if "status" in kw else '"unknown"'
            call = "fio_open(%s, %s, %s, %s)" % (unit, fname, form, status)
            if "err" in kw:
                lab = kw["err"].a
                c.labels_used.add(lab)
                lines.append(ind + "if (%s != 0) goto L%s;" % (call, lab))
            else:
                lines.append(ind + "if (%s != 0) f_ioerror_();" % call)
        elif k == "close":
            x = st.ctl[0]
            if x.k == "kw":
                x = x.b
            lines.append(ind + "fio_close(%s);" % self.conv(*self.ex(c, x), "int"))
        elif k == "inquire":
            kw = {x.a: x.b for x in st.ctl if x.k == "kw"}
            if "file" in kw and "exist" in kw:
                tgt, _ = self.ex(c, kw["exist"])
                lines.append(ind + "%s = fio_exists(%s);" % (tgt, self.ex(c, kw["file"])[0]))
            else:
                lines.append(ind + ";")
        elif k in ("rewind", "backspace", "flush"):
            lines.append(ind + ";")
        else:
            raise GenError("statement kind %s" % k)

    def find_loop(self, c, name):
        if not c.loops:
            raise GenError("exit/cycle outside a loop")
        if name is None:
            return c.loops[-1]
        for lp in reversed(c.loops):
            if lp[0] == name:
                return lp
        raise GenError("no loop named %s" % name)

    def emit_do(self, c, st, ind, lines):
        s, owner = self.var_sym(c, st.var)
        var = self.cname_var(s, owner)
        lo, tlo = self.ex(c, st.lo)
        hi, thi = self.ex(c, st.hi)
        step = self.ex(c, st.step)[0] if st.step is not None else "1"
        trip = c.newtmp("trip")
        stv = c.newtmp("st")
        lines.append(ind + "{ long %s = (long)(%s); long %s = ((long)(%s) - (long)(%s) + %s) / %s;" % (
            stv, step, trip, hi, lo, stv, stv))
        lines.append(ind + "  %s = (int)(%s);" % (var, lo))
        cl, xl = c.newtmp("cyc"), c.newtmp("ext")
        c.loops.append((st.name, cl, xl))
        lines.append(ind + "  for (; %s > 0; --%s, %s += (int)%s) {" % (trip, trip, var, stv))
        inner = []
        saved = c.pre
        c.pre = []
        self.emit_block(c, st.body, ind + "    ", inner)
        c.pre = saved
        lines.extend(inner)
        lines.append(ind + "    %s:;" % cl)
        lines.append(ind + "  }")
        lines.append(ind + "  %s:;" % xl)
        lines.append(ind + "}")
        c.loops.pop()

    def emit_assign(self, c, lhs, rhs, ind, lines):
        lr = self.rank_of(c, lhs)
        if lhs.k == "name":
            s, owner = self.var_sym(c, lhs.a)
            if owner is not None and owner.kind == "function" and lhs.a == owner.name:
                s = owner.syms[owner.result]
        else:
            s, owner = self.lookup(c.u, lhs.a)
        lt = self.type_of(c, lhs)
        if lt == "char":
            code, _ = self.ex(c, rhs)
            tgt = self.ex(c, lhs)[0] if lhs.k == "name" else None
            if lhs.k != "name":
                raise GenError("character substring assignment")
            size = s.charlen or 1
            lines.append(ind + "fstr_assign(%s, %d, %s);" % (tgt, size, code))
            return
        if lr == 0:
            code, rt = self.ex(c, rhs)
            if self.rank_of(c, rhs) > 0:
                raise GenError("array assigned to scalar")
            tgt, _ = self.ex(c, lhs)
            lines.append(ind + "%s = %s;" % (tgt, self.conv(code, rt, lt)))
            return
        sh = self.section_shape(c, lhs)
        lv = [c.newtmp("i") for _ in sh]
        ext = [c.newtmp("n") for _ in sh]
        # aliasing: the target array appears on the right with different subscripts -> temporary
        alias = self.aliases(lhs, rhs)
        for j in range(len(sh)):
            c.pre.append("long %s = %s;" % (ext[j], sh[j]))
        if alias:
            ct = CT[lt]
            tmp = c.newtmp("al")
            n = " * ".join(ext)
            c.pre.append("%s* %s = (%s*)malloc(sizeof(%s) * (size_t)(%s));" % (ct, tmp, ct, ct, n))
            off = lv[0]
            stride = ext[0]
            for j in range(1, len(sh)):
                off = "%s + %s * %s" % (off, stride, lv[j])
                stride = "%s * %s" % (stride, ext[j])
            loops, close = self.loop_nest(lv, ext)
            lines.extend(ind + x for x in loops)
            code, rt = self.ex(c, rhs, lv if self.rank_of(c, rhs) else None)
            lines.append(ind + "%s[%s] = %s;" % (tmp, off, self.conv(code, rt, lt)))
            lines.extend(ind + x for x in close)
            lines.extend(ind + x for x in loops)
            tgt, _ = self.ex(c, lhs, lv)
            lines.append(ind + "%s = %s[%s];" % (tgt, tmp, off))
            lines.extend(ind + x for x in close)
            lines.append(ind + "free(%s);" % tmp)
            return
        loops, close = self.loop_nest(lv, ext)
        # scalar right-hand sides are evaluated once
        if self.rank_of(c, rhs) == 0:
            code, rt = self.ex(c, rhs)
            tmp = c.newtmp("s")
            c.pre.append("%s %s = %s;" % (CT[lt], tmp, self.conv(code, rt, lt)))
            lines.extend(ind + x for x in loops)
            tgt, _ = self.ex(c, lhs, lv)
            lines.append(ind + "%s = %s;" % (tgt, tmp))
            lines.extend(ind + x for x in close)
            return
        lines.extend(ind + x for x in loops)
        tgt, _ = self.ex(c, lhs, lv)
        code, rt = self.ex(c, rhs, lv)
        lines.append(ind + "%s = %s;" % (tgt, self.conv(code, rt, lt)))
        lines.extend(ind + x for x in close)

    def aliases(self, lhs, rhs):
        name = lhs.a
        lsub = repr(lhs.b) if lhs.k == "ref" else None
        found = []

        def walk(e):
            if e is None or not isinstance(e, N):
                return
            if e.k in ("name", "ref") and e.a == name:
                sub = repr(e.b) if e.k == "ref" else None
                if sub != lsub:
                    found.append(e)
            if e.k == "ref":
                for x in e.b:
                    walk(x)
            for x in (e.b, e.c) if e.k in ("bin",) else (e.b,) if e.k == "un" else (e.a,) if e.k == "paren" else ():
                walk(x)
        walk(rhs)
        return bool(found)

    def emit_call(self, c, st, ind, lines):
        name = st.name
        if name in ("exit",):
            lines.append(ind + "f_stop_();")
            return
        if name in ("flush",):
            lines.append(ind + ";")
            return
        name = self.resolve_proc(c, name, st.args)
        pu = self.proc_unit(name)
        if pu is None:
            self.externals.setdefault(name, ("sub", None, len(st.args)))
        args = self.actual_args(c, pu, st.args)
        lines.append(ind + "f_%s(%s);" % (name, ", ".join(args)))

    def emit_alloc(self, c, st, ind, lines):
        stat = None
        for x in st.items:
            if x.k == "kw" and x.a == "stat":
                stat = x.b
        for x in st.items:
            if x.k == "kw":
                continue
            if st.kind == "deallocate":
                s, owner = self.lookup(c.u, x.a)
                lines.append(ind + "fd_free(&%s);" % self.desc(c, s, owner))
                continue
            s, owner = self.lookup(c.u, x.a)
            d = self.desc(c, s, owner)
            lbs, ubs = [], []
            for y in x.b:
                if y.k == "sec":
                    lbs.append(self.conv(*self.ex(c, y.a), "int"))
                    ubs.append(self.conv(*self.ex(c, y.b), "int"))
                else:
                    lbs.append("1")
                    ubs.append(self.conv(*self.ex(c, y), "int"))
            lines.append(ind + "{ long _lb[%d] = {%s}, _ub[%d] = {%s}; fd_alloc(&%s, sizeof(%s), %d, _lb, _ub); }" % (
                len(lbs), ", ".join(lbs), len(ubs), ", ".join(ubs), d, CT[s.type], len(lbs)))
        if stat is not None:
            tgt, _ = self.ex(c, stat)
            lines.append(ind + "%s = 0;" % tgt)

    def emit_io(self, c, st, ind, lines, read):
        unit = None
        fmt = None
        err = end = None
        pos = 0
        for x in st.ctl:
            if x.k == "kw":
                if x.a == "unit":
                    unit = x.b
                elif x.a in ("fmt",):
                    fmt = x.b
                elif x.a == "err":
                    err = x.b.a
                elif x.a == "end":
                    end = x.b.a
                elif x.a == "nml":
                    fmt = N("str", "nml")
                continue
            if pos == 0:
                unit = x
            elif pos == 1:
                fmt = x
            pos += 1
        if read and fmt is not None and fmt.k == "name" and not st.items:
            lines.append(ind + "; /* namelist read: no namelist input is given to the translated reference */")
            return
        if read and fmt is not None and fmt.k == "star":
            ucode = "5" if unit is None or unit.k == "star" else self.conv(*self.ex(c, unit), "int")
            lines.append(ind + "fio_lbegin(%s);" % ucode)
            for it in st.items:
                self.emit_list_item(c, it, ind, lines)
            lab = err or end
            if lab:
                c.labels_used.add(lab)
                lines.append(ind + "if (fio_lend() != 0) goto L%s;" % lab)
            else:
                lines.append(ind + "if (fio_lend() != 0) f_ioerror_();")
            return
        if fmt is not None or unit is None or unit.k == "star" or (unit.k == "num" and unit.a in ("6", "5")):
            # formatted or list-directed: numeric scalar items go to a hook, the rest is dropped
            if read:
                # one character item under (aW) or (a): the record's first W
                # characters (all of it for (a)), blank-padded
                m = re.fullmatch(r"\(\s*a(\d*)\s*\)", fmt.a.strip().lower()) if fmt is not None and fmt.k == "str" \
                    else None
                if m and len(st.items) == 1 and st.items[0][0] == "e" and st.items[0][1].k == "name" \
                        and self.type_of(c, st.items[0][1]) == "char":
                    e = st.items[0][1]
                    s_, _ = self.lookup(c.u, e.a)
                    ucode = "5" if unit is None or unit.k == "star" else self.conv(*self.ex(c, unit), "int")
                    code, _ = self.ex(c, e)
                    lines.append(ind + "if (fio_aread(%s, %s, %d, %s) != 0) f_ioerror_();" % (
                        ucode, code, s_.charlen or 1, m.group(1) or "-1"))
                    return
                lines.append(ind + "f_unsupported_(\"formatted read\");")
                return
            ucode = "-1" if unit is None or unit.k == "star" else self.conv(*self.ex(c, unit), "int")
            items = []
            for it in st.items:
                if it[0] != "e":
                    continue
                try:
                    t = self.type_of(c, it[1])
                    if t in ("int", "real", "logical", "real4") and self.rank_of(c, it[1]) == 0:
                        code, tt = self.ex(c, it[1])
                        items.append("fio_fnum((double)(%s));" % code)
                except GenError:
                    pass
            if c.pre:
                c.pre = []
                items = []
            lines.append(ind + "fio_fbegin(%s); %s fio_fend();" % (ucode, " ".join(items)))
            return
        ucode = self.conv(*self.ex(c, unit), "int")
        fn = "fio_r" if read else "fio_w"
        lines.append(ind + "%sbegin(%s);" % (fn, ucode))
        for it in st.items:
            self.emit_io_item(c, it, ind, lines, fn)
        lab = err or end
        if read and (err or end):
            c.labels_used.add(err or end)
            lines.append(ind + "if (fio_rend() != 0) goto L%s;" % (end or err))
        else:
            lines.append(ind + "if (%send() != 0) f_ioerror_();" % fn)

    def emit_list_item(self, c, it, ind, lines):
        if it[0] != "e":
            raise GenError("implied do in a list-directed read")
        e = it[1]
        if self.rank_of(c, e) > 0 or (e.k == "name" and self.is_array(c, e.a)):
            raise GenError("array in a list-directed read")
        t = self.type_of(c, e)
        code, _ = self.ex(c, e)
        if t == "char":
            s, _ = self.lookup(c.u, e.a)
            lines.append(ind + "fio_lchar(%s, %d);" % (code, s.charlen or 1))
            return
        fn = {"int": "fio_lint", "logical": "fio_llog", "real": "fio_lreal", "real4": "fio_lreal4",
              "complex": "fio_lcx"}[t]
        lines.append(ind + "%s(&%s);" % (fn, code))

    def emit_io_item(self, c, it, ind, lines, fn):
        if it[0] == "do":
            _, sub, var, lo, hi, st = it
            s, owner = self.var_sym(c, var)
            v = self.cname_var(s, owner)
            lines.append(ind + "for (%s = %s; %s <= %s; %s += %s) {" % (
                v, self.ex(c, lo)[0], v, self.ex(c, hi)[0], v, self.ex(c, st)[0] if st else "1"))
            for x in sub:
                self.emit_io_item(c, x, ind + "  ", lines, fn)
            lines.append(ind + "}")
            return
        e = it[1]
        t = self.type_of(c, e)
        t = "real" if t == "real4" else t
        es, per = {"int": (4, 1), "logical": (4, 1), "real": (8, 1), "complex": (8, 2), "real4": (4, 1)}[t]
        if e.k == "name" and self.is_array(c, e.a):
            s, owner = self.lookup(c.u, e.a)
            d = self.desc(c, s, owner)
            lines.append(ind + "%sitem_es(%s.p, %d, %d * fsize(&%s));" % (fn, d, es, per, d))
            return
        if self.rank_of(c, e) > 0:
            # an array section or expression: its elements in array element
            # order (the first index fastest)
            sh = self.section_shape(c, e)
            if sh is None:
                raise GenError("array expression in an I/O list")
            lv = [c.newtmp("i") for _ in sh]
            ext = [c.newtmp("n") for _ in sh]
            lines.append(ind + "{")
            for j in range(len(sh)):
                lines.append(ind + "  long %s = %s;" % (ext[j], sh[j]))
            loops, close = self.loop_nest(lv, ext)
            lines.extend(ind + "  " + x for x in loops)
            code, tt = self.ex(c, e, lv)
            if fn == "fio_r":
                lines.append(ind + "  fio_ritem_es(&%s, %d, %d);" % (code, es, per))
            else:
                tmp = c.newtmp("w")
                lines.append(ind + "  { %s %s = %s; fio_witem_es(&%s, %d, %d); }" % (
                    CT[t], tmp, self.conv(code, tt, t), tmp, es, per))
            lines.extend(ind + "  " + x for x in close)
            lines.append(ind + "}")
            return
        if fn == "fio_r":
            code, _ = self.ex(c, e)
            lines.append(ind + "fio_ritem_es(&%s, %d, %d);" % (code, es, per))
        else:
            code, tt = self.ex(c, e)
            tmp = c.newtmp("w")
            lines.append(ind + "{ %s %s = %s; fio_witem_es(&%s, %d, %d); }" % (CT[t], tmp, self.conv(code, tt, t), tmp, es, per))

    # ---- units ----------------------------------------------------------

    def c_decl_type(self, s):
        return CT[s.type]

    def signature(self, u):
        params = []
        for a in u.args:
            s = u.syms[a]
            if s.kind == "proc" or s.external:
                params.append("void* a_%s" % a)
            elif s.type == "char":
                params.append("char* a_%s" % a)
            elif s.assumed_shape:
                params.append("fdesc* a_%s" % a)
            elif s.dims:
                params.append("void* a_%s" % a)
            else:
                params.append("%s* a_%s" % (CT[s.type], a))
        ret = "void" if u.kind == "subroutine" else CT[u.rtype]
        return "%s f_%s(%s)" % (ret, u.name, ", ".join(params) or "void")

    def sigcode(self, u):
        """One character per dummy: i l d f z c scalars, I L D F Z arrays, S assumed shape, P procedure."""
        out = ""
        for a in u.args:
            s = u.syms[a]
            if s.kind == "proc" or s.external:
                out += "P"
            elif s.type == "char":
                out += "c"
            elif s.assumed_shape:
                out += "S"
            else:
                ch = {"int": "i", "logical": "l", "real": "d", "real4": "f", "complex": "z"}[s.type]
                out += ch.upper() if s.dims else ch
        return out

    def dims_code(self, c, s):
        lbs, ubs = [], []
        for d in s.dims:
            lo, hi = d
            lbs.append(self.conv(*self.ex(c, lo), "int"))
            ubs.append(self.conv(*self.ex(c, hi), "int") if hi is not None else "FD_ASSUMED")
        return lbs, ubs

    def emit_unit(self, u):
        c = Ctx(self, u)
        lines = []
        lines.append(self.signature(u) + " {")
        decl = []
        # locals
        for nm, s in u.syms.items():
            if s.param is not None or s.kind == "proc" or s.external:
                continue
            if u.kind == "function" and nm == u.result:
                decl.append("  %s v_%s = %s;" % (CT[s.type], nm, "cx_r(0.0)" if s.type == "complex" else "0"))
                continue
            if s.dummy:
                if s.assumed_shape:
                    decl.append("  fdesc v_%s = *a_%s;" % (nm, nm))
                elif s.dims:
                    decl.append("  fdesc v_%s;" % nm)
                continue
            st = "static " if (s.save or getattr(u, "save_all", False)) else ""
            if s.type == "char":
                init = ""
                if s.init is not None:
                    init = " = %s" % self.ex(c, s.init)[0]
                decl.append("  %schar v_%s[%d]%s;" % (st, nm, (s.charlen or 1) + 1, init))
                continue
            if s.dims:
                decl.append("  %sfdesc v_%s;%s" % (st, nm, " /* allocatable */" if s.allocatable else ""))
                continue
            init = ""
            if s.init is not None:
                code, t = self.ex(c, s.init)
                init = " = %s" % self.conv(code, t, s.type)
            elif not st:
                init = " = %s" % ("cx_r(0.0)" if s.type == "complex" else "0")
            decl.append("  %s%s v_%s%s;" % (st, CT[s.type if s.type != "real4" else "real4"], nm, init))
        lines.extend(decl)
        # explicit-shape dummies and automatic arrays get their descriptors at entry
        autos = []
        for nm, s in u.syms.items():
            if not s.dims or s.param is not None or s.kind == "proc":
                continue
            if s.dummy and not s.assumed_shape:
                lbs, ubs = self.dims_code(c, s)
                lines.append("  { long _lb[%d] = {%s}, _ub[%d] = {%s}; fd_view(&v_%s, a_%s, sizeof(%s), %d, _lb, _ub); }" % (
                    len(lbs), ", ".join(lbs), len(ubs), ", ".join(ubs), nm, nm, CT[s.type], len(lbs)))
            elif not s.dummy and not s.deferred:
                lbs, ubs = self.dims_code(c, s)
                sv = s.save or s.init is not None
                guard = "if (!v_%s.p) " % nm if sv else ""
                lines.append("  %s{ long _lb[%d] = {%s}, _ub[%d] = {%s}; fd_alloc(&v_%s, sizeof(%s), %d, _lb, _ub); }" % (
                    guard, len(lbs), ", ".join(lbs), len(ubs), ", ".join(ubs), nm, CT[s.type], len(lbs)))
                if not sv:
                    autos.append(nm)
            elif not s.dummy and s.allocatable and not s.save:
                lines.append("  memset(&v_%s, 0, sizeof(fdesc));" % nm)
                autos.append(nm)
        body = []
        self.emit_block(c, u.tree, "  ", body)
        lines.extend(body)
        lines.append("  goto _exit;")
        lines.append("_exit:;")
        for nm in autos:
            lines.append("  fd_free(&v_%s);" % nm)
        if u.kind == "function":
            lines.append("  return v_%s;" % u.result)
        lines.append("}")
        # drop labels that are never targets (C warns, harmless) -- keep all
        return lines

    def emit_module(self, m):
        lines = []
        c = Ctx(self, m)
        for nm, s in m.syms.items():
            if s.param is not None or s.kind == "proc":
                continue
            if s.type == "char":
                init = ""
                if s.init is not None:
                    init = " = %s" % self.ex(c, s.init)[0]
                lines.append("char m_%s[%d]%s;" % (nm, (s.charlen or 1) + 1, init))
                continue
            if s.dims:
                if s.deferred:
                    lines.append("fdesc m_%s;" % nm)
                else:
                    lines.append("fdesc m_%s; /* fixed-size module array, allocated by ref_init */" % nm)
                continue
            init = ""
            if s.init is not None:
                code, t = self.ex(c, s.init)
                init = " = %s" % self.conv(code, t, s.type)
                if s.type == "complex":
                    init = " = {%s}" % code
            lines.append("%s m_%s%s;" % (CT[s.type], nm, init))
        return lines

    def module_fixed_arrays(self):
        out = []
        for m in self.p.modules.values():
            c = Ctx(self, m)
            for nm, s in m.syms.items():
                if s.dims and not s.deferred and s.param is None and s.kind == "var":
                    lbs, ubs = self.dims_code(c, s)
                    out.append("  { long _lb[%d] = {%s}, _ub[%d] = {%s}; fd_alloc(&m_%s, sizeof(%s), %d, _lb, _ub); }" % (
                        len(lbs), ", ".join(lbs), len(ubs), ", ".join(ubs), nm, CT[s.type], len(lbs)))
        return out

    def registry(self):
        """Name -> address tables of module variables, for the harness."""
        scal, arr = [], []
        for m in self.p.modules.values():
            for nm, s in m.syms.items():
                if s.param is not None or s.kind != "var":
                    continue
                if s.dims:
                    arr.append('  {"%s", &m_%s, %d, %d},' % (nm, nm, {"int": 0, "real": 1, "complex": 2,
                                                                      "logical": 0, "char": 3, "real4": 4}[s.type],
                                                            len(s.dims)))
                elif s.type != "char":
                    scal.append('  {"%s", &m_%s, %d, 0},' % (nm, nm, {"int": 0, "real": 1, "complex": 2,
                                                                     "logical": 0, "real4": 4}[s.type]))
                else:
                    scal.append('  {"%s", m_%s, 3, %d},' % (nm, nm, s.charlen or 1))
        return scal, arr


PRELUDE = r"""
#include <math.h>
#include <float.h>
#include <stdlib.h>
#include <string.h>
#include <limits.h>
#include "@HEADER@"

long ref_oob_count = 0;
static char ref_sink[64];

static inline cx cx_mk(double a, double b) { cx z; z.re = a; z.im = b; return z; }
static inline cx cx_r(double a) { cx z; z.re = a; z.im = 0.0; return z; }
static inline cx cx_neg(cx a) { return cx_mk(-a.re, -a.im); }
static inline cx cx_conj(cx a) { return cx_mk(a.re, -a.im); }
static inline cx cx_add(cx a, cx b) { return cx_mk(a.re + b.re, a.im + b.im); }
static inline cx cx_sub(cx a, cx b) { return cx_mk(a.re - b.re, a.im - b.im); }
static inline cx cx_mul(cx a, cx b) { return cx_mk(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re); }
/* Smith (1962), Algorithm 116: range-reduced complex division. */
static inline cx cx_div(cx a, cx b) { cx z; double r, d;
  if (fabs(b.re) < fabs(b.im)) { r = b.re / b.im; d = b.re * r + b.im;
    z.re = (a.re * r + a.im) / d; z.im = (a.im * r - a.re) / d; }
  else { r = b.im / b.re; d = b.im * r + b.re;
    z.re = (a.im * r + a.re) / d; z.im = (a.im - a.re * r) / d; }
  return z; }
/* a real operand: gcc lowers the complex operation component-wise */
static inline cx cx_radd(double a, cx b) { return cx_mk(a + b.re, b.im); }
static inline cx cx_rsub(double a, cx b) { return cx_mk(a - b.re, -b.im); }
static inline cx cx_rmul(double a, cx b) { return cx_mk(a * b.re, a * b.im); }
static inline cx cx_rdiv(double a, cx b) { return cx_div(cx_r(a), b); }
static inline cx cx_addr(cx a, double b) { return cx_mk(a.re + b, a.im); }
static inline cx cx_subr(cx a, double b) { return cx_mk(a.re - b, a.im); }
static inline cx cx_mulr(cx a, double b) { return cx_mk(a.re * b, a.im * b); }
static inline cx cx_divr(cx a, double b) { return cx_mk(a.re / b, a.im / b); }
static inline int cx_eq(cx a, cx b) { return a.re == b.re && a.im == b.im; }
static inline double cx_abs(cx a) { return hypot(a.re, a.im); }
static inline cx cx_from(double _Complex z) { return cx_mk(creal(z), cimag(z)); }
static inline double _Complex cx_to(cx a) { return a.re + I * a.im; }
static inline cx cx_sqrt(cx a) { return cx_from(csqrt(cx_to(a))); }
static inline cx cx_exp(cx a) { return cx_from(cexp(cx_to(a))); }
static inline cx cx_log(cx a) { return cx_from(clog(cx_to(a))); }
static inline cx cx_sin(cx a) { return cx_from(csin(cx_to(a))); }
static inline cx cx_cos(cx a) { return cx_from(ccos(cx_to(a))); }
static inline cx cx_tanh(cx a) { return cx_from(ctanh(cx_to(a))); }
static inline cx cx_pow(cx a, cx b) { return cx_from(cpow(cx_to(a), cx_to(b))); }
static inline cx cx_powi(cx a, long n) { cx r = cx_r(1.0); int neg = n < 0; if (neg) n = -n;
  while (n) { if (n & 1) r = cx_mul(r, a); a = cx_mul(a, a); n >>= 1; } return neg ? cx_div(cx_r(1.0), r) : r; }
/* x**n for a constant integer n, as gcc's powi expansion multiplies */
static inline double powi_0(double x) { (void)x; return 1.0; }
static inline double powi_1(double x) { return x; }
static inline double powi_2(double x) { return x * x; }
static inline double powi_3(double x) { return x * x * x; }
static inline double powi_4(double x) { double y = x * x; return y * y; }
static inline double powi_5(double x) { double y = x * x; return y * y * x; }
static inline double powi_6(double x) { double y = x * x; y = y * x; return y * y; }
static inline double powi_7(double x) { double y = x * x; double z = y * x; return z * z * x; }
static inline double powi_8(double x) { double y = x * x; y = y * y; return y * y; }
static inline double powi_n(double x, long n) { double r = 1.0; int neg = n < 0; if (neg) n = -n;
  while (n) { if (n & 1) r *= x; x *= x; n >>= 1; } return neg ? 1.0 / r : r; }
static inline double powi_m1(double x) { return 1.0 / x; }
static inline double powi_m2(double x) { return 1.0 / (x * x); }
static inline double powi_m3(double x) { return 1.0 / (x * x * x); }
static inline double powi_m4(double x) { double y = x * x; return 1.0 / (y * y); }
static inline double powi_m5(double x) { return 1.0 / powi_5(x); }
static inline double powi_m6(double x) { return 1.0 / powi_6(x); }
static inline double powi_m7(double x) { return 1.0 / powi_7(x); }
static inline double powi_m8(double x) { return 1.0 / powi_8(x); }
static inline long ipow(long x, long n) { long r = 1; while (n > 0) { if (n & 1) r *= x; x *= x; n >>= 1; } return r; }
static inline int iabs_(int a) { return a < 0 ? -a : a; }
static inline int ifmax_(int a, int b) { return a > b ? a : b; }
static inline int ifmin_(int a, int b) { return a < b ? a : b; }
/* Fortran MAX/MIN: the later argument wins only when strictly larger/smaller */
static inline double fmax_(double a, double b) { return b > a ? b : a; }
static inline double fmin_(double a, double b) { return b < a ? b : a; }
static inline double fsign_(double a, double b) { return signbit(b) ? -fabs(a) : fabs(a); }
static inline int isign_(int a, int b) { return b < 0 ? -iabs_(a) : iabs_(a); }
static inline long fext(long lo, long hi, long st) { long n = (hi - lo + st) / st; return n > 0 ? n : 0; }
static inline long fsize(const fdesc* d) { long n = 1; for (int k = 0; k < d->rank; ++k) n *= d->n[k]; return n; }

/* Element address from the linear column-major offset, as compiled Fortran
   computes it.  With REF_BOUNDS an offset outside the array's storage is
   counted in ref_oob_count and redirected to a zeroed scratch cell; a
   subscript outside its own dimension that still lands inside the storage
   (the reference's transposed-index fault) is counted in ref_dim_count and
   performed, as the compiled reference performs it. */
long ref_dim_count = 0;
static inline void* fat_off(const fdesc* d, size_t es, long off, int dim_ok) {
#ifdef REF_BOUNDS
  long size = 1;
  for (int k = 0; k < d->rank; ++k) size *= d->n[k];
  if (!d->p || off < 0 || off >= size) { ++ref_oob_count; memset(ref_sink, 0, sizeof ref_sink); return ref_sink; }
  if (!dim_ok) ++ref_dim_count;
#else
  (void)dim_ok;
#endif
  return (char*)d->p + off * (long)es; }
#define CHK(k, i) (((i) - d->lb[k]) >= 0 && ((i) - d->lb[k]) < d->n[k])
static inline void* FAT1(const fdesc* d, size_t es, long i) {
  return fat_off(d, es, (i - d->lb[0]) * d->st[0], CHK(0, i)); }
static inline void* FAT2(const fdesc* d, size_t es, long i, long j) {
  return fat_off(d, es, (i - d->lb[0]) * d->st[0] + (j - d->lb[1]) * d->st[1], CHK(0, i) && CHK(1, j)); }
static inline void* FAT3(const fdesc* d, size_t es, long i, long j, long k) {
  return fat_off(d, es, (i - d->lb[0]) * d->st[0] + (j - d->lb[1]) * d->st[1] + (k - d->lb[2]) * d->st[2],
                 CHK(0, i) && CHK(1, j) && CHK(2, k)); }
static inline void* FAT4(const fdesc* d, size_t es, long i, long j, long k, long l) {
  return fat_off(d, es, (i - d->lb[0]) * d->st[0] + (j - d->lb[1]) * d->st[1] + (k - d->lb[2]) * d->st[2]
                 + (l - d->lb[3]) * d->st[3], CHK(0, i) && CHK(1, j) && CHK(2, k) && CHK(3, l)); }
static inline void* FAT5(const fdesc* d, size_t es, long i, long j, long k, long l, long m) {
  return fat_off(d, es, (i - d->lb[0]) * d->st[0] + (j - d->lb[1]) * d->st[1] + (k - d->lb[2]) * d->st[2]
                 + (l - d->lb[3]) * d->st[3] + (m - d->lb[4]) * d->st[4],
                 CHK(0, i) && CHK(1, j) && CHK(2, k) && CHK(3, l) && CHK(4, m)); }
#undef CHK
"""

RT_HEADER = r"""/* Generated by oracle/f90sub2c.py: runtime types of the translated reference. */
#pragma once
#include <complex.h>
#undef I
#define I _Complex_I
typedef struct { double re, im; } cx;
/* Array descriptor: column-major, bounds lb..lb+n-1, element strides st. */
typedef struct { void* p; int rank; int owned; long lb[7]; long n[7]; long st[7]; } fdesc;
#define FD_ASSUMED (-1)
extern long ref_oob_count;
extern long ref_dim_count;
void fd_view(fdesc* d, void* p, unsigned long es, int rank, const long* lb, const long* ub);
void fd_alloc(fdesc* d, unsigned long es, int rank, const long* lb, const long* ub);
void fd_free(fdesc* d);
/* I/O and runtime hooks implemented by the harness */
int fio_open(int unit, const char* file, const char* form, const char* status);
void fio_close(int unit);
void fio_rbegin(int unit); void fio_ritem_es(void* p, unsigned long es, unsigned long count); int fio_rend(void);
void fio_wbegin(int unit); void fio_witem_es(const void* p, unsigned long es, unsigned long count); int fio_wend(void);
void fio_fbegin(int unit); void fio_fnum(double v); void fio_fend(void);
void fio_lbegin(int unit); void fio_lint(int* p); void fio_llog(int* p); void fio_lreal(double* p);
void fio_lreal4(float* p); void fio_lcx(cx* p); void fio_lchar(char* p, int len); int fio_lend(void);
int fio_aread(int unit, char* p, int len, int width);
int fio_exists(const char* file);
void f_stop_(void);
void f_ioerror_(void);
void f_unsupported_(const char* what);
const char* fstr_cat(const char* a, const char* b);
const char* fstr_char(int c);
const char* fstr_trim(const char* a);
const char* fstr_adjustl(const char* a);
const char* fstr_sub(const char* a, long lo, long hi);
int fstr_cmp(const char* a, const char* b);
int fstr_index(const char* a, const char* b);
void fstr_assign(char* dst, int len, const char* src);
typedef struct { const char* name; void* addr; int type; int rank; } ref_sym;
typedef struct { const char* name; void* fn; int nargs; const char* sig; } ref_proc;
extern const ref_proc ref_procs[];
"""


def main():
    argv = sys.argv[1:]
    defines = {}
    while argv and argv[0] in ("-D", "-P"):
        if argv[0] == "-D":
            defines[argv[1]] = "1"
            argv = argv[2:]
        else:
            f, ln = argv[1].split(":")
            PATCHES.append((f, int(ln), argv[2], argv[3]))
            argv = argv[4:]
    out_c, out_h, srcs = argv[0], argv[1], argv[2:]
    prog = Program()
    for path in srcs:
        build_units(read_source(path, defines), prog)
    gen = Gen(prog)
    units_code = []
    protos = []
    for u in prog.order:
        if u.kind in ("subroutine", "function"):
            protos.append(gen.signature(u) + ";")
            units_code.append(gen.emit_unit(u))
    mod_code = []
    for m in prog.modules.values():
        mod_code.extend(gen.emit_module(m))
    ext_protos = []
    for name, (kind, t, n) in sorted(gen.externals.items()):
        if name in prog.procs:
            continue
        ret = "void" if kind == "sub" else CT[t]
        ext_protos.append("%s f_%s();" % (ret, name))
    scal, arr = gen.registry()
    with open(out_h, "w") as f:
        f.write(RT_HEADER)
        f.write("\n/* translated procedures */\n")
        f.write("\n".join(protos) + "\n")
        # the harness leaves out its stand-ins of procedures translated here
        f.write("".join("#define REF_HAVE_%s 1\n" % nm for nm in sorted(prog.procs)))
        f.write("\n/* procedures the harness provides */\n")
        f.write("\n".join(ext_protos) + "\n")
        f.write("extern const ref_sym ref_scalars[];\nextern const ref_sym ref_arrays[];\nvoid ref_init(void);\n")
    with open(out_c, "w") as f:
        f.write("/* Generated by oracle/f90sub2c.py from the reference sources. Build product: do not edit. */\n")
        f.write(PRELUDE.replace("@HEADER@", out_h.split("/")[-1]))
        f.write("\n/* module variables */\n")
        f.write("\n".join(mod_code) + "\n")
        f.write("\n/* prototypes */\n" + "\n".join(protos) + "\n" + "\n".join(ext_protos) + "\n")
        for lines in units_code:
            f.write("\n".join(lines) + "\n\n")
        f.write("const ref_sym ref_scalars[] = {\n%s\n  {0, 0, 0, 0}};\n" % "\n".join(scal))
        f.write("const ref_sym ref_arrays[] = {\n%s\n  {0, 0, 0, 0}};\n" % "\n".join(arr))
        f.write("void ref_init(void) {\n%s\n}\n" % "\n".join(gen.module_fixed_arrays()))
        f.write("const ref_proc ref_procs[] = {\n%s\n  {0, 0, 0, 0}};\n" % "\n".join(
            '  {"%s", (void*)f_%s, %d, "%s"},' % (u.name, u.name, len(u.args), gen.sigcode(u))
            for u in prog.order if u.kind in ("subroutine", "function")))
    if gen.unresolved:
        sys.stderr.write("f90sub2c: unresolved names treated as external functions: %s\n" %
                         ", ".join(sorted(gen.unresolved)))


if __name__ == "__main__":
    try:
        main()
    except (SyntaxError, GenError) as ex:
        sys.stderr.write("f90sub2c: %s\n" % ex)
        sys.exit(1)
