"""Test infrastructure: an interpreter for the Fortran 95 subset the BSAM 1.2
reference is written in, so that the reference's own source runs here
(no Fortran compiler exists on these machines) and its outputs pin the C
oracle.  Only tests/golden/make_reference_golden.py uses it, to write golden
fixtures; nothing in the library, the bench or the GPU tests imports it.

Semantics follow the Fortran standard as gfortran implements it without
fast-math: every REAL(8) operation is one IEEE double operation, evaluated
left to right with the standard's precedence, no fused multiply-adds; SUM
adds in array element order; integer division truncates; arguments are
passed by reference (array sections as views, copy-in/copy-out for
non-contiguous actuals of explicit-shape dummies); derived-type assignment
copies components (pointer components by association); locals with
initialisers are SAVEd.  Python hooks can stand in for named procedures
(the harness's QInit, output routines).
"""
import math
import re

import numpy as np

# --------------------------------------------------------------------------
# source -> statements


def _strip_comment(line):
    out, q = [], None
    for ch in line:
        if q:
            out.append(ch)
            if ch == q:
                q = None
        elif ch in "'\"":
            q = ch
            out.append(ch)
        elif ch == "!":
            break
        else:
            out.append(ch)
    return "".join(out)


def _split_semicolons(s):
    parts, cur, q = [], [], None
    for ch in s:
        if q:
            cur.append(ch)
            if ch == q:
                q = None
        elif ch in "'\"":
            q = ch
            cur.append(ch)
        elif ch == ";":
            parts.append("".join(cur))
            cur = []
        else:
            cur.append(ch)
    parts.append("".join(cur))
    return [p for p in parts if p.strip()]


def statements(text, fname):
    """(file, line, label, text) per statement: comments removed,
    continuation lines joined, ';' split."""
    out = []
    lines = text.split("\n")
    i = 0
    while i < len(lines):
        start = i + 1
        s = _strip_comment(lines[i]).rstrip()
        i += 1
        while s.endswith("&"):
            s = s[:-1]
            nxt = _strip_comment(lines[i]).strip() if i < len(lines) else ""
            i += 1
            if nxt.startswith("&"):
                nxt = nxt[1:]
            s = s + " " + nxt if not s.endswith(" ") else s + nxt
            s = s.rstrip()
        for part in _split_semicolons(s):
            part = part.strip()
            m = re.match(r"^(\d+)\s+(.*)$", part)
            label = None
            if m:
                label, part = int(m.group(1)), m.group(2)
            out.append((fname, start, label, part))
    return out


# --------------------------------------------------------------------------
# tokens

_TOK = re.compile(r"""
  (?P<ws>\s+)
 |(?P<str>'(?:[^']|'')*'|"(?:[^"]|"")*")
 |(?P<real>(?:\d+\.\d*(?![a-z]+\.)(?:[ed][+-]?\d+)?|\.\d+(?:[ed][+-]?\d+)?|\d+[ed][+-]?\d+)(?:_\w+)?)
 |(?P<int>\d+(?:_\w+)?)
 |(?P<dotop>\.(?:and|or|not|eqv|neqv|eq|ne|lt|le|gt|ge|true|false)\.)
 |(?P<name>[a-z_]\w*)
 |(?P<op>\*\*|//|==|/=|<=|>=|=>|::|\(/|/\)|[-+*/<>=(),:%])
""", re.X | re.I)


class Tok:
    __slots__ = ("k", "v")

    def __init__(self, k, v):
        self.k, self.v = k, v

    def __repr__(self):
        return f"{self.k}:{self.v}"


def tokenize(s):
    toks, pos = [], 0
    while pos < len(s):
        m = _TOK.match(s, pos)
        if not m:
            raise SyntaxError(f"cannot tokenize at {s[pos:pos + 30]!r} in {s!r}")
        pos = m.end()
        k = m.lastgroup
        v = m.group(k)
        if k == "ws":
            continue
        if k == "name" or k == "dotop":
            v = v.lower()
        if k == "real":
            v = v.lower()
        toks.append(Tok(k, v))
    return toks


def _real_value(text):
    t = text.split("_")[0].replace("d", "e")
    return float(t)


# --------------------------------------------------------------------------
# expressions (Pratt parser) -> tuples

_BINPREC = {".eqv.": 1, ".neqv.": 1, ".or.": 2, ".and.": 3, "==": 5, "/=": 5, "<": 5, "<=": 5, ">": 5, ">=": 5,
            ".eq.": 5, ".ne.": 5, ".lt.": 5, ".le.": 5, ".gt.": 5, ".ge.": 5, "//": 6, "+": 7, "-": 7, "*": 8,
            "/": 8, "**": 10}
_RELMAP = {".eq.": "==", ".ne.": "/=", ".lt.": "<", ".le.": "<=", ".gt.": ">", ".ge.": ">="}


class Parser:
    def __init__(self, toks):
        self.t, self.i = toks, 0

    def peek(self, k=0):
        j = self.i + k
        return self.t[j] if j < len(self.t) else None

    def at(self, v):
        p = self.peek()
        return p is not None and p.v == v

    def take(self, v=None):
        p = self.peek()
        if p is None or (v is not None and p.v != v):
            raise SyntaxError(f"expected {v!r}, got {p!r} in {self.t}")
        self.i += 1
        return p

    def done(self):
        return self.i >= len(self.t)

    def expr(self, minp=0):
        p = self.peek()
        if p is not None and p.v in ("+", "-") and p.k == "op":
            self.i += 1
            operand = self.expr(8)  # binds tighter than + -, looser than * / **
            left = ("neg", operand) if p.v == "-" else operand
        elif p is not None and p.v == ".not.":
            self.i += 1
            left = ("not", self.expr(4))
        else:
            left = self.primary()
        while True:
            p = self.peek()
            if p is None or p.v not in _BINPREC:
                break
            prec = _BINPREC[p.v]
            if prec < minp:
                break
            self.i += 1
            op = _RELMAP.get(p.v, p.v)
            if op == "**":
                right = self.expr(prec)  # right associative
            else:
                right = self.expr(prec + 1)
            left = ("bin", op, left, right)
        return left

    def primary(self):
        p = self.take()
        if p.k == "int":
            return ("num", int(p.v.split("_")[0]))
        if p.k == "real":
            return ("num", _real_value(p.v))
        if p.k == "str":
            q = p.v[0]
            return ("str", p.v[1:-1].replace(q + q, q))
        if p.v in (".true.", ".false."):
            return ("log", p.v == ".true.")
        if p.v == "(":
            e = self.expr()
            if self.at(","):  # complex literal: not used
                raise SyntaxError("complex constants are not supported")
            self.take(")")
            return ("paren", e)
        if p.v == "(/":
            items = []
            while not self.at("/)"):
                items.append(self.ac_item())
                if self.at(","):
                    self.take(",")
            self.take("/)")
            return ("arr", items)
        if p.k == "name":
            node = ("name", p.v)
            while True:
                if self.at("("):
                    self.take("(")
                    args = self.arglist(")")
                    node = ("ref", node, args)
                elif self.at("%"):
                    self.take("%")
                    node = ("comp", node, self.take().v)
                else:
                    break
            return node
        raise SyntaxError(f"unexpected {p!r}")

    def ac_item(self):
        # implied-do (expr, i = a, b) inside an array constructor
        if self.at("(") and self._is_implied_do():
            self.take("(")
            body = self.expr()
            self.take(",")
            var = self.take().v
            self.take("=")
            lo = self.expr()
            self.take(",")
            hi = self.expr()
            st = None
            if self.at(","):
                self.take(",")
                st = self.expr()
            self.take(")")
            return ("impdo", body, var, lo, hi, st)
        return self.expr()

    def _is_implied_do(self):
        depth, j = 0, self.i
        while j < len(self.t):
            v = self.t[j].v
            if v in ("(", "(/"):
                depth += 1
            elif v in (")", "/)"):
                depth -= 1
                if depth == 0:
                    return False
            elif v == "=" and depth == 1:
                return True
            j += 1
        return False

    def arglist(self, close):
        args = []
        if self.at(close):
            self.take(close)
            return args
        while True:
            args.append(self.arg())
            if self.at(","):
                self.take(",")
                continue
            self.take(close)
            return args

    def arg(self):
        # keyword argument, section triplet or expression
        p0, p1 = self.peek(), self.peek(1)
        if p0 is not None and p0.k == "name" and p1 is not None and p1.v == "=":
            self.i += 2
            return ("kw", p0.v, self.arg())
        lo = hi = st = None
        if self.at("*") and self.peek(1) is not None and self.peek(1).v in (",", ")"):
            self.take("*")
            return ("star",)
        if self.at(":"):
            self.take(":")
            if not (self.at(",") or self.at(")") or self.at(":")):
                hi = self.expr()
            if self.at(":"):
                self.take(":")
                st = self.expr()
            return ("range", None, hi, st)
        e = self.expr()
        if self.at(":"):
            self.take(":")
            if not (self.at(",") or self.at(")") or self.at(":")):
                hi = self.expr()
            if self.at(":"):
                self.take(":")
                st = self.expr()
            return ("range", e, hi, st)
        return e


def parse_expr(text):
    p = Parser(tokenize(text))
    e = p.expr()
    if not p.done():
        raise SyntaxError(f"trailing tokens in {text!r}: {p.t[p.i:]}")
    return e


# --------------------------------------------------------------------------
# program units and statements

class Decl:
    __slots__ = ("name", "type", "dims", "attrs", "init", "charlen")

    def __init__(self, name, type_, dims, attrs, init, charlen=None):
        self.name, self.type, self.dims, self.attrs, self.init, self.charlen = name, type_, dims, attrs, init, charlen

    def is_array(self):
        return self.dims is not None


class Unit:
    def __init__(self, kind, name, parent=None):
        self.kind, self.name, self.parent = kind, name, parent
        self.args, self.result, self.prefix = [], None, set()
        self.decls, self.uses, self.types = {}, [], {}
        self.body, self.contains, self.namelists = [], [], {}
        self.dummy_procs = set()
        self.default_private = False
        self.public, self.private = set(), set()
        self.save_all = False


_TYPEKW = ("integer", "real", "logical", "character", "double", "type")


def _split_top(toks, sep=","):
    parts, cur, depth = [], [], 0
    for t in toks:
        if t.v in ("(", "(/"):
            depth += 1
        elif t.v in (")", "/)"):
            depth -= 1
        if t.v == sep and depth == 0:
            parts.append(cur)
            cur = []
        else:
            cur.append(t)
    parts.append(cur)
    return parts


def _find_top(toks, vals):
    depth = 0
    for i, t in enumerate(toks):
        if t.v in ("(", "(/"):
            depth += 1
        elif t.v in (")", "/)"):
            depth -= 1
        elif depth == 0 and t.v in vals:
            return i
    return -1


def _expr_of(toks):
    p = Parser(toks)
    e = p.expr()
    if not p.done():
        raise SyntaxError(f"trailing tokens {p.t[p.i:]}")
    return e


def _parse_dims(toks):
    """DIMENSION spec (list of (lo, hi) expressions; None for deferred or
    assumed bounds)"""
    dims = []
    for part in _split_top(toks):
        c = _find_top(part, (":",))
        if c < 0:
            dims.append((("num", 1), _expr_of(part)))
        else:
            lo = _expr_of(part[:c]) if c > 0 else None
            hi = _expr_of(part[c + 1:]) if c + 1 < len(part) else None
            dims.append((lo, hi))
    return dims


class SourceParser:
    def __init__(self):
        self.units = []

    def parse(self, stmts):
        self.stmts, self.k = stmts, 0
        while self.k < len(self.stmts):
            f, line, label, text = self.stmts[self.k]
            toks = tokenize(text)
            v = toks[0].v
            if v == "module":
                self.k += 1
                self.units.append(self.unit_body(Unit("module", toks[1].v), ("module",)))
            elif v == "program":
                self.k += 1
                self.units.append(self.unit_body(Unit("program", toks[1].v), ("program",)))
            else:
                u = self.proc_header(toks, None)
                if u is None:
                    raise SyntaxError(f"{f}:{line}: unexpected {text!r}")
                self.k += 1
                self.units.append(self.unit_body(u, (u.kind,)))
        return self.units

    def proc_header(self, toks, parent):
        i, prefix = 0, set()
        while i < len(toks) and toks[i].v in ("recursive", "elemental", "pure", "integer", "real", "logical"):
            prefix.add(toks[i].v)
            i += 1
            if i < len(toks) and toks[i].v == "(":  # REAL(KIND=r8) FUNCTION
                depth = 0
                while True:
                    if toks[i].v == "(":
                        depth += 1
                    elif toks[i].v == ")":
                        depth -= 1
                    i += 1
                    if depth == 0:
                        break
        if i >= len(toks) or toks[i].v not in ("subroutine", "function"):
            return None
        u = Unit(toks[i].v, toks[i + 1].v, parent)
        u.prefix = prefix
        j = i + 2
        if j < len(toks) and toks[j].v == "(":
            j += 1
            while toks[j].v != ")":
                if toks[j].v != ",":
                    u.args.append(toks[j].v)
                j += 1
            j += 1
        if j < len(toks) and toks[j].v == "result":
            u.result = toks[j + 2].v
        if u.kind == "function" and u.result is None:
            u.result = u.name
        return u

    def unit_body(self, u, endkw):
        in_contains = False
        block_stack = []
        while True:
            f, line, label, text = self.stmts[self.k]
            toks = tokenize(text)
            v = toks[0].v
            if v == "end" and (len(toks) == 1 or toks[1].v in ("module", "program", "subroutine", "function")) \
                    and not block_stack:
                self.k += 1
                return u
            if v == "contains":
                in_contains = True
                self.k += 1
                continue
            if in_contains:
                sub = self.proc_header(toks, u)
                if sub is None:
                    raise SyntaxError(f"{f}:{line}: expected a procedure, got {text!r}")
                self.k += 1
                u.contains.append(self.unit_body(sub, (sub.kind,)))
                continue
            if self.spec_stmt(u, toks, f, line):
                self.k += 1
                continue
            u.body.extend(self.exec_block(u, stop=("end_unit",)))
            # exec_block stops at the END of the unit or CONTAINS

    # ---- specification statements ----
    def spec_stmt(self, u, toks, f, line):
        v = toks[0].v
        if v == "use":
            name = toks[1].v
            only = None
            renames = {}
            if len(toks) > 2 and toks[2].v == "," and toks[3].v == "only":
                only = []
                for part in _split_top(toks[5:]):
                    if not part:
                        continue
                    if len(part) == 3 and part[1].v == "=>":
                        renames[part[0].v] = part[2].v
                        only.append(part[0].v)
                    else:
                        only.append(part[0].v)
            u.uses.append((name, only, renames))
            return True
        if v == "implicit":
            return True
        if v == "save" and len(toks) == 1:
            u.save_all = True
            return True
        if v in ("private", "public") and (len(toks) == 1 or toks[1].v in ("::",) or toks[1].k == "name"):
            names = [t.v for t in toks[1:] if t.k == "name"]
            if not names:
                u.default_private = v == "private"
            else:
                (u.private if v == "private" else u.public).update(names)
            return True
        if v == "namelist":
            grp = toks[2].v
            u.namelists[grp] = [t.v for t in toks[4:] if t.k == "name"]
            return True
        if v == "interface":
            self.k += 1
            while True:
                t2 = tokenize(self.stmts[self.k][3])
                if t2[0].v == "end" and len(t2) > 1 and t2[1].v == "interface":
                    return True
                sub = self.proc_header(t2, u)
                if sub is not None:
                    u.dummy_procs.add(sub.name)
                    self.k += 1
                    self.unit_body(sub, (sub.kind,))
                    continue
                self.k += 1
        if v == "type" and (len(toks) == 1 or toks[1].v != "("):
            # derived type definition
            names = [t.v for t in toks[1:] if t.k == "name"]
            tname = names[-1]
            attrs = set(n for n in names[:-1])
            comps = {}
            self.k += 1
            while True:
                t2 = tokenize(self.stmts[self.k][3])
                if t2[0].v == "end" and len(t2) > 1 and t2[1].v == "type":
                    break
                if t2[0].v not in ("private", "sequence"):
                    for d in self.declaration(t2):
                        comps[d.name] = d
                self.k += 1
            u.types[tname] = comps
            if "public" in attrs:
                u.public.add(tname)
            return True
        if v in _TYPEKW and (v != "type" or toks[1].v == "("):
            if _find_top(toks, ("::",)) >= 0 or not any(t.v in ("function",) for t in toks):
                for d in self.declaration(toks):
                    if "public" in d.attrs:
                        u.public.add(d.name)
                    if "private" in d.attrs:
                        u.private.add(d.name)
                    if "external" in d.attrs:
                        u.dummy_procs.add(d.name)
                    u.decls[d.name] = d
                return True
        if v in ("intent", "dimension", "pointer", "allocatable", "optional", "target", "external"):
            raise SyntaxError(f"{f}:{line}: attribute statements are not supported")
        if v == "format":
            return True
        return False

    def declaration(self, toks):
        i = 0
        v = toks[0].v
        charlen = None
        if v == "double":
            type_ = "real"
            i = 2
        elif v == "type":
            type_ = ("type", toks[2].v)
            i = 4
        else:
            type_ = v
            i = 1
            if i < len(toks) and toks[i].v == "(":
                depth, j = 0, i
                while True:
                    if toks[j].v == "(":
                        depth += 1
                    elif toks[j].v == ")":
                        depth -= 1
                    j += 1
                    if depth == 0:
                        break
                inner = toks[i + 1:j - 1]
                if v == "character":
                    for part in _split_top(inner):
                        if part and part[0].v == "len":
                            charlen = _expr_of(part[2:])
                        elif part and part[0].v != "kind":
                            charlen = _expr_of(part)
                i = j
        attrs, dims = set(), None
        dc = _find_top(toks, ("::",))
        if dc >= 0:
            for part in _split_top(toks[i:dc]):
                if not part:
                    continue
                a = part[0].v
                if a == "dimension":
                    dims = _parse_dims(part[2:-1])
                elif a == "intent":
                    attrs.add("intent_" + "".join(t.v for t in part[2:-1]))
                else:
                    attrs.add(a)
            rest = toks[dc + 1:]
        else:
            rest = toks[i:]
            if rest and rest[0].v == ",":
                rest = rest[1:]
        out = []
        for part in _split_top(rest):
            if not part:
                continue
            name = part[0].v
            j = 1
            d_dims = dims
            if j < len(part) and part[j].v == "(":
                depth, k = 0, j
                while True:
                    if part[k].v == "(":
                        depth += 1
                    elif part[k].v == ")":
                        depth -= 1
                    k += 1
                    if depth == 0:
                        break
                d_dims = _parse_dims(part[j + 1:k - 1])
                j = k
            init = None
            if j < len(part) and part[j].v in ("=", "=>"):
                init = _expr_of(part[j + 1:])
            out.append(Decl(name, type_, d_dims, set(attrs), init, charlen))
        return out

    # ---- executable statements ----
    def exec_block(self, u, stop):
        body = []
        while self.k < len(self.stmts):
            f, line, label, text = self.stmts[self.k]
            toks = tokenize(text)
            v = toks[0].v
            key = self._block_key(toks)
            if key in stop or (key == "end_unit" and "end_unit" in stop) or (v == "contains" and "end_unit" in stop):
                return body
            self.k += 1
            st = self.statement(u, toks, f, line)
            if st is not None:
                body.append(st)
        return body

    def _block_key(self, toks):
        v = toks[0].v
        if v == "end":
            if len(toks) == 1 or toks[1].v in ("module", "program", "subroutine", "function"):
                return "end_unit"
            return "end_" + toks[1].v
        if v == "endif":
            return "end_if"
        if v == "enddo":
            return "end_do"
        if v == "else":
            return "else"
        if v == "elseif":
            return "else"
        if v == "case":
            return "case"
        if v == "elsewhere":
            return "elsewhere"
        return None

    def statement(self, u, toks, f, line):
        where = (f, line)
        v = toks[0].v
        # construct name  "name: DO"
        cname = None
        if len(toks) > 2 and toks[0].k == "name" and toks[1].v == ":" and toks[2].v in ("do", "select", "if"):
            cname = v
            toks = toks[2:]
            v = toks[0].v
        if v == "if" and toks[1].v == "(":
            close = self._match(toks, 1)
            cond = _expr_of(toks[2:close])
            if close + 1 < len(toks) and toks[close + 1].v == "then" and close + 2 == len(toks):
                arms = [(cond, self.exec_block(u, ("else", "end_if")))]
                els = None
                while True:
                    t2 = tokenize(self.stmts[self.k][3])
                    key = self._block_key(t2)
                    self.k += 1
                    if key == "end_if":
                        break
                    # else / else if
                    if len(t2) > 1 and t2[1].v == "if" or t2[0].v == "elseif":
                        j = 2 if t2[0].v == "else" else 1
                        c2 = self._match(t2, j)
                        arms.append((_expr_of(t2[j + 1:c2]), self.exec_block(u, ("else", "end_if"))))
                    else:
                        els = self.exec_block(u, ("end_if",))
                return ("if", arms, els, where)
            inner = self.statement(u, toks[close + 1:], f, line)
            return ("if", [(cond, [inner])], None, where)
        if v == "do":
            if len(toks) == 1:
                body = self.exec_block(u, ("end_do",))
                self.k += 1
                return ("loop", body, cname, where)
            if toks[1].v == "while":
                close = self._match(toks, 2)
                cond = _expr_of(toks[3:close])
                body = self.exec_block(u, ("end_do",))
                self.k += 1
                return ("dowhile", cond, body, cname, where)
            var = toks[1].v
            parts = _split_top(toks[3:])
            lo, hi = _expr_of(parts[0]), _expr_of(parts[1])
            st = _expr_of(parts[2]) if len(parts) > 2 else None
            body = self.exec_block(u, ("end_do",))
            self.k += 1
            return ("do", var, lo, hi, st, body, cname, where)
        if v == "select":
            close = self._match(toks, 2)
            sel = _expr_of(toks[3:close])
            cases = []
            while True:
                t2 = tokenize(self.stmts[self.k][3])
                key = self._block_key(t2)
                self.k += 1
                if key == "end_select":
                    break
                if key != "case":
                    raise SyntaxError(f"{f}:{line}: expected CASE")
                if t2[1].v == "default":
                    sel_list = None
                else:
                    c2 = self._match(t2, 1)
                    sel_list = []
                    for part in _split_top(t2[2:c2]):
                        c = _find_top(part, (":",))
                        if c < 0:
                            sel_list.append((_expr_of(part), _expr_of(part)))
                        else:
                            sel_list.append((_expr_of(part[:c]) if c > 0 else None,
                                             _expr_of(part[c + 1:]) if c + 1 < len(part) else None))
                cases.append((sel_list, self.exec_block(u, ("case", "end_select"))))
            return ("select", sel, cases, cname, where)
        if v == "where":
            close = self._match(toks, 1)
            mask = _expr_of(toks[2:close])
            if close + 1 < len(toks):
                return ("where", mask, [self.statement(u, toks[close + 1:], f, line)], [], where)
            yes = self.exec_block(u, ("elsewhere", "end_where"))
            no = []
            t2 = tokenize(self.stmts[self.k][3])
            self.k += 1
            if self._block_key(t2) == "elsewhere":
                no = self.exec_block(u, ("end_where",))
                self.k += 1
            return ("where", mask, yes, no, where)
        if v == "call":
            name = toks[1].v
            args = []
            if len(toks) > 2:
                p = Parser(toks[2:])
                p.take("(")
                args = p.arglist(")")
            return ("call", name, args, where)
        if v == "exit":
            return ("exit", toks[1].v if len(toks) > 1 else None, where)
        if v == "cycle":
            return ("cycle", toks[1].v if len(toks) > 1 else None, where)
        if v == "return":
            return ("return", where)
        if v == "stop":
            return ("stop", where)
        if v == "continue":
            return None
        if v == "format":
            return None
        if v == "print":
            k = _find_top(toks, (",",))
            items = []
            if k > 0:
                ip = Parser(toks[k + 1:])
                while not ip.done():
                    items.append(ip.ac_item())
                    if ip.at(","):
                        ip.take(",")
            return ("print", items, where)
        if v in ("write", "read", "open", "close", "allocate", "deallocate", "nullify", "inquire", "backspace", "rewind"):
            close = self._match(toks, 1)
            p = Parser(toks[1:close + 1])
            p.take("(")
            ctl = p.arglist(")")
            items = []
            rest = toks[close + 1:]
            if rest and rest[0].v == ",":
                rest = rest[1:]
            if rest:
                ip = Parser(rest)
                while not ip.done():
                    items.append(ip.ac_item())
                    if ip.at(","):
                        ip.take(",")
            return (v, ctl, items, where)
        # assignment or pointer assignment
        k = _find_top(toks, ("=", "=>"))
        if k > 0:
            lhs = _expr_of(toks[:k])
            rhs = _expr_of(toks[k + 1:])
            return ("ptr" if toks[k].v == "=>" else "assign", lhs, rhs, where)
        raise SyntaxError(f"{f}:{line}: cannot parse {' '.join(t.v for t in toks)}")

    def _match(self, toks, i):
        depth = 0
        for j in range(i, len(toks)):
            if toks[j].v in ("(", "(/"):
                depth += 1
            elif toks[j].v in (")", "/)"):
                depth -= 1
                if depth == 0:
                    return j
        raise SyntaxError("unbalanced parentheses")


def parse_sources(paths):
    sp = SourceParser()
    for p in paths:
        with open(p) as fh:
            sp.parse(statements(fh.read(), p))
    return sp.units


# --------------------------------------------------------------------------
# runtime values

class FArray:
    """A Fortran array: a numpy array in column-major order with the
    Fortran lower bound of each dimension."""
    __slots__ = ("a", "lb")

    def __init__(self, a, lb):
        self.a, self.lb = a, tuple(lb)


class DTObj:
    """A derived-type object: its type name and components."""
    __slots__ = ("t", "c")

    def __init__(self, t, c):
        self.t, self.c = t, c


MISSING = object()  # an absent OPTIONAL argument


class FortranStop(Exception):
    pass


class _Exit(Exception):
    def __init__(self, name):
        self.name = name


class _Cycle(Exception):
    def __init__(self, name):
        self.name = name


class _Return(Exception):
    pass


class SlotRef:
    __slots__ = ("d", "k")

    def __init__(self, d, k):
        self.d, self.k = d, k

    def get(self):
        return self.d[self.k]

    def set(self, v):
        self.d[self.k] = v


class ElemRef:
    __slots__ = ("a", "i")

    def __init__(self, a, i):
        self.a, self.i = a, i

    def get(self):
        v = self.a[self.i]
        return v.item() if isinstance(v, np.generic) else v

    def set(self, v):
        self.a[self.i] = v


class ValRef:
    __slots__ = ("v",)

    def __init__(self, v):
        self.v = v

    def get(self):
        return self.v

    def set(self, v):
        self.v = v


def _np_dtype(type_):
    if type_ == "real":
        return np.float64
    if type_ == "integer":
        return np.int64
    if type_ == "logical":
        return np.bool_
    return object


def _conv(type_, v):
    """value of v converted for assignment to a scalar of type type_"""
    if type_ == "integer":
        if isinstance(v, (bool, np.bool_)):
            return int(v)
        if isinstance(v, float):
            return int(v)  # truncation, as INT
        return int(v)
    if type_ == "real":
        return float(v)
    if type_ == "logical":
        return bool(v)
    if type_ == "character":
        return str(v)
    return v


def _idiv(a, b):
    q = abs(a) // abs(b)
    return q if (a >= 0) == (b > 0) else -q


def _div(a, b):
    if isinstance(a, (int, np.integer)) and isinstance(b, (int, np.integer)) and not isinstance(a, bool):
        return _idiv(int(a), int(b))
    if isinstance(a, np.ndarray) and a.dtype.kind == "i" and (isinstance(b, (int, np.integer)) or
                                                             (isinstance(b, np.ndarray) and b.dtype.kind == "i")):
        return np.sign(a) * np.sign(b) * (np.abs(a) // np.abs(b))
    if isinstance(b, np.ndarray) and b.dtype.kind == "i" and isinstance(a, (int, np.integer)):
        return np.sign(a) * np.sign(b) * (np.abs(a) // np.abs(b))
    return a / b


def _pow(a, b):
    if isinstance(b, (int, np.integer)) and not isinstance(b, bool):
        if isinstance(a, (int, np.integer)) and not isinstance(a, np.ndarray):
            return int(a) ** int(b) if b >= 0 else _idiv(1, int(a) ** (-int(b)))
        n = int(b)
        if n == 2:
            return a * a
        if n == 3:
            return a * a * a
        return a ** n
    return a ** b


def _nint(x):
    if isinstance(x, np.ndarray):
        return (np.sign(x) * np.floor(np.abs(x) + 0.5)).astype(np.int64)
    t = math.trunc(x)
    r = x - t
    if abs(r) >= 0.5:
        return int(t + (1 if x > 0 else -1))
    return int(t)


def _seq_sum(a, axis=None):
    """SUM in array element order (one addition after another)."""
    a = np.asarray(a)
    if axis is None:
        flat = a.ravel(order="F")
        if flat.size == 0:
            return 0 if a.dtype.kind in "iub" else 0.0
        if a.dtype.kind in "iub":
            return int(flat.astype(np.int64).sum())
        return float(np.add.accumulate(flat)[-1])
    if a.dtype.kind in "iub":
        return a.astype(np.int64).sum(axis=axis)
    if a.shape[axis] == 0:
        return np.zeros(np.delete(a.shape, axis))
    return np.take(np.add.accumulate(a, axis=axis), -1, axis=axis)


def _val(v):
    """a runtime value in expression form: arrays as numpy arrays"""
    if isinstance(v, FArray):
        return v.a
    if isinstance(v, np.generic):
        return v.item()
    return v


# --------------------------------------------------------------------------
# the interpreter

_INTRINSICS = {
    "abs", "sqrt", "exp", "log", "tanh", "sin", "cos", "atan", "max", "min", "mod", "modulo", "int", "nint",
    "real", "dble", "float", "floor", "ceiling", "size", "lbound", "ubound", "shape", "sum", "product", "maxval",
    "minval", "any", "all", "count", "present", "associated", "allocated", "trim", "adjustl", "len", "len_trim",
    "huge", "tiny", "epsilon", "sign", "reshape", "null", "kind", "selected_real_kind", "selected_int_kind",
    "maxloc", "minloc", "merge", "dot_product", "spread", "index", "char", "ichar",
}
_INTRINSIC_SUBS = {"random_number", "cpu_time", "date_and_time", "random_seed"}


class ModRT:
    def __init__(self, interp, unit):
        self.interp, self.u, self.name = interp, unit, unit.name
        self.vars = {}
        self.procs = {}

    def accessible(self, name):
        if name in self.u.private:
            return False
        if name in self.u.public:
            return True
        return not self.u.default_private

    def own(self, name):
        """a symbol this module defines or use-associates (accessibility not
        checked)"""
        u = self.u
        if name in u.decls:
            return ("var", ("mod", self), u.decls[name])
        if name in self.procs:
            return ("proc", self.procs[name])
        if name in u.types:
            return ("type", name, u.types[name])
        if name in u.namelists:
            return ("nml", u.namelists[name], self)
        return self.interp.from_uses(u.uses, name, self)

    def export(self, name):
        if not self.accessible(name):
            return None
        return self.own(name)

    def lookup(self, name):
        s = self.own(name)
        if s is None and (name in _INTRINSICS or name in _INTRINSIC_SUBS):
            return ("intr", name)
        return s

    def find_type(self, tname):
        return self.interp.type_of(self, tname)


class Proc:
    def __init__(self, interp, unit, mod):
        self.interp, self.u, self.mod = interp, unit, mod
        self.name = unit.name
        self.is_func = unit.kind == "function"
        self.elemental = "elemental" in unit.prefix
        self.body = None
        self.saved = {}
        self.saved_init = False
        self.hook = None

    # symbols visible in the procedure body
    def lookup(self, name):
        u = self.u
        if name in u.dummy_procs:
            return ("dproc", name)
        if name in u.decls or name in u.args or name == u.result:
            d = u.decls.get(name)
            if d is None:  # an undeclared dummy is a dummy procedure or implicitly typed; not used here
                return ("dproc", name)
            if name not in u.args and name != u.result and (d.init is not None and "parameter" not in d.attrs
                                                            or "save" in d.attrs or u.save_all):
                return ("var", ("saved", self), d)
            return ("var", ("frame",), d)
        if name in u.namelists:
            return ("nml", u.namelists[name], self)
        if name in u.types:
            return ("type", name, u.types[name])
        s = self.interp.from_uses(u.uses, name, self)
        if s is not None:
            return s
        if self.mod is not None:
            s = self.mod.own(name)
            if s is not None:
                return s
        if name in _INTRINSICS or name in _INTRINSIC_SUBS:
            return ("intr", name)
        return None

    def find_type(self, tname):
        s = self.lookup(tname)
        if s is None or s[0] != "type":
            raise NameError(f"type {tname} not found in {self.name}")
        return s[2]


class Interp:
    def __init__(self, paths, files=None, cwd_files=None):
        self.units = parse_sources(paths)
        self.modules = {}
        self.hooks = {}
        self.printed = []
        self.files = dict(files or {})
        self.units_open = {}
        self.program = None
        self.type_scope, self.dt_plans = {}, {}
        for u in self.units:
            if u.kind == "module":
                m = ModRT(self, u)
                self.modules[u.name] = m
                for c in u.contains:
                    m.procs[c.name] = Proc(self, c, m)
                for comps in u.types.values():
                    self.type_scope[id(comps)] = m
            elif u.kind == "program":
                self.program = Proc(self, u, None)
        for u in self.units:  # module variables, in dependency order of appearance
            if u.kind == "module":
                self._init_module(self.modules[u.name])

    def from_uses(self, uses, name, where):
        for mname, only, renames in uses:
            m = self.modules.get(mname)
            if m is None:
                raise NameError(f"module {mname} not found")
            if only is not None:
                if name not in only:
                    continue
                s = m.export(renames.get(name, name))
                if s is not None:
                    return s
                continue
            s = m.export(name)
            if s is not None:
                return s
        return None

    # ---- storage creation ----
    def default_scalar(self, type_):
        if type_ == "integer":
            return 0
        if type_ == "real":
            return 0.0
        if type_ == "logical":
            return False
        if type_ == "character":
            return ""
        return None

    def new_dt(self, comps, scope, tname):
        plans = self.dt_plans.get(id(comps))
        if plans is None:
            where = self.type_scope[id(comps)]
            C = Compiler(self, where)
            plans = [(n, _storage_plan(C, d)) for n, d in comps.items()]
            self.dt_plans[id(comps)] = plans
        return DTObj(tname, {n: mk({}) for n, mk in plans})

    def new_storage(self, d, scope, f):
        """fresh storage for declaration d (None for pointers and
        allocatables)"""
        if "pointer" in d.attrs or "allocatable" in d.attrs:
            return None
        if d.dims is not None:
            lb, shape = [], []
            for lo, hi in d.dims:
                lv = self.const_eval(lo, scope, f) if lo is not None else 1
                hv = self.const_eval(hi, scope, f)
                lb.append(int(lv))
                shape.append(max(int(hv) - int(lv) + 1, 0))
            if isinstance(d.type, tuple):
                comps = scope.find_type(d.type[1]) if hasattr(scope, "find_type") else self.type_of(scope, d.type[1])
                a = np.empty(shape, dtype=object, order="F")
                for idx in np.ndindex(*shape):
                    a[idx] = self.new_dt(comps, scope, d.type[1])
                return FArray(a, lb)
            if d.init is not None:
                v = self.const_eval(d.init, scope, f)
                a = np.empty(shape, dtype=_np_dtype(d.type), order="F")
                a[...] = v
                return FArray(a, lb)
            return FArray(np.zeros(shape, dtype=_np_dtype(d.type), order="F"), lb)
        if isinstance(d.type, tuple):
            comps = scope.find_type(d.type[1]) if hasattr(scope, "find_type") else self.type_of(scope, d.type[1])
            return self.new_dt(comps, scope, d.type[1])
        if d.init is not None:
            return _conv(d.type, self.const_eval(d.init, scope, f))
        return self.default_scalar(d.type)

    def type_of(self, mod, tname):
        s = mod.own(tname)
        if s is None or s[0] != "type":
            raise NameError(f"type {tname} not found")
        return s[2]

    def const_eval(self, e, scope, f):
        fn = Compiler(self, scope).expr(e)
        return _val(fn(f if f is not None else {}))

    def _init_module(self, m):
        C = Compiler(self, m)
        for n, d in m.u.decls.items():
            m.vars[n] = _storage_plan(C, d)({})

    # ---- running ----
    def proc(self, name):
        for m in self.modules.values():
            if name in m.procs:
                return m.procs[name]
        raise NameError(name)

    def run_program(self):
        try:
            self.call_proc(self.program, [], {})
        except FortranStop:
            pass

    def bind(self, p, actuals, f_caller):
        """the callee frame with p's dummies bound to actuals (for hooks)"""
        if p.body is None:
            p.body = Compiler(self, p).compile_proc()
        return p.bind(actuals, f_caller)[0]

    def call_proc(self, p, actuals, f_caller):
        """actuals: list of (keyword or None, Actual)"""
        if p.hook is not None:
            return p.hook(self, p, actuals, f_caller)
        if p.body is None:
            p.body = Compiler(self, p).compile_proc()
        return p.body(actuals, f_caller)


def _dt_copy(dst, src):
    """intrinsic assignment of derived-type objects: components copied,
    pointer components by association (dst's own storage is kept)"""
    for k, v in src.c.items():
        cur = dst.c.get(k)
        if isinstance(v, DTObj) and isinstance(cur, DTObj) and cur is not v:
            _dt_copy(cur, v)
        elif isinstance(v, FArray) and isinstance(cur, FArray) and cur is not v and cur.a.shape == v.a.shape:
            cur.a[...] = v.a
        else:
            dst.c[k] = v


class Actual:
    __slots__ = ("desig", "ev", "proc", "kw")

    def __init__(self, desig, ev, proc, kw):
        self.desig, self.ev, self.proc, self.kw = desig, ev, proc, kw


class DVar:
    """a named variable"""

    def __init__(self, C, name, sym):
        _, storage, d = sym
        self.name, self.decl, self.type = name, d, d.type
        self.rank = len(d.dims) if d.dims is not None else 0
        self.pointer = "pointer" in d.attrs
        self.is_dt = isinstance(d.type, tuple)
        st = storage[0]
        n = name
        if st == "frame":
            u = C.s.u
            byref = n in u.args and (self.pointer or (d.dims is None and not self.is_dt))
            if byref:
                self.get_slot = lambda f: f[n].get()
                self.set_slot = lambda f, v: f[n].set(v)
                self.ref = lambda f: f[n]
            else:
                self.get_slot = lambda f: f[n]

                def set_slot(f, v):
                    f[n] = v
                self.set_slot = set_slot
                self.ref = lambda f: SlotRef(f, n)
            self.raw = lambda f: f.get(n, MISSING)
        else:
            store = storage[1].saved if st == "saved" else storage[1].vars
            if st == "saved":
                C.saved_decls[n] = d
            self.get_slot = lambda f: store[n]

            def set_slot(f, v):
                store[n] = v
            self.set_slot = set_slot
            self.ref = lambda f: SlotRef(store, n)
            self.raw = lambda f: store[n]
        _finish_desig(self)


def _finish_desig(D):
    gs = D.get_slot
    if D.rank > 0:
        D.val = lambda f: gs(f).a
        D.obj = gs

        def assign(f, v):
            A = gs(f)
            if D.is_dt:
                for idx in np.ndindex(*A.a.shape):
                    _dt_copy(A.a[idx], v if isinstance(v, DTObj) else v[idx])
            else:
                A.a[...] = v
        D.assign = assign
    elif D.is_dt:
        D.val = gs
        D.obj = gs
        D.assign = lambda f, v: _dt_copy(gs(f), v)
    else:
        t = D.type
        D.val = gs
        D.obj = gs
        ss = D.set_slot

        def assign(f, v):
            if isinstance(v, np.ndarray):
                ss(f, v)  # an elemental procedure's body on array arguments
            else:
                ss(f, _conv(t, v))
        D.assign = assign


class DComp:
    """a component of a derived-type object"""

    def __init__(self, C, base, name):
        if not base.is_dt:
            raise TypeError(f"%{name} of a non-derived-type designator")
        comps = C.find_type(base.type[1])
        d = comps[name]
        self.name, self.decl, self.type = name, d, d.type
        self.rank = len(d.dims) if d.dims is not None else 0
        if base.rank > 0:
            raise NotImplementedError("components of arrays of derived type")
        self.pointer = "pointer" in d.attrs
        self.is_dt = isinstance(d.type, tuple)
        bo = base.obj
        self.get_slot = lambda f: bo(f).c[name]

        def set_slot(f, v):
            bo(f).c[name] = v
        self.set_slot = set_slot
        self.ref = lambda f: SlotRef(bo(f).c, name)
        self.raw = lambda f: bo(f).c[name]
        _finish_desig(self)


class DElem:
    """an element or a section of an array designator"""

    def __init__(self, C, base, args):
        self.type, self.is_dt, self.decl = base.type, base.is_dt, base.decl
        self.pointer = False
        bo = base.obj
        ranges = [a for a in args if a[0] == "range"]
        self.rank = len(ranges)
        if not ranges:
            ix = [C.expr(a) for a in args]
            if len(ix) == 1:
                i0 = ix[0]

                def loc(f):
                    A = bo(f)
                    return A.a, (i0(f) - A.lb[0],)
            elif len(ix) == 2:
                i0, i1 = ix

                def loc(f):
                    A = bo(f)
                    lb = A.lb
                    return A.a, (i0(f) - lb[0], i1(f) - lb[1])
            elif len(ix) == 3:
                i0, i1, i2 = ix

                def loc(f):
                    A = bo(f)
                    lb = A.lb
                    return A.a, (i0(f) - lb[0], i1(f) - lb[1], i2(f) - lb[2])
            else:
                def loc(f):
                    A = bo(f)
                    return A.a, tuple(e(f) - l for e, l in zip(ix, A.lb))

            def val(f):
                a, i = loc(f)
                v = a[i]
                return v.item() if isinstance(v, np.generic) else v
            self.val = val
            self.obj = val
            self.get_slot = val

            def set_slot(f, v):
                a, i = loc(f)
                a[i] = v
            self.set_slot = set_slot

            def ref(f):
                a, i = loc(f)
                return ElemRef(a, i)
            self.ref = ref
            self.raw = val
            if self.is_dt:
                self.assign = lambda f, v: _dt_copy(val(f), v)
            else:
                t = self.type

                def assign(f, v):
                    a, i = loc(f)
                    a[i] = _conv(t, v) if not isinstance(v, np.ndarray) else v
                self.assign = assign
            return
        parts = []
        for a in args:
            if a[0] == "range":
                lo = C.expr(a[1]) if a[1] is not None else None
                hi = C.expr(a[2]) if a[2] is not None else None
                st = C.expr(a[3]) if a[3] is not None else None
                parts.append(("r", lo, hi, st))
            else:
                parts.append(("i", C.expr(a)))

        def loc(f):
            A = bo(f)
            sl = []
            for k, p in enumerate(parts):
                l = A.lb[k]
                if p[0] == "i":
                    sl.append(p[1](f) - l)
                    continue
                lo = p[1](f) - l if p[1] is not None else 0
                hi = p[2](f) - l if p[2] is not None else A.a.shape[k] - 1
                st = p[3](f) if p[3] is not None else 1
                if st > 0:
                    sl.append(slice(lo, hi + 1 if hi >= lo else lo, st))
                else:
                    sl.append(slice(lo, hi - 1 if hi - 1 >= 0 else None, st) if hi <= lo else slice(lo, lo, st))
            return A.a, tuple(sl)

        def val(f):
            a, s = loc(f)
            return a[s]
        self.val = val
        rank = self.rank
        self.obj = lambda f: FArray(val(f), (1,) * rank)

        def assign(f, v):
            a, s = loc(f)
            a[s] = v
        self.assign = assign
        self.get_slot = self.obj
        self.raw = self.obj
        self.ref = lambda f: ValRef(val(f))

        def set_slot(f, v):
            raise TypeError("pointer assignment to an array section")
        self.set_slot = set_slot


def _and(a, b):
    def run(f):
        x = a(f)
        if isinstance(x, np.ndarray):
            return np.logical_and(x, b(f))
        return bool(x) and bool(b(f)) if x else False
    return run


def _or(a, b):
    def run(f):
        x = a(f)
        if isinstance(x, np.ndarray):
            return np.logical_or(x, b(f))
        return True if x else bool(b(f))
    return run


def _cmp(op):
    import operator as o
    fn = {"==": o.eq, "/=": o.ne, "<": o.lt, "<=": o.le, ">": o.gt, ">=": o.ge}[op]

    def c(x, y):
        if isinstance(x, str) and isinstance(y, str):
            return fn(x.rstrip(), y.rstrip())
        return fn(x, y)
    return c


class Compiler:
    def __init__(self, interp, scope):
        self.I, self.s = interp, scope
        self.saved_decls = {}

    def find_type(self, tname):
        return self.s.find_type(tname)

    def lookup(self, name):
        s = self.s.lookup(name)
        if s is None:
            raise NameError(f"{name} is not defined in {getattr(self.s, 'name', '?')}")
        return s

    # ---- expressions ----
    def expr(self, e):
        k = e[0]
        if k in ("num", "str", "log"):
            v = e[1]
            return lambda f: v
        if k == "paren":
            return self.expr(e[1])
        if k == "neg":
            x = self.expr(e[1])
            return lambda f: -x(f)
        if k == "not":
            x = self.expr(e[1])

            def nt(f):
                v = x(f)
                return np.logical_not(v) if isinstance(v, np.ndarray) else not v
            return nt
        if k == "bin":
            op, a, b = e[1], self.expr(e[2]), self.expr(e[3])
            if op == "+":
                return lambda f: a(f) + b(f)
            if op == "-":
                return lambda f: a(f) - b(f)
            if op == "*":
                return lambda f: a(f) * b(f)
            if op == "/":
                return lambda f: _div(a(f), b(f))
            if op == "**":
                return lambda f: _pow(a(f), b(f))
            if op == "//":
                return lambda f: a(f) + b(f)
            if op == ".and.":
                return _and(a, b)
            if op == ".or.":
                return _or(a, b)
            if op in (".eqv.", ".neqv."):
                return (lambda f: a(f) == b(f)) if op == ".eqv." else (lambda f: a(f) != b(f))
            c = _cmp(op)
            return lambda f: c(a(f), b(f))
        if k == "arr":
            return self.array_constructor(e[1])
        if k in ("name", "ref", "comp"):
            if k == "name":
                s = self.lookup(e[1])
                if s[0] == "var":
                    d = s[2]
                    if "parameter" in d.attrs and d.dims is None:
                        v = self.I.const_eval(d.init, self.s, None)
                        v = _conv(d.type, v)
                        return lambda f: v
                    return self.desig(e).val
                if s[0] == "proc":  # a function referenced without arguments is not used here
                    raise NameError(f"procedure {e[1]} used as a value")
            if k == "ref" and e[1][0] == "name":
                s = self.lookup(e[1][1])
                if s[0] in ("proc", "dproc"):
                    return self.call_expr(s, e[1][1], e[2])
                if s[0] == "intr":
                    return self.intrinsic(e[1][1], e[2])
                if s[0] == "type":
                    raise NotImplementedError("structure constructors")
            return self.desig(e).val
        if k == "star":
            return lambda f: "*"
        raise NotImplementedError(f"expression {e}")

    def array_constructor(self, items):
        parts = []
        for it in items:
            if it[0] == "impdo":
                body, var, lo, hi, st = it[1], it[2], self.expr(it[3]), self.expr(it[4]), it[5]
                stc = self.expr(st) if st is not None else (lambda f: 1)
                bc = self.expr(body)
                vd = self.desig(("name", var))

                def gen(f, bc=bc, vd=vd, lo=lo, hi=hi, stc=stc):
                    out = []
                    l, h, s = lo(f), hi(f), stc(f)
                    n = max(_idiv(h - l + s, s), 0)
                    v = l
                    for _ in range(n):
                        vd.assign(f, v)
                        out.append(bc(f))
                        v += s
                    return out
                parts.append(("g", gen))
            else:
                parts.append(("e", self.expr(it)))

        def run(f):
            vals = []
            for kind, fn in parts:
                got = fn(f) if kind == "g" else [fn(f)]
                for v in got:
                    v = _val(v)
                    if isinstance(v, np.ndarray):
                        vals.extend(v.ravel(order="F").tolist())
                    else:
                        vals.append(v)
            if all(isinstance(v, (bool, np.bool_)) for v in vals) and vals:
                return np.array(vals, dtype=bool)
            if all(isinstance(v, (int, np.integer)) and not isinstance(v, bool) for v in vals):
                return np.array(vals, dtype=np.int64)
            if all(isinstance(v, str) for v in vals):
                return np.array(vals, dtype=object)
            return np.array(vals, dtype=np.float64)
        return run

    def desig(self, e):
        k = e[0]
        if k == "name":
            s = self.lookup(e[1])
            if s[0] != "var":
                raise NameError(f"{e[1]} is not a variable")
            return DVar(self, e[1], s)
        if k == "comp":
            return DComp(self, self.desig(e[1]), e[2])
        if k == "ref":
            base = self.desig(e[1])
            if base.rank == 0:
                if base.type == "character":
                    raise NotImplementedError("substrings")
                raise TypeError(f"subscripted scalar {e}")
            return DElem(self, base, e[2])
        if k == "paren":
            return self.desig(e[1])
        raise TypeError(f"not a designator: {e}")

    def is_desig(self, e):
        if e[0] == "name":
            s = self.s.lookup(e[1])
            return s is not None and s[0] == "var"
        if e[0] == "comp":
            return True
        if e[0] == "ref" and e[1][0] == "name":
            s = self.s.lookup(e[1][1])
            return s is not None and s[0] == "var"
        if e[0] == "ref":
            return self.is_desig(e[1])
        return False

    def actual(self, a):
        kw = None
        if a[0] == "kw":
            kw, a = a[1], a[2]
        if a[0] == "name":
            s = self.s.lookup(a[1])
            if s is not None and s[0] == "proc":
                p = s[1]
                return Actual(None, None, lambda f: p, kw)
            if s is not None and s[0] == "dproc":
                n = a[1]
                return Actual(None, None, lambda f: f[n], kw)
        if self.is_desig(a):
            d = self.desig(a)
            return Actual(d, d.val, None, kw)
        return Actual(None, self.expr(a), None, kw)

    def call_expr(self, s, name, args):
        acts = [self.actual(a) for a in args]
        I = self.I
        if s[0] == "proc":
            p = s[1]
            return lambda f: I.call_proc(p, acts, f)
        return lambda f: I.call_proc(f[name], acts, f)

    # ---- intrinsics ----
    def intrinsic(self, name, args):
        kws = {}
        pos = []
        for a in args:
            if a[0] == "kw":
                kws[a[1]] = a[2]
            else:
                pos.append(a)
        I = self.I
        if name == "present":
            d = self.desig(pos[0])
            return lambda f: d.raw(f) is not MISSING
        if name == "associated":
            d = self.desig(pos[0])
            if len(pos) > 1:
                t = self.desig(pos[1])
                return lambda f: d.get_slot(f) is not None and d.get_slot(f) is t.obj(f)
            return lambda f: d.get_slot(f) is not None
        if name == "allocated":
            d = self.desig(pos[0])
            return lambda f: d.get_slot(f) is not None
        if name == "null":
            return lambda f: None
        if name in ("size", "lbound", "ubound", "shape"):
            if self.is_desig(pos[0]):
                dd = self.desig(pos[0])
                src = dd.obj
            else:
                ev = self.expr(pos[0])
                src = lambda f: FArray(np.asarray(ev(f)), (1,) * np.ndim(ev(f)))
            dim = self.expr(pos[1]) if len(pos) > 1 else (self.expr(kws["dim"]) if "dim" in kws else None)

            def run(f):
                A = src(f)
                if not isinstance(A, FArray):
                    A = FArray(np.asarray(A), (1,) * np.ndim(A))
                shp = A.a.shape
                if name == "size":
                    return int(np.prod(shp)) if dim is None else int(shp[dim(f) - 1])
                if name == "shape":
                    return np.array(shp, dtype=np.int64)
                if name == "lbound":
                    return int(A.lb[dim(f) - 1]) if dim is not None else np.array(A.lb, dtype=np.int64)
                ub = [l + s - 1 for l, s in zip(A.lb, shp)]
                return int(ub[dim(f) - 1]) if dim is not None else np.array(ub, dtype=np.int64)
            return run
        ev = [self.expr(a) for a in pos]
        kv = {k: self.expr(v) for k, v in kws.items()}
        fn = _INTRINSIC_FUNCS.get(name)
        if fn is None:
            raise NotImplementedError(f"intrinsic {name}")
        if len(ev) == 1 and not kv:
            e0 = ev[0]
            return lambda f: fn(_val(e0(f)))
        if len(ev) == 2 and not kv:
            e0, e1 = ev
            return lambda f: fn(_val(e0(f)), _val(e1(f)))
        return lambda f: fn(*[_val(e(f)) for e in ev], **{k: _val(v(f)) for k, v in kv.items()})


def _maxmin(fn, npfn):
    def run(*xs):
        if any(isinstance(x, np.ndarray) for x in xs):
            r = xs[0]
            for x in xs[1:]:
                r = npfn(r, x)
            return r
        return fn(xs)
    return run


def _reduce_masked(values, mask, dim, op):
    a = np.asarray(values)
    if mask is not None:
        a = a[np.asarray(mask)] if dim is None else np.where(mask, a, op[1])
    if dim is None:
        return op[0](a)
    return op[2](a, dim - 1)


def _sum(a, dim=None, mask=None):
    a = np.asarray(a)
    if mask is not None:
        m = np.broadcast_to(np.asarray(mask), a.shape)
        if dim is None:
            flat = a.ravel(order="F")[m.ravel(order="F")]
            return _seq_sum(flat)
        a = np.where(m, a, 0)
    return _seq_sum(a, None if dim is None else dim - 1)


def _maxval(a, dim=None, mask=None):
    a = np.asarray(a)
    if mask is not None:
        a = a[np.asarray(mask)]
        if a.size == 0:
            return -np.inf if a.dtype.kind == "f" else -(2 ** 31 - 1)
    r = a.max() if dim is None else a.max(axis=dim - 1)
    return r.item() if isinstance(r, np.generic) else r


def _minval(a, dim=None, mask=None):
    a = np.asarray(a)
    if mask is not None:
        a = a[np.asarray(mask)]
        if a.size == 0:
            return np.inf if a.dtype.kind == "f" else 2 ** 31 - 1
    r = a.min() if dim is None else a.min(axis=dim - 1)
    return r.item() if isinstance(r, np.generic) else r


def _elementwise(sfn, afn):
    return lambda x: afn(x) if isinstance(x, np.ndarray) else sfn(x)


def _mod(a, p):
    if isinstance(a, np.ndarray) or isinstance(p, np.ndarray):
        if np.asarray(a).dtype.kind == "i" and np.asarray(p).dtype.kind == "i":
            return np.fmod(a, p)
        return np.fmod(a, p)
    if isinstance(a, int) and isinstance(p, int):
        return a - _idiv(a, p) * p
    return math.fmod(a, p)


def _modulo(a, p):
    if isinstance(a, np.ndarray) or isinstance(p, np.ndarray):
        return np.mod(a, p)
    if isinstance(a, int) and isinstance(p, int):
        return a % p
    return a - math.floor(a / p) * p


def _int(x, kind=None):
    if isinstance(x, np.ndarray):
        return np.trunc(x).astype(np.int64)
    return int(x)


def _real(x, kind=None):
    if isinstance(x, np.ndarray):
        return x.astype(np.float64)
    return float(x)


def _sign(a, b):
    if isinstance(a, np.ndarray) or isinstance(b, np.ndarray):
        return np.where(np.asarray(b) >= 0, np.abs(a), -np.abs(a))
    return abs(a) if b >= 0 else -abs(a)


def _huge(x):
    if isinstance(x, (int, np.integer)) or (isinstance(x, np.ndarray) and x.dtype.kind == "i"):
        return 2 ** 31 - 1
    return 1.7976931348623157e308


def _reshape(src, shape, **kw):
    return np.reshape(np.asarray(src), tuple(int(s) for s in np.asarray(shape)), order="F")


def _selected_int_kind(r):
    return 1 if r <= 2 else (2 if r <= 4 else (4 if r <= 9 else 8))


def _maxloc(a, dim=None, mask=None):
    a = np.asarray(a)
    if a.size == 0:
        return np.zeros(a.ndim, dtype=np.int64)
    flat = np.argmax(a.ravel(order="F"))
    return np.array(np.unravel_index(flat, a.shape, order="F"), dtype=np.int64) + 1


def _minloc(a, dim=None, mask=None):
    a = np.asarray(a)
    if a.size == 0:
        return np.zeros(a.ndim, dtype=np.int64)
    flat = np.argmin(a.ravel(order="F"))
    return np.array(np.unravel_index(flat, a.shape, order="F"), dtype=np.int64) + 1


def _dot(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return _seq_sum(a * b)


_INTRINSIC_FUNCS = {
    "abs": _elementwise(abs, np.abs),
    "sqrt": _elementwise(math.sqrt, np.sqrt),
    "exp": _elementwise(math.exp, np.exp),
    "log": _elementwise(math.log, np.log),
    "tanh": _elementwise(math.tanh, np.tanh),
    "sin": _elementwise(math.sin, np.sin),
    "cos": _elementwise(math.cos, np.cos),
    "atan": _elementwise(math.atan, np.arctan),
    "max": _maxmin(max, np.maximum),
    "min": _maxmin(min, np.minimum),
    "mod": _mod,
    "modulo": _modulo,
    "int": _int,
    "nint": _nint,
    "real": _real,
    "dble": _real,
    "float": _real,
    "floor": _elementwise(lambda x: int(math.floor(x)), lambda x: np.floor(x).astype(np.int64)),
    "ceiling": _elementwise(lambda x: int(math.ceil(x)), lambda x: np.ceil(x).astype(np.int64)),
    "sum": _sum,
    "product": lambda a, dim=None, mask=None: (int(np.prod(np.asarray(a))) if np.asarray(a).dtype.kind == "i"
                                               else float(np.prod(np.asarray(a)))),
    "maxval": _maxval,
    "minval": _minval,
    "any": lambda a, dim=None: bool(np.any(a)) if dim is None else np.any(a, axis=dim - 1),
    "all": lambda a, dim=None: bool(np.all(a)) if dim is None else np.all(a, axis=dim - 1),
    "count": lambda a, dim=None: int(np.count_nonzero(a)) if dim is None else np.count_nonzero(a, axis=dim - 1),
    "trim": lambda s: s.rstrip(),
    "adjustl": lambda s: s.lstrip() + " " * (len(s) - len(s.lstrip())),
    "len": lambda s: len(s),
    "len_trim": lambda s: len(s.rstrip()),
    "huge": _huge,
    "tiny": lambda x: 2.2250738585072014e-308,
    "epsilon": lambda x: 2.220446049250313e-16,
    "sign": _sign,
    "reshape": _reshape,
    "kind": lambda x: 8,
    "selected_real_kind": lambda p=15, r=307: 8,
    "selected_int_kind": _selected_int_kind,
    "maxloc": _maxloc,
    "minloc": _minloc,
    "merge": lambda t, fv, mask: np.where(mask, t, fv) if isinstance(mask, np.ndarray) else (t if mask else fv),
    "dot_product": _dot,
    "spread": lambda src, dim, ncopies: np.repeat(np.expand_dims(np.asarray(src), dim - 1), ncopies, axis=dim - 1),
    "index": lambda s, sub: s.find(sub) + 1,
    "char": lambda i: chr(i),
    "ichar": lambda c: ord(c[0]),
}


def _ctl(ctl):
    """(positional list, keyword dict) of an I/O or ALLOCATE control list"""
    pos, kw = [], {}
    for a in ctl:
        if a[0] == "kw":
            kw[a[1]] = a[2]
        else:
            pos.append(a)
    return pos, kw


def _format_items(fmt, vals):
    """the subset of edit descriptors internal writes use (A, Aw, Iw, Iw.m,
    Fw.d, X and quoted strings)"""
    out = []
    items = list(vals)
    body = fmt.strip()[1:-1]
    for part in re.findall(r"'[^']*'|\d*[aifx][\d.]*|\d+x", body, re.I):
        p = part.lower()
        if p.startswith("'"):
            out.append(part[1:-1])
            continue
        m = re.match(r"(\d*)([aifx])(\d*)(?:\.(\d+))?", p)
        rep = int(m.group(1)) if m.group(1) else 1
        kind, w, d = m.group(2), m.group(3), m.group(4)
        for _ in range(rep):
            if kind == "x":
                out.append(" ")
                continue
            v = items.pop(0)
            if kind == "a":
                s = str(v)
                out.append(s if not w else s[:int(w)].ljust(int(w)))
            elif kind == "i":
                s = str(int(v))
                if d:
                    s = ("-" if int(v) < 0 else "") + str(abs(int(v))).zfill(int(d))
                out.append(s.rjust(int(w)) if w else s)
            elif kind == "f":
                out.append(("%" + w + "." + d + "f") % v)
    return "".join(out)


class _StmtCompiler:
    """statement compilation (mixed into Compiler)"""

    def block(self, stmts):
        fs = [self.stmt(s) for s in stmts if s is not None]
        fs = [x for x in fs if x is not None]
        if not fs:
            return lambda f: None
        if len(fs) == 1:
            return fs[0]
        if len(fs) == 2:
            a, b = fs

            def run2(f):
                a(f)
                b(f)
            return run2

        def run(f):
            for s in fs:
                s(f)
        return run

    def stmt(self, s):
        try:
            return self._stmt(s)
        except Exception as e:
            where = s[-1]
            raise type(e)(f"{where[0]}:{where[1]}: {e}") from e

    def _stmt(self, s):
        k = s[0]
        I = self.I
        if k == "assign":
            d = self.desig(s[1])
            r = self.expr(s[2])
            a = d.assign
            return lambda f: a(f, r(f))
        if k == "ptr":
            d = self.desig(s[1])
            rhs = s[2]
            ss = d.set_slot
            if rhs[0] == "ref" and rhs[1] == ("name", "null"):
                return lambda f: ss(f, None)
            t = self.desig(rhs)
            if isinstance(t, DElem) and t.rank > 0:
                to = t.obj
            else:
                to = t.get_slot
            return lambda f: ss(f, to(f))
        if k == "if":
            arms = [(self.expr(c), self.block(b)) for c, b in s[1]]
            els = self.block(s[2]) if s[2] is not None else None
            if len(arms) == 1:
                c0, b0 = arms[0]
                if els is None:
                    def if1(f):
                        if c0(f):
                            b0(f)
                    return if1

                def if2(f):
                    if c0(f):
                        b0(f)
                    else:
                        els(f)
                return if2

            def ifn(f):
                for c, b in arms:
                    if c(f):
                        b(f)
                        return
                if els is not None:
                    els(f)
            return ifn
        if k == "do":
            _, var, lo, hi, st, body, name, _w = s
            vd = self.desig(("name", var))
            va = vd.assign
            lo, hi = self.expr(lo), self.expr(hi)
            stc = self.expr(st) if st is not None else None
            b = self.block(body)

            def do(f):
                l, h = lo(f), hi(f)
                step = stc(f) if stc is not None else 1
                n = max(_idiv(h - l + step, step), 0)
                v = l
                for _ in range(n):
                    va(f, v)
                    try:
                        b(f)
                    except _Cycle as c:
                        if c.name is not None and c.name != name:
                            raise
                    except _Exit as e:
                        if e.name is not None and e.name != name:
                            raise
                        return
                    v += step
                va(f, v)
            return do
        if k in ("dowhile", "loop"):
            if k == "dowhile":
                cond, body, name = self.expr(s[1]), self.block(s[2]), s[3]
            else:
                cond, body, name = (lambda f: True), self.block(s[1]), s[2]

            def loop(f):
                while cond(f):
                    try:
                        body(f)
                    except _Cycle as c:
                        if c.name is not None and c.name != name:
                            raise
                    except _Exit as e:
                        if e.name is not None and e.name != name:
                            raise
                        return
            return loop
        if k == "select":
            sel = self.expr(s[1])
            cases = []
            for sl, body in s[2]:
                b = self.block(body)
                if sl is None:
                    cases.append((None, b))
                else:
                    cases.append(([(self.expr(lo) if lo is not None else None,
                                    self.expr(hi) if hi is not None else None) for lo, hi in sl], b))

            def select(f):
                v = sel(f)
                if isinstance(v, str):
                    v = v.rstrip()
                default = None
                for sl, b in cases:
                    if sl is None:
                        default = b
                        continue
                    for lo, hi in sl:
                        lv = lo(f) if lo is not None else None
                        hv = hi(f) if hi is not None else None
                        if isinstance(lv, str):
                            lv = lv.rstrip()
                        if isinstance(hv, str):
                            hv = hv.rstrip()
                        if (lv is None or lv <= v) and (hv is None or v <= hv):
                            b(f)
                            return
                if default is not None:
                    default(f)
            return select
        if k == "where":
            mask = self.expr(s[1])
            yes = [(self.desig(a[1]), self.expr(a[2])) for a in s[2]]
            no = [(self.desig(a[1]), self.expr(a[2])) for a in s[3]]

            def where(f):
                m = np.asarray(mask(f), dtype=bool)
                for d, r in yes:
                    view = d.val(f)
                    v = r(f)
                    view[m] = v[m] if isinstance(v, np.ndarray) else v
                for d, r in no:
                    view = d.val(f)
                    v = r(f)
                    view[~m] = v[~m] if isinstance(v, np.ndarray) else v
            return where
        if k == "call":
            name, args = s[1], s[2]
            sym = self.lookup(name)
            if sym[0] == "intr":
                return self.intrinsic_sub(name, args)
            acts = [self.actual(a) for a in args]
            if sym[0] == "proc":
                p = sym[1]
                return lambda f: I.call_proc(p, acts, f)
            if sym[0] == "dproc":
                return lambda f: I.call_proc(f[name], acts, f)
            raise NameError(f"CALL of {name}")
        if k == "exit":
            nm = s[1]

            def ex(f):
                raise _Exit(nm)
            return ex
        if k == "cycle":
            nm = s[1]

            def cy(f):
                raise _Cycle(nm)
            return cy
        if k == "return":
            def ret(f):
                raise _Return()
            return ret
        if k == "stop":
            def stop(f):
                raise FortranStop()
            return stop
        if k == "print":
            items = [self.io_item(it) for it in s[1]]

            def pr(f):
                vals = []
                for it in items:
                    vals.extend(it(f))
                I.printed.append(vals)
            return pr
        if k in ("allocate", "deallocate", "nullify"):
            return self.alloc_stmt(k, s[1])
        if k in ("open", "close", "read", "write", "inquire", "backspace", "rewind"):
            return self.io_stmt(k, s[1], s[2])
        raise NotImplementedError(f"statement {k}")

    def io_item(self, it):
        if it[0] == "impdo":
            body, var, lo, hi, st = it[1], it[2], self.expr(it[3]), self.expr(it[4]), it[5]
            stc = self.expr(st) if st is not None else (lambda f: 1)
            bc = self.io_item(body)
            vd = self.desig(("name", var))

            def gen(f):
                out = []
                l, h, sp = lo(f), hi(f), stc(f)
                v = l
                for _ in range(max(_idiv(h - l + sp, sp), 0)):
                    vd.assign(f, v)
                    out.extend(bc(f))
                    v += sp
                return out
            return gen
        e = self.expr(it)

        def one(f):
            v = _val(e(f))
            if isinstance(v, np.ndarray):
                return v.ravel(order="F").tolist()
            return [v]
        return one

    def intrinsic_sub(self, name, args):
        ds = [self.desig(a) if self.is_desig(a) else None for a in args]
        if name == "random_number":
            d = ds[0]

            def rn(f):
                o = d.val(f)
                if isinstance(o, np.ndarray):
                    o[...] = 0.5
                else:
                    d.assign(f, 0.5)
            return rn
        if name == "cpu_time":
            d = ds[0]
            return lambda f: d.assign(f, 0.0)
        if name == "date_and_time":
            def dt(f):
                vals = ["20000101", "000000.000", "+0000"]
                for dd, v in zip(ds, vals):
                    if dd is not None:
                        dd.assign(f, v)
                if len(ds) > 3 and ds[3] is not None:
                    ds[3].assign(f, 0)
            return dt
        if name == "random_seed":
            return lambda f: None
        raise NotImplementedError(name)

    def alloc_stmt(self, k, ctl):
        pos, kw = _ctl(ctl)
        stat = self.desig(kw["stat"]) if "stat" in kw else None
        ops = []
        I = self.I
        for a in pos:
            if k == "allocate" and a[0] == "ref" and self._alloc_target_is_array(a[1]):
                d = self.desig(a[1])
                bnds = []
                for r in a[2]:
                    if r[0] == "range":
                        bnds.append((self.expr(r[1]) if r[1] is not None else (lambda f: 1), self.expr(r[2])))
                    else:
                        bnds.append(((lambda f: 1), self.expr(r)))
                npd = _np_dtype(d.type)
                is_dt = d.is_dt
                comps = self.find_type(d.type[1]) if is_dt else None

                def al(f, d=d, bnds=bnds, npd=npd, is_dt=is_dt, comps=comps):
                    lb = [int(lo(f)) for lo, _ in bnds]
                    shape = [max(int(hi(f)) - l + 1, 0) for (lo, hi), l in zip(bnds, lb)]
                    if is_dt:
                        arr = np.empty(shape, dtype=object, order="F")
                        for idx in np.ndindex(*shape):
                            arr[idx] = I.new_dt(comps, None, d.type[1])
                    else:
                        arr = np.zeros(shape, dtype=npd, order="F")
                    d.set_slot(f, FArray(arr, lb))
                ops.append(al)
            else:
                d = self.desig(a)
                if k == "allocate":
                    comps = self.find_type(d.type[1])
                    tn = d.type[1]
                    ops.append(lambda f, d=d, comps=comps, tn=tn: d.set_slot(f, I.new_dt(comps, None, tn)))
                else:
                    ops.append(lambda f, d=d: d.set_slot(f, None))

        def run(f):
            for o in ops:
                o(f)
            if stat is not None:
                stat.assign(f, 0)
        return run

    def _alloc_target_is_array(self, e):
        try:
            d = self.desig(e)
        except Exception:
            return False
        return d.rank > 0 or (d.decl.dims is not None)

    def io_stmt(self, k, ctl, items):
        I = self.I
        pos, kw = _ctl(ctl)
        iostat = self.desig(kw["iostat"]) if "iostat" in kw else None
        unit = kw.get("unit", pos[0] if pos else None)
        if k == "open":
            ue = self.expr(unit)
            fe = self.expr(kw["file"])
            status = kw.get("status")
            se = self.expr(status) if status is not None else (lambda f: "UNKNOWN")

            def op(f):
                name = str(fe(f)).strip()
                I.units_open[ue(f)] = name
                ok = not (se(f).upper() == "OLD" and name not in I.files)
                if iostat is not None:
                    iostat.assign(f, 0 if ok else 1)
            return op
        if k in ("close", "backspace", "rewind"):
            return lambda f: None
        if k == "inquire":
            fe = self.expr(kw["file"])
            ex = self.desig(kw["exist"])
            return lambda f: ex.assign(f, str(fe(f)).strip() in I.files)
        if k == "read":
            if "nml" in kw:
                grp = kw["nml"][1]
                sym = self.lookup(grp)
                names, where = sym[1], sym[2]
                wc = Compiler(I, where) if where is not self.s else self
                targets = {n: wc for n in names}
                ue = self.expr(unit)

                def rd(f):
                    text = I.files[I.units_open[ue(f)]]
                    _read_namelist(text, grp, targets, f if wc is self else {})
                    if iostat is not None:
                        iostat.assign(f, 0)
                return rd
            raise NotImplementedError("formatted READ")
        if k == "write":
            if "nml" in kw:
                return lambda f: None
            fmt = kw.get("fmt", pos[1] if len(pos) > 1 else None)
            its = [self.io_item(it) for it in items]
            if unit is not None and unit[0] != "star" and self.is_desig(unit):
                d = self.desig(unit)
                if d.type == "character":
                    fe = self.expr(fmt)

                    def iw(f):
                        vals = []
                        for it in its:
                            vals.extend(it(f))
                        d.assign(f, _format_items(fe(f), vals))
                    return iw
            return lambda f: None
        raise NotImplementedError(k)


def _read_namelist(text, grp, targets, f):
    m = re.search(r"&" + grp + r"\b(.*?)/\s*$", text, re.I | re.S)
    if m is None:
        m = re.search(r"&" + grp + r"\b(.*?)/", text, re.I | re.S)
    body = m.group(1)
    for lhs, rhs in re.findall(r"([a-z]\w*(?:\([^)]*\))?)\s*=\s*([^=]*?)(?=(?:[,\s]+[a-z]\w*(?:\([^)]*\))?\s*=)|\s*$)",
                               body, re.I | re.S):
        name = lhs.split("(")[0].lower()
        C = targets[name]
        vals = [v for v in re.split(r"[,\s]+", rhs.strip()) if v]
        pv = []
        for v in vals:
            lv = v.lower()
            if lv in (".true.", "t", ".t."):
                pv.append(True)
            elif lv in (".false.", "f", ".f."):
                pv.append(False)
            elif re.match(r"^[-+]?\d+$", lv):
                pv.append(int(lv))
            elif lv.startswith("'") or lv.startswith('"'):
                pv.append(v[1:-1])
            else:
                pv.append(float(lv.replace("d", "e")))
        e = parse_expr(lhs.lower())
        d = C.desig(e)
        if d.rank == 0:
            d.assign(f, pv[0])
        else:
            view = d.val(f)
            view.ravel(order="F")[:len(pv)] = pv
            if not view.flags.f_contiguous:
                raise NotImplementedError("namelist fill of a non-contiguous array")


for _k, _v in list(vars(_StmtCompiler).items()):
    if not _k.startswith("__"):
        setattr(Compiler, _k, _v)


def _storage_plan(C, d):
    """a function of the frame that creates storage for local declaration d"""
    I = C.I
    if "pointer" in d.attrs or "allocatable" in d.attrs:
        return lambda f: None
    is_dt = isinstance(d.type, tuple)
    comps = C.find_type(d.type[1]) if is_dt else None
    if d.dims is not None:
        bnds = [(C.expr(lo) if lo is not None else (lambda f: 1), C.expr(hi)) for lo, hi in d.dims]
        init = C.expr(d.init) if d.init is not None else None
        npd = _np_dtype(d.type)

        def make(f):
            lb = [int(lo(f)) for lo, _ in bnds]
            shape = [max(int(hi(f)) - l + 1, 0) for (lo, hi), l in zip(bnds, lb)]
            if is_dt:
                a = np.empty(shape, dtype=object, order="F")
                for idx in np.ndindex(*shape):
                    a[idx] = I.new_dt(comps, None, d.type[1])
            else:
                a = np.zeros(shape, dtype=npd, order="F")
                if init is not None:
                    a[...] = _val(init(f))
            return FArray(a, lb)
        return make
    if is_dt:
        tn = d.type[1]
        return lambda f: I.new_dt(comps, None, tn)
    if d.init is not None:
        ini = C.expr(d.init)
        t = d.type
        return lambda f: _conv(t, _val(ini(f)))
    dv = I.default_scalar(d.type)
    return lambda f: dv


def _binder(C, name, d, is_proc):
    if is_proc:
        def bp(act, f, fc, post):
            f[name] = act.proc(fc) if act.proc is not None else act.ev(fc)
        return bp
    if d is None:
        raise NameError(f"dummy {name} is not declared")
    if "pointer" in d.attrs:
        def bptr(act, f, fc, post):
            f[name] = act.desig.ref(fc) if act.desig is not None else ValRef(act.ev(fc))
        return bptr
    if d.dims is not None:
        if all(hi is None for _, hi in d.dims):
            lbs = [C.expr(lo) if lo is not None else (lambda f: 1) for lo, _ in d.dims]

            def bassumed(act, f, fc, post):
                o = act.desig.obj(fc) if act.desig is not None else act.ev(fc)
                arr = o.a if isinstance(o, FArray) else np.asarray(o)
                f[name] = FArray(arr, [int(l(f)) for l in lbs])
            return bassumed
        bnds = [(C.expr(lo) if lo is not None else (lambda f: 1), C.expr(hi)) for lo, hi in d.dims]
        intent_in = "intent_in" in d.attrs

        def bexplicit(act, f, fc, post):
            o = act.desig.obj(fc) if act.desig is not None else act.ev(fc)
            arr = o.a if isinstance(o, FArray) else np.asarray(o)
            lb = [int(lo(f)) for lo, _ in bnds]
            shape = [max(int(hi(f)) - l + 1, 0) for (lo, hi), l in zip(bnds, lb)]
            n = int(np.prod(shape))
            if arr.flags.f_contiguous and arr.size == n:
                view = arr.reshape(shape, order="F")
            elif arr.flags.f_contiguous and arr.size > n:
                view = arr.ravel(order="F")[:n].reshape(shape, order="F")
            else:
                view = np.array(arr.ravel(order="F")[:n]).reshape(shape, order="F")
                if not intent_in:
                    post.append((arr, view))
            f[name] = FArray(view, lb)
        return bexplicit
    if isinstance(d.type, tuple):
        def bdt(act, f, fc, post):
            f[name] = act.desig.obj(fc) if act.desig is not None else act.ev(fc)
        return bdt

    def bscalar(act, f, fc, post):
        if act.desig is not None and act.desig.rank == 0:
            f[name] = act.desig.ref(fc)
        else:
            f[name] = ValRef(act.ev(fc))
    return bscalar


def _compile_proc(C):
    p = C.s
    u = p.u
    I = C.I
    if p.is_func and u.result not in u.decls:
        t = next((x for x in ("integer", "real", "logical") if x in u.prefix), None)
        u.decls[u.result] = Decl(u.result, t, None, set(), None)
    args = list(u.args)
    binders = [_binder(C, a, u.decls.get(a), a in u.dummy_procs) for a in args]
    array_dummy = [a not in u.dummy_procs and u.decls.get(a) is not None and u.decls[a].dims is not None
                   and "pointer" not in u.decls[a].attrs for a in args]
    order = [i for i in range(len(args)) if not array_dummy[i]] + [i for i in range(len(args)) if array_dummy[i]]
    plans, saved_plans = [], []
    for n, d in u.decls.items():
        if n in args:
            continue
        if "parameter" in d.attrs and d.dims is None:
            continue
        sym = p.lookup(n)
        if sym[0] == "var" and sym[1][0] == "saved":
            saved_plans.append((n, _storage_plan(C, d)))
        else:
            plans.append((n, _storage_plan(C, d)))
    body = C.block(u.body)
    res = u.result
    res_saved = res is not None and p.lookup(res)[1][0] == "saved" if res is not None else False

    def bind(actuals, fc):
        f = {}
        bound = [MISSING] * len(args)
        k = 0
        for a in actuals:
            if a.kw is None:
                bound[k] = a
                k += 1
            else:
                bound[args.index(a.kw)] = a
        post = []
        for i in order:
            a = bound[i]
            if a is MISSING:
                f[args[i]] = MISSING
            else:
                binders[i](a, f, fc, post)
        return f, post

    def run(actuals, fc):
        f, post = bind(actuals, fc)
        if not p.saved_init:
            for n, mk in saved_plans:
                p.saved[n] = mk(f)
            p.saved_init = True
        for n, mk in plans:
            f[n] = mk(f)
        try:
            body(f)
        except _Return:
            pass
        for arr, view in post:
            arr[...] = view.ravel(order="F").reshape(arr.shape, order="F")
        if res is not None:
            r = p.saved[res] if res_saved else f[res]
            if isinstance(r, FArray):
                return r.a
            if isinstance(r, (SlotRef, ElemRef, ValRef)):
                return r.get()
            return r
        return None
    p.bind = bind
    return run


Compiler.compile_proc = lambda self: _compile_proc(self)


class PyProc:
    """a Python function standing in where the reference passes a procedure
    (ApplyOnLevel's callback): called with the actual arguments' objects"""

    def __init__(self, fn):
        self.hook = lambda I, p, actuals, fc: fn(*[a.desig.obj(fc) if a.desig is not None else a.ev(fc)
                                                   for a in actuals])
        self.name = getattr(fn, "__name__", "pyproc")
