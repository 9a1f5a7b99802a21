"""ASCII catalogue reading as FCFC does it: ASCII_FORMATTER, column
expressions for POSITION / WEIGHT, and SELECTION criteria.

FCFC reads each line with the scanf conversions of ASCII_FORMATTER
(src/io/ascii_fmtr.c:114-300, src/io/read_ascii.c:181-257); `$n` / `${n}` is
the n-th conversion that is not suppressed with `*`.  POSITION and WEIGHT
entries are expressions evaluated in double precision, SELECTION a boolean
expression (src/io/read_ascii.c:540-760), both in the syntax of FCFC's
expression library (src/lib/libast.h): numbers, "strings", columns,
parentheses, abs sqrt ln log isfinite, unary - ! ~, ** * / % + - << >>
< <= > >= == != & ^ | && ||, with libast's precedences (unary operators
above `**`, all binary operators left-associative).

Numbers are evaluated in FP64 as FCFC's double build does; a `%f` (float)
column is rounded to float first, like the float variable scanf fills.
Integer-only operators (~ << >> & ^ |) need integer columns or literals.
"""
from __future__ import annotations

import math
import re

import numpy as np

from .capi import ERR_CFG, ERR_FILE, FCFCGError

# --------------------------------------------------------------------------
# the formatter

_CONV = re.compile(r"%(\*?)(\d*)(hh|h|ll|l|j|z|t|L)?([diouxXaAeEfFgGsc\[])")


def parse_formatter(fmt: str):
    """Conversions of a scanf formatter: list of (suppressed, kind) with kind
    'int', 'float', 'double', 'str' or 'other'; literal text between
    conversions is kept as regex separators."""
    convs, seps = [], []
    pos = 0
    sep = ""
    while pos < len(fmt):
        if fmt[pos] == "%":
            if fmt.startswith("%%", pos):
                sep += "%"
                pos += 2
                continue
            m = _CONV.match(fmt, pos)
            if not m:
                raise FCFCGError(ERR_CFG, "invalid ASCII_FORMATTER: %r" % fmt)
            skip, _, lmod, conv = m.groups()
            if conv in "dioux" or conv == "X":
                kind = "int"
            elif conv in "aAeEfFgG":
                kind = "double" if lmod in ("l", "L") else "float"
            elif conv in "sc[":
                kind = "str"
                if conv == "[":
                    end = fmt.find("]", m.end() + (1 if fmt[m.end():m.end() + 1] in "^]" else 0))
                    if end < 0:
                        raise FCFCGError(ERR_CFG, "invalid ASCII_FORMATTER: %r" % fmt)
                    pos = end + 1
                    seps.append(sep)
                    convs.append((bool(skip), kind))
                    sep = ""
                    continue
            else:
                kind = "other"
            seps.append(sep)
            convs.append((bool(skip), kind))
            sep = ""
            pos = m.end()
        else:
            sep += fmt[pos]
            pos += 1
    return convs, seps


def _is_plain(seps) -> bool:
    return all(s.strip() == "" for s in seps)


# --------------------------------------------------------------------------
# expressions (libast syntax)

_TOKEN = re.compile(r"""
    \s*(?:
      (?P<num>(?:\d+\.?\d*|\.\d+)(?:[eE][+-]?\d+)?)
    | (?P<col>\$\{?\d+\}?)
    | (?P<str>"[^"]*"|'[^']*')
    | (?P<func>abs|sqrt|ln|log|isfinite)\b
    | (?P<op>\*\*|<<|>>|<=|>=|==|!=|&&|\|\||[-+*/%<>!~&^|()])
    )""", re.X)

_BIN = {"**": 11, "*": 10, "/": 10, "%": 10, "+": 9, "-": 9, "<<": 8,
        ">>": 8, "<": 7, "<=": 7, ">": 7, ">=": 7, "==": 6, "!=": 6,
        "&": 5, "^": 4, "|": 3, "&&": 2, "||": 1}


def _tokens(expr: str):
    out, pos = [], 0
    expr = expr.strip()
    while pos < len(expr):
        m = _TOKEN.match(expr, pos)
        if not m or m.end() == pos:
            raise FCFCGError(ERR_CFG, "invalid expression: %r" % expr)
        kind = m.lastgroup
        out.append((kind, m.group(kind)))
        pos = m.end()
        while pos < len(expr) and expr[pos].isspace():
            pos += 1
    return out


class _Parser:
    def __init__(self, expr):
        self.expr = expr
        self.t = _tokens(expr)
        self.i = 0
        self.cols = set()

    def peek(self):
        return self.t[self.i] if self.i < len(self.t) else (None, None)

    def take(self):
        tok = self.peek()
        self.i += 1
        return tok

    def parse(self):
        node = self.binary(1)
        if self.i != len(self.t):
            raise FCFCGError(ERR_CFG, "invalid expression: %r" % self.expr)
        return node

    def binary(self, minp):
        left = self.unary()
        while True:
            kind, v = self.peek()
            if kind != "op" or v not in _BIN or _BIN[v] < minp:
                return left
            self.take()
            right = self.binary(_BIN[v] + 1)      # left-associative
            left = ("bin", v, left, right)

    def unary(self):
        kind, v = self.peek()
        if kind == "op" and v in ("-", "!", "~", "+"):
            self.take()
            return ("un", v, self.unary())
        return self.atom()

    def atom(self):
        kind, v = self.take()
        if kind == "num":
            return ("num", float(v))
        if kind == "str":
            return ("str", v[1:-1])
        if kind == "col":
            n = int(v.strip("${}"))
            if n < 1:
                raise FCFCGError(ERR_CFG, "invalid column: %r" % v)
            self.cols.add(n)
            return ("col", n)
        if kind == "func":
            k2, v2 = self.take()
            if v2 != "(":
                raise FCFCGError(ERR_CFG, "invalid expression: %r" % self.expr)
            arg = self.binary(1)
            if self.take()[1] != ")":
                raise FCFCGError(ERR_CFG, "invalid expression: %r" % self.expr)
            return ("fn", v, arg)
        if v == "(":
            node = self.binary(1)
            if self.take()[1] != ")":
                raise FCFCGError(ERR_CFG, "unbalanced parentheses: %r" % self.expr)
            return node
        raise FCFCGError(ERR_CFG, "invalid expression: %r" % self.expr)


def _libm(f, a):
    """The C library's function element by element (numpy's vectorised
    versions may differ from it in the last bit)."""
    a = np.asarray(a, np.float64)
    return np.fromiter((f(float(v)) for v in a.ravel()), np.float64,
                       a.size).reshape(a.shape)


def _ln(v):
    return math.log(v) if v > 0 else (-math.inf if v == 0 else math.nan)


def _log10(v):
    return math.log10(v) if v > 0 else (-math.inf if v == 0 else math.nan)


def _eval(node, cols, n):
    kind = node[0]
    if kind == "num":
        return np.full(n, node[1])
    if kind == "str":
        return np.full(n, node[1], dtype=object)
    if kind == "col":
        return cols[node[1]]
    if kind == "fn":
        a = _eval(node[2], cols, n)
        f = node[1]
        if f == "abs":
            return np.abs(a)
        if f == "sqrt":
            return np.sqrt(np.asarray(a, np.float64))
        if f == "ln":
            return _libm(_ln, a)
        if f == "log":
            return _libm(_log10, a)
        return np.isfinite(np.asarray(a, np.float64))
    if kind == "un":
        a = _eval(node[2], cols, n)
        if node[1] == "-":
            return -a
        if node[1] == "+":
            return a
        if node[1] == "!":
            return ~np.asarray(a, bool)
        return ~_as_int(a)
    op, a, b = node[1], _eval(node[2], cols, n), _eval(node[3], cols, n)
    if op in ("==", "!="):
        eq = (a == b) if (a.dtype == object or b.dtype == object) else (
            np.asarray(a, np.float64) == np.asarray(b, np.float64))
        return eq if op == "==" else ~eq
    if op in ("&&", "||"):
        a, b = np.asarray(a, bool), np.asarray(b, bool)
        return (a & b) if op == "&&" else (a | b)
    if op in ("<<", ">>", "&", "^", "|"):
        ia, ib = _as_int(a), _as_int(b)
        return {"<<": ia << ib, ">>": ia >> ib, "&": ia & ib, "^": ia ^ ib,
                "|": ia | ib}[op]
    fa, fb = np.asarray(a, np.float64), np.asarray(b, np.float64)
    with np.errstate(all="ignore"):
        if op == "+":
            return fa + fb
        if op == "-":
            return fa - fb
        if op == "*":
            return fa * fb
        if op == "/":
            return fa / fb
        if op == "%":
            return np.fmod(fa, fb)
        if op == "**":
            return _libm_pow(fa, fb)
        return {"<": fa < fb, "<=": fa <= fb, ">": fa > fb,
                ">=": fa >= fb}[op]


def _pow(x, y):
    """C's pow: NaN for a negative base with a non-integer exponent,
    +-inf for a zero base with a negative exponent and on overflow."""
    try:
        return math.pow(x, y)
    except ValueError:
        if x == 0 and y < 0:
            odd = float(y).is_integer() and int(y) % 2 == 1
            return math.copysign(math.inf, x) if odd else math.inf
        return math.nan
    except OverflowError:
        neg = x < 0 and float(y).is_integer() and int(y) % 2 == 1
        return -math.inf if neg else math.inf


def _libm_pow(a, b):
    return np.fromiter((_pow(float(x), float(y)) for x, y in
                        zip(a.ravel(), b.ravel())), np.float64,
                       a.size).reshape(a.shape)


def _as_int(a):
    a = np.asarray(a)
    if a.dtype.kind in "iub":
        return a.astype(np.int64)
    if a.dtype.kind == "f" and np.all(a == np.floor(a)):
        return a.astype(np.int64)
    raise FCFCGError(ERR_CFG, "integer operator on a non-integer value")


def compile_expr(expr: str):
    """Parsed expression and the columns it uses."""
    p = _Parser(str(expr))
    node = p.parse()
    return node, p.cols


# --------------------------------------------------------------------------
# reading

def _split_lines(path, skip, comment):
    with open(path) as f:
        lines = f.read().splitlines()
    out = []
    for k, line in enumerate(lines):
        if k < skip:
            continue
        s = line.lstrip()
        if not s or (comment and s.startswith(comment)):
            continue
        out.append(line)
    return out


def _columns_plain(lines, convs, need):
    """Whitespace-separated conversions."""
    nconv = len(convs)
    kept = [i for i, (sk, _) in enumerate(convs) if not sk]
    toks = [ln.split() for ln in lines]
    for t in toks:
        if len(t) < nconv:
            raise FCFCGError(ERR_FILE, "failed to read line: %s" % " ".join(t))
    cols = {}
    for n in need:
        ci = kept[n - 1]
        kind = convs[ci][1]
        raw = [t[ci] for t in toks]
        cols[n] = _convert(raw, kind)
    return cols


def _columns_regex(lines, convs, seps, need):
    pat = ""
    for (sk, kind), sep in zip(convs, seps):
        pat += "".join(r"\s*" if ch.isspace() else re.escape(ch) for ch in sep)
        body = r"\s*(\S+?)" if kind != "str" else r"\s*(\S+)"
        pat += body
    rx = re.compile(pat)
    kept = [i for i, (sk, _) in enumerate(convs) if not sk]
    rows = []
    for ln in lines:
        m = rx.match(ln)
        if not m:
            raise FCFCGError(ERR_FILE, "failed to read line: %s" % ln)
        rows.append(m.groups())
    cols = {}
    for n in need:
        ci = kept[n - 1]
        cols[n] = _convert([r[ci] for r in rows], convs[ci][1])
    return cols


def _convert(raw, kind):
    if kind == "str":
        return np.array(raw, dtype=object)
    if kind == "int":
        return np.array([int(v, 0) if v[:2].lower() == "0x" else int(v) for v in raw],
                        np.int64)
    a = np.array([float(v) for v in raw], np.float64)
    if kind == "float":
        a = a.astype(np.float32).astype(np.float64)
    return a


def read_ascii(path, formatter, position, weight=None, selection=None,
               skip=0, comment=None):
    """(xyz N x 3, w or None) of an ASCII catalogue, FCFC's way: the first
    `skip` lines are dropped, then empty lines and lines starting (after
    blanks) with the ASCII_COMMENT character (none by default)."""
    convs, seps = parse_formatter(formatter)
    nread = sum(1 for sk, _ in convs if not sk)
    exprs = [compile_expr(p) for p in position]
    wexpr = compile_expr(weight) if weight else None
    sexpr = compile_expr(selection) if selection else None
    need = set()
    for _, c in exprs + ([wexpr] if wexpr else []) + ([sexpr] if sexpr else []):
        need |= c
    if need and max(need) > nread:
        raise FCFCGError(ERR_CFG, "not enough columns for the expressions")
    lines = _split_lines(path, int(skip or 0), comment)
    cols = (_columns_plain(lines, convs, need) if _is_plain(seps)
            else _columns_regex(lines, convs, seps, need))
    n = len(lines)
    sel = None
    if sexpr:
        sel = np.asarray(_eval(sexpr[0], cols, n), bool)
    xyz = np.stack([np.asarray(_eval(e[0], cols, n), np.float64) for e in exprs],
                   axis=1)
    w = np.asarray(_eval(wexpr[0], cols, n), np.float64) if wexpr else None
    if sel is not None:
        xyz = xyz[sel]
        w = w[sel] if w is not None else None
    return np.ascontiguousarray(xyz), (None if w is None else np.ascontiguousarray(w))
