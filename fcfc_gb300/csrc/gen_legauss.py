#!/usr/bin/env python3
"""Write legauss_tab.h: Gauss-Legendre nodes and weights, orders 4..32.

The nodes are the roots of the Legendre polynomial P_n, found by Newton's
method in 60-digit arithmetic (mpmath) from the Tricomi initial guess
cos(pi (k - 1/4) / (n + 1/2)); the weights are 2 / ((1 - x^2) P_n'(x)^2).
Both are rounded to the nearest double.

Layout (what FCFC's redshift integration walks, src/fcfc/2pt/cnvt_coord.c:
219-239): for each order n, the n/2 positive nodes in descending order, then,
for odd n, the node x = 0.  The weight array runs in the same order.  Order n
starts at n*n/4 - 4 (integer division), so the table holds 268 entries.

Run: python fcfc_gb300/csrc/gen_legauss.py [--check FCFC_SRC/src/math/legauss.c]
(needs mpmath).  --check also compares every entry with FCFC's own table and
fails unless all 2 x 268 doubles are identical.
"""
import os
import sys

import mpmath as mp
from mpmath.libmp import to_float

MIN_ORDER, MAX_ORDER = 4, 32


def start(n):
    return (n * n) // 4 - (MIN_ORDER * MIN_ORDER) // 4


def legendre(n, x):
    """P_n(x) and P_n'(x) by the three-term recurrence."""
    p0, p1 = mp.mpf(1), x
    for k in range(2, n + 1):
        p0, p1 = p1, ((2 * k - 1) * x * p1 - (k - 1) * p0) / k
    dp = n * (x * p1 - p0) / (x * x - 1)
    return p1, dp


def nodes(n):
    out = []
    for k in range(1, n // 2 + 1):
        x = mp.cos(mp.pi * (k - mp.mpf(1) / 4) / (n + mp.mpf(1) / 2))
        for _ in range(100):
            p, dp = legendre(n, x)
            dx = p / dp
            x -= dx
            if abs(dx) < mp.mpf(10) ** (-mp.mp.dps + 5):
                break
        p, dp = legendre(n, x)
        out.append((x, 2 / ((1 - x * x) * dp * dp)))
    if n & 1:
        _, dp = legendre(n, mp.mpf(0))
        out.append((mp.mpf(0), 2 / (dp * dp)))
    return out


def dbl(v):
    return to_float(mp.mpf(v)._mpf_, rnd="n")


def table():
    xs, ws = [], []
    for n in range(MIN_ORDER, MAX_ORDER + 1):
        assert len(xs) == start(n)
        for x, w in nodes(n):
            xs.append(dbl(x))
            ws.append(dbl(w))
    assert len(xs) == start(MAX_ORDER + 1)
    return xs, ws


def check(path, xs, ws):
    src = open(path).read()

    def arr(name):
        body = src[src.index(name):]
        body = body[body.index("{") + 1:body.index("};")]
        toks = [t.strip() for t in body.replace("\n", " ").split(",") if t.strip()]
        return [float.fromhex(t) if "x" in t else float(t) for t in toks]

    rx, rw = arr("legauss_x["), arr("legauss_w[")
    bad = [i for i in range(len(xs)) if xs[i] != rx[i] or ws[i] != rw[i]]
    if len(rx) != len(xs) or len(rw) != len(ws) or bad:
        raise SystemExit("table differs from %s at %s" % (path, bad[:10]))
    print("all %d nodes and weights identical to %s" % (len(xs), path))


def main():
    mp.mp.dps = 60
    xs, ws = table()
    if "--check" in sys.argv:
        check(sys.argv[sys.argv.index("--check") + 1], xs, ws)
    here = os.path.dirname(os.path.abspath(__file__))
    with open(os.path.join(here, "legauss_tab.h"), "w") as f:
        f.write("/* Gauss-Legendre nodes and weights, orders %d..%d, rounded to the\n"
                " * nearest double; generated by gen_legauss.py (do not edit). */\n"
                % (MIN_ORDER, MAX_ORDER))
        f.write("#define FCFCG_GL_MIN_ORDER %d\n#define FCFCG_GL_MAX_ORDER %d\n"
                % (MIN_ORDER, MAX_ORDER))
        f.write("#define FCFCG_GL_START(n) ((((n) * (n)) >> 2) - %d)\n"
                % ((MIN_ORDER * MIN_ORDER) // 4))
        f.write("#define FCFCG_GL_LEN %d\n" % len(xs))
        for name, arr in (("FCFCG_GL_X", xs), ("FCFCG_GL_W", ws)):
            f.write("#define %s_INIT { \\\n" % name)
            for i in range(0, len(arr), 3):
                f.write("  " + ", ".join(v.hex() for v in arr[i:i + 3]) +
                        (", \\\n" if i + 3 < len(arr) else " \\\n"))
            f.write("}\n")


if __name__ == "__main__":
    main()
