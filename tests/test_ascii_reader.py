"""Catalogue reading as FCFC does it (ASCII_FORMATTER, POSITION / WEIGHT
expressions, SELECTION; src/io/read_ascii.c, src/lib/libast): expression
semantics, formatter handling, and a golden case whose catalogue FCFC read
through expressions and a selection."""
import os

import numpy as np
import pytest

from fcfc_gb300 import ascii
from fcfc_gb300.capi import FCFCGError
from golden_cases import Case
from oracle import fcfc_oracle as fo


def _val(expr, cols=None, n=1):
    node, _ = ascii.compile_expr(expr)
    cols = cols or {}
    return ascii._eval(node, {k: np.asarray(v) for k, v in cols.items()}, n)


def test_precedence_and_associativity():
    # unary minus binds above **, binary operators are left-associative
    assert _val("-2**2")[0] == 4.0
    assert _val("2**3**2")[0] == 64.0
    assert _val("1 + 2 * 3")[0] == 7.0
    assert _val("(1 + 2) * 3")[0] == 9.0
    assert _val("10 - 4 - 3")[0] == 3.0
    assert _val("7 % 4 * 2")[0] == 6.0
    assert bool(_val("1 < 2 && 3 >= 3 || 0")[0])
    assert not bool(_val("!(2 > 1)")[0])
    assert _val("6 & 3 | 8")[0] == 10
    assert _val("1 << 4 >> 2")[0] == 4


def test_functions_and_columns():
    c = {1: [4.0, 9.0], 2: [-1.5, 2.0], 3: ["A", "B"]}
    np.testing.assert_array_equal(_val("sqrt($1) + abs(${2})", c, 2), [3.5, 5.0])
    np.testing.assert_allclose(_val("ln($1)", c, 2), np.log([4.0, 9.0]), rtol=0)
    np.testing.assert_allclose(_val("log($1)", c, 2), np.log10([4.0, 9.0]), rtol=0)
    np.testing.assert_array_equal(_val('$3 == "A"', c, 2), [True, False])
    np.testing.assert_array_equal(_val("isfinite($2 / 0)", c, 2), [False, False])


def test_invalid_expressions():
    for bad in ("1 +", "(1", "$0", "foo(1)", "1 @ 2"):
        with pytest.raises(FCFCGError):
            ascii.compile_expr(bad)


def test_formatter_columns(tmp_path):
    fn = str(tmp_path / "c.txt")
    with open(fn, "w") as f:
        f.write("skip me\n")
        f.write("# a comment\n\n")
        f.write("1,0.1,x,3\n")
        f.write("  2,0.2,y,4\n")
    xyz, w = ascii.read_ascii(fn, "%d,%f,%*s,%lf", ["$1", "$2", "$3"], "$1*$3",
                              None, skip=1, comment="#")
    assert xyz.shape == (2, 3)
    # %f fills a float: the value is rounded to single precision
    assert xyz[0, 1] == float(np.float32(0.1))
    np.testing.assert_array_equal(w, [3.0, 8.0])
    # whitespace-separated with a skipped string column
    fn2 = str(tmp_path / "d.txt")
    with open(fn2, "w") as f:
        f.write("1.5 a 2.5 3.5\n4.5 b 5.5 6.5\n")
    xyz, w = ascii.read_ascii(fn2, "%lf %*s %lf %lf", ["$1", "$2", "$3"],
                              None, "$1 > 2")
    np.testing.assert_array_equal(xyz, [[4.5, 5.5, 6.5]])
    assert w is None


def test_golden_catalogue_read_through_expressions():
    """FCFC read this catalogue with POSITION = [$1*2, ${2} + 1.5, $3],
    WEIGHT = $4 * $5 and a SELECTION on an integer and a string column; the
    same reading gives its weight sum and its weighted pair counts."""
    case = Case("box_smu_expr")
    a = case.cats["D"]
    ref = case.pcfile("DD")
    assert a[:, 3].sum() == pytest.approx(float(ref.tracers[0]), rel=1e-13)
    ob = fo.Bins(False, 1, ns=10, smin=0, ds=4, nmu=10, box=300.0)
    got = ob.count(a[:, :3], wa=a[:, 3], mode=3) * 2
    np.testing.assert_allclose(got, ref.cnt, rtol=1e-12, atol=0)
