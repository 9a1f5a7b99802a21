"""The C drivers' ASCII catalogue reader (fcfc_gb300/csrc/driver/catalog.c):
chunked, multi-threaded parsing with a strtod fast path must give exactly
the rows and values of the Python reader (which follows FCFC's reading and
is pinned to a golden case FCFC read through expressions and a selection),
whatever the thread count and chunk size; malformed lines fail with the
same line number.  CPU only: the reader is compiled into a small harness
here."""
import os
import random
import shutil
import subprocess

import numpy as np
import pytest

from fcfc_gb300 import ascii

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DRV = os.path.join(ROOT, "fcfc_gb300", "csrc", "driver")

HARNESS = r"""
#include <stdio.h>
#include <stdlib.h>
#include "catalog.h"
/* argv: file fmtr x y z w sel skip comment out */
int main(int argc, char **argv) {
  if (argc != 11) return 2;
  const char *pos[3] = {argv[3], argv[4], argv[5]};
  const char *wx = *argv[6] ? argv[6] : NULL, *sel = *argv[7] ? argv[7] : NULL;
  double *xyz[3], *w = NULL;
  size_t n = 0;
  char err[512];
  if (cat_read_ascii(argv[1], argv[2], pos, wx, sel, atol(argv[8]),
                     argv[9][0], xyz, &w, &n, err, sizeof err)) {
    printf("%s\n", err);
    return 1;
  }
  FILE *fp = fopen(argv[10], "wb");
  fwrite(&n, sizeof n, 1, fp);
  for (int k = 0; k < 3; k++) fwrite(xyz[k], sizeof(double), n, fp);
  if (w) fwrite(w, sizeof(double), n, fp);
  fclose(fp);
  return 0;
}
"""


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    if not shutil.which("gcc"):
        pytest.skip("gcc not available")
    d = tmp_path_factory.mktemp("reader")
    src = d / "h.c"
    src.write_text(HARNESS)
    exe = str(d / "h")
    subprocess.run(["gcc", "-O2", "-std=c11", "-I", DRV, str(src),
                    os.path.join(DRV, "catalog.c"), os.path.join(DRV, "expr.c"),
                    "-lm", "-lpthread", "-o", exe], check=True)
    return exe


def _c_read(exe, path, fmt, pos, w="", sel="", skip=0, comment="#",
            threads=1, chunk=None):
    out = path + ".out"
    env = dict(os.environ, OMP_NUM_THREADS=str(threads))
    if chunk:
        env["FCFCG_ASCII_CHUNK"] = str(chunk)
    r = subprocess.run([exe, path, fmt, *pos, w, sel, str(skip), comment, out],
                       capture_output=True, text=True, env=env)
    if r.returncode:
        return None, r.stdout.strip()
    raw = open(out, "rb").read()
    n = int(np.frombuffer(raw[:8], np.uint64)[0])
    a = np.frombuffer(raw[8:], np.float64)
    xyz = a[:3 * n].reshape(3, n).T
    return (xyz, a[3 * n:] if w else None), ""


def _mixed_file(path, n, seed, bad_line=None):
    rng = np.random.default_rng(seed)
    rnd = random.Random(seed)
    lines = ["# header", "", "   "]
    for i in range(n):
        x, y, z = rng.random(3) * 1000
        seps = [rnd.choice([" ", "  ", "\t", " \t "]) for _ in range(5)]
        vals = ["%.17g" % x, "%.9g" % y, "%.6e" % z,
                rnd.choice(["gal", "qso", "star"]),
                str(int(rng.integers(-5, 5))), "%.17g" % rng.lognormal()]
        ln = vals[0]
        for s, v in zip(seps, vals[1:]):
            ln += s + v
        if i % 97 == 7:
            ln = "  # " + ln
        if i % 77 == 3:
            ln += "\r"
        lines.append(ln)
    if bad_line is not None:
        lines[bad_line] = "1.0 2.0 oops gal 3 1.0"
    # no newline after the last line
    open(path, "w").write("\n".join(lines))


CASES = [
    ("%lf %f %lf %s %d %lf", ("$1", "$2", "$3*2"), "$6",
     '$4 == "gal" && $5 >= 0', 3),
    ("%lf %f %lf %*s %d %lf", ("$1", "$2", "$3"), "$5", "", 0),
    ("%lf %lf %lf %s %i %lf", ("$1 + $5", "$2", "sqrt($3)"), "", "$6 > 1", 1),
    ("%lf %lf %*lf %s %ld %lf", ("$1", "$2", "$5"), "$4", "", 0),
]


@pytest.mark.parametrize("case", range(len(CASES)))
def test_c_reader_matches_python_reader(harness, tmp_path, case):
    fmt, pos, w, sel, skip = CASES[case]
    path = str(tmp_path / "cat.txt")
    _mixed_file(path, 20000, seed=case)
    xyz, wt = ascii.read_ascii(path, fmt, list(pos), weight=w or None,
                               selection=sel or None, skip=skip, comment="#")
    ref = None
    for threads, chunk in ((1, None), (4, 4096), (3, 10007)):
        got, err = _c_read(harness, path, fmt, pos, w, sel, skip, "#",
                           threads, chunk)
        assert got is not None, err
        np.testing.assert_array_equal(got[0], xyz)
        if w:
            np.testing.assert_array_equal(got[1], wt)
        if ref is None:
            ref = got
        else:
            assert got[0].tobytes() == ref[0].tobytes()


def test_c_reader_reports_the_failing_line(harness, tmp_path):
    path = str(tmp_path / "bad.txt")
    _mixed_file(path, 5000, seed=9, bad_line=4003)
    for threads, chunk in ((1, None), (4, 4096)):
        got, err = _c_read(harness, path, "%lf %lf %lf %s %d %lf",
                           ("$1", "$2", "$3"), threads=threads, chunk=chunk)
        assert got is None
        assert "line 4004 " in err, err


def test_c_reader_unusable_columns(harness, tmp_path):
    """`%Lf` (long double) is read past and is unusable, as in FCFC."""
    path = str(tmp_path / "c.txt")
    _mixed_file(path, 100, seed=2)
    got, err = _c_read(harness, path, "%lf %lf %*lf %s %ld %Lf",
                       ("$1", "$2", "$5"))
    assert got is None and "cannot evaluate" in err
    got, err = _c_read(harness, path, "%lf %lf %*lf %s %ld %Lf",
                       ("$1", "$2", "$4"))
    assert got is not None, err
