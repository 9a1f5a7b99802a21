"""End to end on the GPU: the FCFC run flow (config keys -> catalogues ->
counts -> pair-count files -> xi -> multipoles / w_p) against the files the
upstream FCFC wrote.  Unweighted runs must reproduce them byte for byte;
weighted runs to 1e-10 relative (FP64 sums in a different order)."""
import os

import numpy as np
import pytest

from fcfc_gb300 import pcfile
from golden_cases import Case, case_names

pytestmark = pytest.mark.gpu

CASES = case_names()


def _write_conf(case, tmp):
    m = case.meta
    lines = []
    files = []
    fmts = []
    pos = []
    wts = []
    if m.get("catalog_text"):
        # the catalogue file and FCFC's own reader keys, verbatim
        lines.append("CATALOG = [%s]" % ", ".join(
            os.path.join(case.dir, m["catalog_text"][l]) for l in m["labels"]))
        lines.append("CATALOG_LABEL = [%s]" % ", ".join(m["labels"]))
        lines += ["%s = %s" % kv for kv in m["keys"].items()]
    for lab in ([] if m.get("catalog_text") else m["labels"]):
        a = case.cats[lab]
        fn = os.path.join(tmp, lab + ".txt")
        np.savetxt(fn, a, fmt="%.17g")
        files.append(fn)
        fmts.append('"%s"' % " ".join(["%lf"] * a.shape[1]))
        pos += ["$1", "$2", "$3"]
        wts.append("$4" if a.shape[1] > 3 else "''")
    if not m.get("catalog_text"):
        lines.append("CATALOG = [%s]" % ", ".join(files))
        lines.append("CATALOG_LABEL = [%s]" % ", ".join(m["labels"]))
        lines.append("ASCII_FORMATTER = [%s]" % ", ".join(fmts))
        lines.append("POSITION = [%s]" % ", ".join(pos))
        if any(case.cats[l].shape[1] > 3 for l in m["labels"]):
            lines.append("WEIGHT = [%s]" % ", ".join(wts))
    if case.box:
        lines.append("BOX_SIZE = [%s]" % ", ".join(repr(v) for v in m["box"]))
    if case.convert:
        lines.append("COORD_CONVERT = [%s]" % ", ".join("T" for _ in m["labels"]))
        if m.get("zfile"):
            lines.append("Z_CMVDST_FILE = %s" % os.path.join(case.dir, m["zfile"]))
        else:
            lines.append("OMEGA_M = %r" % m.get("omega_m", 0.31))
            for key, name in (("omega_l", "OMEGA_LAMBDA"), ("dew", "DE_EOS_W"),
                              ("cmvdst_err", "CMVDST_ERR")):
                if key in m:
                    lines.append("%s = %r" % (name, m[key]))
    lines.append("BINNING_SCHEME = %d" % m["bintype"])
    lines.append("PAIR_COUNT = [%s]" % ", ".join(m["pairs"]))
    lines.append("PAIR_COUNT_FILE = [%s]" % ", ".join(
        os.path.join(tmp, p + ".bin") for p in m["pairs"]))
    lines.append("CF_ESTIMATOR = [%s]" % ", ".join('"%s"' % e for e in m["cf"]))
    lines.append("CF_OUTPUT_FILE = [%s]" % os.path.join(tmp, "xi.txt"))
    if m.get("poles"):
        lines.append("MULTIPOLE = [%s]" % ", ".join(map(str, m["poles"])))
        lines.append("MULTIPOLE_FILE = [%s]" % os.path.join(tmp, "mp.txt"))
    if m.get("wp"):
        lines.append("PROJECTED_CF = T")
        lines.append("PROJECTED_FILE = [%s]" % os.path.join(tmp, "wp.txt"))
    if m.get("sfile"):
        lines.append("SEP_BIN_FILE = %s" % os.path.join(case.dir, m["sfile"]))
    else:
        s = m["sbin"]
        lines += ["SEP_BIN_MIN = %r" % s["smin"], "SEP_BIN_MAX = %r" % s["smax"],
                  "SEP_BIN_SIZE = %r" % s["ds"]]
    if m["bintype"] == 1:
        lines.append("MU_BIN_NUM = %d" % m.get("nmu", 10))
    if m["bintype"] == 2:
        p = m["pbin"]
        lines += ["PI_BIN_MIN = %r" % p["pmin"], "PI_BIN_MAX = %r" % p["pmax"],
                  "PI_BIN_SIZE = %r" % p["dpi"]]
    lines += ["OUTPUT_FORMAT = 0", "OVERWRITE = 2"]
    fn = os.path.join(tmp, "run.conf")
    open(fn, "w").write("\n".join(lines) + "\n")
    return fn


def _numbers(path):
    rows = [l.split() for l in open(path) if not l.startswith("#")]
    return np.array(rows, dtype=float)


@pytest.mark.parametrize("name", CASES)
def test_run_matches_upstream_outputs(name, tmp_path):
    from fcfc_gb300 import runner
    case = Case(name)
    conf = runner.parse_conf(open(_write_conf(case, str(tmp_path))).read())
    runner.run(conf, "box" if case.box else "survey", with_mu_one=case.mu_one)
    any_wt = False
    for pair in case.meta["pairs"]:
        want = open(os.path.join(case.dir, pair + ".bin"), "rb").read()
        got = open(str(tmp_path / (pair + ".bin")), "rb").read()
        ref = case.pcfile(pair)
        mine = pcfile.read_binary(str(tmp_path / (pair + ".bin")))
        if ref.weighted:
            any_wt = True
            np.testing.assert_allclose(mine.cnt, ref.cnt, rtol=1e-10)
            np.testing.assert_allclose(mine.norm, ref.norm, rtol=1e-12)
        else:
            assert got == want, pair
    for fn in ("xi.txt", "mp.txt", "wp.txt"):
        ref = os.path.join(case.dir, fn)
        if not os.path.exists(ref):
            continue
        got = str(tmp_path / fn)
        if any_wt:
            np.testing.assert_allclose(_numbers(got), _numbers(ref), rtol=1e-8,
                                       atol=1e-12)
        else:
            assert open(got).read() == open(ref).read(), fn


def test_resume_reads_existing_counts(tmp_path):
    """OVERWRITE = 1 keeps an existing pair-count file and reads it back
    (FCFC's check_output), so a second run recounts nothing."""
    from fcfc_gb300 import runner
    case = Case("box_smu_auto")
    conf_path = _write_conf(case, str(tmp_path))
    conf = runner.parse_conf(open(conf_path).read())
    runner.run(conf, "box")
    first = open(str(tmp_path / "DD.bin"), "rb").read()
    conf["OVERWRITE"] = "1"
    os.remove(str(tmp_path / "xi.txt"))
    out = runner.run(conf, "box")
    assert open(str(tmp_path / "DD.bin"), "rb").read() == first
    assert os.path.exists(str(tmp_path / "xi.txt"))
    np.testing.assert_array_equal(out["counts"]["DD"], case.pcfile("DD").cnt)


@pytest.mark.parametrize("name", CASES)
def test_run_graph_and_per_count_paths_write_the_same_files(name, tmp_path):
    """Every count through one CUDA graph (default) or one count_pairs per
    pair: byte-identical files, weighted ones included."""
    from fcfc_gb300 import runner
    case = Case(name)
    out = {}
    for graph in (True, False):
        d = tmp_path / ("graph" if graph else "plain")
        d.mkdir()
        conf = runner.parse_conf(open(_write_conf(case, str(d))).read())
        runner.run(conf, "box" if case.box else "survey",
                   with_mu_one=case.mu_one, graph=graph)
        out[graph] = {f: open(os.path.join(d, f), "rb").read()
                      for f in sorted(os.listdir(d))
                      if not f.endswith(".conf")}   # holds the directory
    assert out[True].keys() == out[False].keys()
    for f in out[True]:
        assert out[True][f] == out[False][f], f
