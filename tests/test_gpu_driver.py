"""The C command line drivers FCFC_2PT_BOX_GPU / FCFC_2PT_GPU (FCFC's main
flow in C over the library) reproduce the upstream files of every golden
case: unweighted pair counts, xi, multipoles and w_p byte for byte, weighted
ones to 1e-10."""
import os
import subprocess

import numpy as np
import pytest

from fcfc_gb300 import pcfile
from golden_cases import Case, case_names
from test_gpu_runner import _numbers, _write_conf

pytestmark = pytest.mark.gpu

BIN = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                   "fcfc_gb300", "bin")


@pytest.mark.parametrize("name", case_names())
def test_driver_matches_upstream_outputs(name, tmp_path):
    case = Case(name)
    conf = _write_conf(case, str(tmp_path))
    exe = os.path.join(BIN, "FCFC_2PT_BOX_GPU" if case.box else "FCFC_2PT_GPU")
    cmd = [exe, "-c", conf] + (["--with-mu-one"] if case.mu_one else [])
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    any_wt = False
    for pair in case.meta["pairs"]:
        ref = case.pcfile(pair)
        got = str(tmp_path / (pair + ".bin"))
        if ref.weighted:
            any_wt = True
            mine = pcfile.read_binary(got)
            np.testing.assert_allclose(mine.cnt, ref.cnt, rtol=1e-10)
        else:
            assert open(got, "rb").read() == \
                open(os.path.join(case.dir, pair + ".bin"), "rb").read(), pair
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


@pytest.mark.parametrize("name", case_names())
def test_driver_graph_and_per_count_paths_write_the_same_files(name, tmp_path):
    """All counts of a run in one CUDA graph (the default) or one fcfcg_count
    at a time (--no-graph): byte-identical files, weighted ones included
    (the weighted sums are exact fixed-point sums either way)."""
    case = Case(name)
    exe = os.path.join(BIN, "FCFC_2PT_BOX_GPU" if case.box else "FCFC_2PT_GPU")
    out = {}
    for mode in ("graph", "no-graph"):
        d = tmp_path / mode
        d.mkdir()
        conf = _write_conf(case, str(d))
        cmd = [exe, "-c", conf] + (["--with-mu-one"] if case.mu_one else [])
        if mode == "no-graph":
            cmd.append("--no-graph")
        r = subprocess.run(cmd, capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        out[mode] = {f: open(os.path.join(d, f), "rb").read()
                     for f in sorted(os.listdir(d))
                     if f.endswith((".bin", ".txt"))}
    assert out["graph"].keys() == out["no-graph"].keys()
    for f in out["graph"]:
        assert out["graph"][f] == out["no-graph"][f], f


# FCFC's long options and the keys they set (src/fcfc/2pt_box/load_conf.c:
# 477-515, src/fcfc/2pt/load_conf.c:512-553)
LONG_OPTS = {
    "CATALOG": "input", "CATALOG_LABEL": "label", "CATALOG_TYPE": "type",
    "ASCII_SKIP": "skip", "ASCII_COMMENT": "comment",
    "ASCII_FORMATTER": "formatter", "POSITION": "position",
    "WEIGHT": "weight", "SELECTION": "select", "COORD_CONVERT": "convert",
    "OMEGA_M": "omega-m", "OMEGA_LAMBDA": "omega-l", "DE_EOS_W": "eos-w",
    "CMVDST_ERR": "cmvdst-err", "Z_CMVDST_FILE": "cmvdst-file",
    "BOX_SIZE": "box", "DATA_STRUCT": "data-struct",
    "BINNING_SCHEME": "bin", "PAIR_COUNT": "pair",
    "PAIR_COUNT_FILE": "pair-output", "CF_ESTIMATOR": "cf",
    "CF_OUTPUT_FILE": "cf-output", "MULTIPOLE": "multipole",
    "MULTIPOLE_FILE": "mp-output", "PROJECTED_CF": "wp",
    "PROJECTED_FILE": "wp-output", "SEP_BIN_FILE": "s-file",
    "SEP_BIN_MIN": "s-min", "SEP_BIN_MAX": "s-max", "SEP_BIN_SIZE": "s-step",
    "MU_BIN_NUM": "mu-num", "PI_BIN_FILE": "pi-file", "PI_BIN_MIN": "pi-min",
    "PI_BIN_MAX": "pi-max", "PI_BIN_SIZE": "pi-step",
    "OUTPUT_FORMAT": "out-format", "OVERWRITE": "overwrite",
    "VERBOSE": "verbose",
}


@pytest.mark.parametrize("name", case_names())
def test_driver_from_command_line_options_alone(name, tmp_path):
    """Every key of the golden case given as FCFC's long option, with no
    configuration file: the same files as the configuration-file run."""
    case = Case(name)
    exe = os.path.join(BIN, "FCFC_2PT_BOX_GPU" if case.box else "FCFC_2PT_GPU")
    extra = ["--with-mu-one"] if case.mu_one else []
    out = {}
    for mode in ("file", "options"):
        d = tmp_path / mode
        d.mkdir()
        conf = _write_conf(case, str(d))
        inputs = set(os.listdir(d))
        if mode == "file":
            cmd = [exe, "-c", conf]
        else:
            cmd = [exe]
            for line in open(conf).read().splitlines():
                if "=" not in line or line.lstrip().startswith("#"):
                    continue
                key, val = (t.strip() for t in line.split("=", 1))
                cmd.append("--%s=%s" % (LONG_OPTS[key], val))
            os.remove(conf)
        r = subprocess.run(cmd + extra, capture_output=True, text=True,
                           cwd=str(d))
        assert r.returncode == 0, r.stderr
        out[mode] = {f: open(os.path.join(d, f), "rb").read()
                     for f in sorted(os.listdir(d))
                     if f not in inputs}
    assert out["file"].keys() == out["options"].keys() and out["file"]
    for f in out["file"]:
        assert out["file"][f] == out["options"][f], f


@pytest.mark.parametrize("runner", [False, True], ids=["driver", "runner"])
def test_multipoles_sorted_without_duplicates(runner, tmp_path):
    """MULTIPOLE = [4, 2, 0, 2] gives FCFC's file for [0, 2, 4]: FCFC sorts
    the orders and drops duplicates (load_conf.c:915-941)."""
    case = Case("box_smu_auto")
    conf = _write_conf(case, str(tmp_path))
    text = open(conf).read().replace("MULTIPOLE = [0, 2, 4]",
                                     "MULTIPOLE = [4, 2, 0, 2]")
    assert "[4, 2, 0, 2]" in text
    open(conf, "w").write(text)
    if runner:
        from fcfc_gb300 import runner as rn
        rn.run(rn.parse_conf(text), "box")
    else:
        r = subprocess.run([os.path.join(BIN, "FCFC_2PT_BOX_GPU"), "-c", conf],
                           capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
    assert open(tmp_path / "mp.txt").read() == \
        open(os.path.join(case.dir, "mp.txt")).read()


@pytest.mark.parametrize("runner", [False, True], ids=["driver", "runner"])
def test_unit_weight_counts_without_weights(runner, tmp_path):
    """WEIGHT = 1 is FCFC's way of saying no weights: the integer pair-count
    file of the unweighted golden case, byte for byte."""
    case = Case("box_smu_auto")
    conf = _write_conf(case, str(tmp_path))
    text = open(conf).read()
    assert "WEIGHT" not in text
    text += "WEIGHT = [1]\n"
    open(conf, "w").write(text)
    if runner:
        from fcfc_gb300 import runner as rn
        rn.run(rn.parse_conf(text), "box")
    else:
        r = subprocess.run([os.path.join(BIN, "FCFC_2PT_BOX_GPU"), "-c", conf],
                           capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
    for pair in case.meta["pairs"]:
        assert open(tmp_path / (pair + ".bin"), "rb").read() == \
            open(os.path.join(case.dir, pair + ".bin"), "rb").read(), pair


def test_catalogue_errors_from_the_reading_thread(tmp_path):
    """A catalogue that cannot be read, or a line that does not parse, is
    reported (the catalogues are read on a helper thread while the device is
    set up) and the run ends with an error and no pair-count file."""
    good = tmp_path / "d.txt"
    np.savetxt(good, np.random.default_rng(1).random((100, 3)) * 50.0)
    bad = tmp_path / "bad.txt"
    bad.write_text("1 2 3\n4 five 6\n")
    for cat, word in ((tmp_path / "missing.txt", "cannot read"),
                      (bad, "failed to read line 2")):
        conf = tmp_path / "c.conf"
        conf.write_text(
            "CATALOG = [%s]\nCATALOG_LABEL = [D]\nASCII_FORMATTER = "
            "[\"%%lf %%lf %%lf\"]\nPOSITION = [$1, $2, $3]\nBOX_SIZE = 100\n"
            "BINNING_SCHEME = 0\nSEP_BIN_MIN = 0\nSEP_BIN_MAX = 10\n"
            "SEP_BIN_SIZE = 1\nPAIR_COUNT = [DD]\nPAIR_COUNT_FILE = [%s]\n"
            "OVERWRITE = 2\n" % (cat, tmp_path / "dd.bin"))
        r = subprocess.run([os.path.join(BIN, "FCFC_2PT_BOX_GPU"), "-c",
                            str(conf)], capture_output=True, text=True)
        assert r.returncode != 0 and word in r.stderr, r.stderr
        assert not (tmp_path / "dd.bin").exists()
