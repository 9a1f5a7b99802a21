"""The command line drivers without a GPU: usage text, and configuration
errors reported before any device work."""
import os
import subprocess

import pytest

BIN = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                   "fcfc_gb300", "bin")


@pytest.fixture(scope="module")
def drivers():
    from fcfc_gb300 import build
    build.build()
    return [os.path.join(BIN, n) for n in ("FCFC_2PT_BOX_GPU", "FCFC_2PT_GPU")]


def test_usage(drivers):
    for exe in drivers:
        r = subprocess.run([exe, "-h"], capture_output=True, text=True)
        assert r.returncode == 0 and "Usage" in r.stdout


def test_config_errors(drivers, tmp_path):
    conf = tmp_path / "c.conf"
    cases = [
        ("BINNING_SCHEME = 1\n", "CATALOG"),
        ("CATALOG = [a.txt]\nPOSITION = [$1, $2]\n", "POSITION"),
        ("CATALOG = [a.txt]\nCATALOG_TYPE = [1]\nPOSITION = [$1, $2, $3]\n",
         "ASCII"),
        ("CATALOG = [a.txt]\nPOSITION = [$1, $2, $3]\nDATA_STRUCT = 2\n",
         "DATA_STRUCT"),
        ("CATALOG = [a.txt]\nASCII_SKIP = [-1]\nPOSITION = [$1, $2, $3]\n",
         "ASCII_SKIP"),
        ("CATALOG = [a.txt]\nASCII_COMMENT = [' ']\nPOSITION = [$1, $2, $3]\n",
         "ASCII_COMMENT"),
    ]
    for text, word in cases:
        conf.write_text(text)
        r = subprocess.run([drivers[0], "-c", str(conf)], capture_output=True,
                           text=True)
        assert r.returncode != 0 and word in r.stderr, (text, r.stderr)
    r = subprocess.run([drivers[0], "-c", str(tmp_path / "missing.conf")],
                       capture_output=True, text=True)
    assert r.returncode != 0


def test_runner_rejects_data_struct():
    """The Python run flow rejects DATA_STRUCT values FCFC rejects (0 and 1,
    its k-d and ball trees, both map to the cell grid), before device work."""
    from fcfc_gb300 import runner
    from fcfc_gb300.capi import FCFCGError
    conf = runner.parse_conf("CATALOG = [a.txt]\nPOSITION = [$1, $2, $3]\n"
                             "DATA_STRUCT = 2\nPAIR_COUNT = [AA]\n")
    with pytest.raises(FCFCGError, match="DATA_STRUCT"):
        runner.run(conf, "box")


def _base_conf(extra=""):
    return ("CATALOG = [a.txt]\nPOSITION = [$1, $2, $3]\nBOX_SIZE = 100\n"
            "BINNING_SCHEME = 0\nSEP_BIN_MIN = 0\nSEP_BIN_MAX = 10\n"
            "SEP_BIN_SIZE = 1\n" + extra)


def test_version_and_template(drivers):
    for exe, key in zip(drivers, ("BOX_SIZE", "OMEGA_M")):
        r = subprocess.run([exe, "-V"], capture_output=True, text=True)
        assert r.returncode == 0 and r.stdout
        r = subprocess.run([exe, "--template"], capture_output=True, text=True)
        assert r.returncode == 0
        for k in ("CATALOG", "POSITION", "SEP_BIN_MIN", "PAIR_COUNT_FILE",
                  "VERBOSE", key):
            assert "\n%s = " % k in r.stdout, k


def test_command_line_beats_the_file(drivers, tmp_path):
    """FCFC's option table and libcfg's rules: an option sets its key over
    the file's value, in the -x VALUE, -x=VALUE, --long VALUE and
    --long=VALUE forms."""
    conf = tmp_path / "c.conf"
    conf.write_text(_base_conf("DATA_STRUCT = 2\n"))
    r = subprocess.run([drivers[0], "-c", str(conf)], capture_output=True,
                       text=True)
    assert r.returncode != 0 and "DATA_STRUCT" in r.stderr
    for opt in (["-S", "0"], ["-S=1"], ["--data-struct", "0"],
                ["--data-struct=1"]):
        r = subprocess.run([drivers[0], "-c", str(conf)] + opt,
                           capture_output=True, text=True)
        # past the bins: the next missing key is reported
        assert r.returncode != 0 and "PAIR_COUNT" in r.stderr, (opt, r.stderr)
    # a command line value also wins when it comes before -c
    r = subprocess.run([drivers[0], "--data-struct=0", "--conf", str(conf)],
                       capture_output=True, text=True)
    assert "PAIR_COUNT" in r.stderr, r.stderr


def test_first_value_of_a_key_is_kept(drivers, tmp_path):
    """A key given twice in the file keeps its first value (libcfg warns
    about the duplicate); twice on the command line likewise."""
    conf = tmp_path / "c.conf"
    conf.write_text(_base_conf("DATA_STRUCT = 0\nDATA_STRUCT = 2\n"))
    r = subprocess.run([drivers[0], "-c", str(conf)], capture_output=True,
                       text=True)
    assert "PAIR_COUNT" in r.stderr and "duplicate" in r.stderr, r.stderr
    conf.write_text(_base_conf())
    r = subprocess.run([drivers[0], "-c", str(conf), "-S", "3", "-S", "0"],
                       capture_output=True, text=True)
    assert "DATA_STRUCT" in r.stderr and "duplicate" in r.stderr, r.stderr


def test_options_without_a_configuration_file(drivers, tmp_path):
    """No readable configuration file: a warning, and the run goes on with
    the command line's keys alone."""
    r = subprocess.run([drivers[0], "-i", "a.txt", "-x", "[$1, $2, $3]",
                        "-b", "100", "-B", "0", "--s-min", "0", "--s-max",
                        "10", "--s-step=1"], capture_output=True, text=True,
                       cwd=str(tmp_path))
    assert r.returncode != 0
    assert "configuration file" in r.stderr and "PAIR_COUNT" in r.stderr, \
        r.stderr
    # a value-less non-Boolean option is an error; an unknown one a warning
    r = subprocess.run([drivers[0], "-B"], capture_output=True, text=True,
                       cwd=str(tmp_path))
    assert r.returncode != 0 and "argument not found" in r.stderr
    r = subprocess.run([drivers[0], "--no-such-option", "-B", "0"],
                       capture_output=True, text=True, cwd=str(tmp_path))
    assert "unrecognised" in r.stderr and "CATALOG" in r.stderr


def _pc_conf(tmp_path, extra):
    return _base_conf("CATALOG_LABEL = [D]\nPAIR_COUNT = [DD]\n"
                      "PAIR_COUNT_FILE = [%s]\n%s" % (tmp_path / "dd.bin", extra))


def test_overwrite_rules(drivers, tmp_path):
    """FCFC's check_output: OVERWRITE = 0 refuses an existing output, a
    negative value asks on the terminal, a missing directory is an error --
    all before any device work."""
    conf = tmp_path / "c.conf"
    (tmp_path / "dd.bin").write_bytes(b"x")
    run = lambda inp=None: subprocess.run(
        [drivers[0], "-c", str(conf)], capture_output=True, text=True,
        input=inp)
    conf.write_text(_pc_conf(tmp_path, "OVERWRITE = 0\n"))
    r = run()
    assert r.returncode != 0 and "abort to avoid overwriting" in r.stderr
    conf.write_text(_pc_conf(tmp_path, "OVERWRITE = -2\n"))
    for inp in ("", "x\nq\n"):
        r = run(inp)
        assert r.returncode != 0 and "too many failed inputs" in r.stderr, inp
    # an answer: no refusal (the run goes on to the catalogue or the device)
    for inp in ("n\n", "x\ny\n"):
        r = run(inp)
        assert "abort" not in r.stderr and "failed inputs" not in r.stderr, \
            (inp, r.stderr)
    # correlation function outputs: refused with 0, overwritten with 1
    (tmp_path / "dd.bin").unlink()
    (tmp_path / "xi.txt").write_text("old")
    est = 'CF_ESTIMATOR = ["DD / @@ - 1"]\nCF_OUTPUT_FILE = [%s]\n' % (
        tmp_path / "xi.txt")
    conf.write_text(_pc_conf(tmp_path, est + "OVERWRITE = 0\n"))
    r = run()
    assert "abort to avoid overwriting CF_OUTPUT_FILE" in r.stderr, r.stderr
    conf.write_text(_pc_conf(tmp_path, est + "OVERWRITE = 1\n"))
    r = run()
    assert "will be overwritten" in r.stderr and "abort" not in r.stderr
    conf.write_text(_base_conf("CATALOG_LABEL = [D]\nPAIR_COUNT = [DD]\n"
                               "PAIR_COUNT_FILE = [%s]\n"
                               % (tmp_path / "no" / "dd.bin")))
    r = run()
    assert "cannot access the directory" in r.stderr, r.stderr


def test_multipole_checks(drivers, tmp_path):
    conf = tmp_path / "c.conf"
    conf.write_text(_base_conf(
        "MU_BIN_NUM = 10\nCATALOG_LABEL = [D]\nPAIR_COUNT = [DD]\n"
        "PAIR_COUNT_FILE = [%s]\nCF_ESTIMATOR = [DD / @@ - 1]\n"
        "CF_OUTPUT_FILE = [%s]\nMULTIPOLE = [0, 8]\nMULTIPOLE_FILE = [%s]\n"
        % (tmp_path / "dd.bin", tmp_path / "xi.txt", tmp_path / "mp.txt")))
    # (s, mu) from the command line, over the file's BINNING_SCHEME = 0
    r = subprocess.run([drivers[0], "-c", str(conf), "-B", "1"],
                       capture_output=True, text=True)
    assert r.returncode != 0 and "MULTIPOLE must be" in r.stderr, r.stderr
    r = subprocess.run([drivers[0], "-c", str(conf), "-B", "1", "-m", "[2, 0]",
                        "-M", "[]"], capture_output=True, text=True)
    assert r.returncode != 0 and "MULTIPOLE_FILE is not set" in r.stderr


def test_runner_check_output(tmp_path):
    from fcfc_gb300 import runner
    from fcfc_gb300.capi import FCFCGError
    f = tmp_path / "dd.bin"
    assert runner.check_output(str(f), "PAIR_COUNT_FILE", 0, 2) is False
    f.write_bytes(b"x")
    with pytest.raises(FCFCGError, match="abort"):
        runner.check_output(str(f), "PAIR_COUNT_FILE", 0, 2)
    assert runner.check_output(str(f), "PAIR_COUNT_FILE", 1, 2) is True
    assert runner.check_output(str(f), "PAIR_COUNT_FILE", 2, 2) is False
    assert runner.check_output(str(f), "CF_OUTPUT_FILE", 1, 1) is False
    answers = iter(["maybe", "n"])
    assert runner.check_output(str(f), "PAIR_COUNT_FILE", -3, 2,
                               ask=lambda _: next(answers)) is True
    with pytest.raises(FCFCGError, match="failed inputs"):
        runner.check_output(str(f), "PAIR_COUNT_FILE", -1, 2,
                            ask=lambda _: "?")
    with pytest.raises(FCFCGError, match="directory"):
        runner.check_output(str(tmp_path / "no" / "x"), "CF_OUTPUT_FILE", 2, 1)


def test_labels_and_unit_weights(drivers, tmp_path):
    """CATALOG_LABEL: capital letters, each once; WEIGHT = 1 counts without
    weights (FCFC's load_conf.c:675-705, 780-789)."""
    conf = tmp_path / "c.conf"
    for lab, word in (("[d]", "invalid CATALOG_LABEL"),
                      ("[D, D]", "duplicate CATALOG_LABEL")):
        conf.write_text("CATALOG = [a.txt, b.txt]\nCATALOG_LABEL = %s\n" % lab)
        r = subprocess.run([drivers[0], "-c", str(conf)], capture_output=True,
                           text=True)
        assert r.returncode != 0 and word in r.stderr, (lab, r.stderr)
    from fcfc_gb300 import runner
    from fcfc_gb300.capi import FCFCGError
    with pytest.raises(FCFCGError, match="duplicate CATALOG_LABEL"):
        runner.run(runner.parse_conf("CATALOG = [a, b]\nCATALOG_LABEL = [D, D]\n"
                                     "POSITION = [$1,$2,$3,$1,$2,$3]\n"), "box")


def test_runner_command_line(tmp_path, monkeypatch):
    """python -m fcfc_gb300.runner takes FCFC's options too, over the file's
    values, and FCFC's default file name."""
    from fcfc_gb300 import runner
    from fcfc_gb300.capi import FCFCGError
    conf = tmp_path / "c.conf"
    conf.write_text(_base_conf("DATA_STRUCT = 2\n"))
    with pytest.raises(FCFCGError, match="DATA_STRUCT"):
        runner.main(["--box", "-c", str(conf)])
    with pytest.raises(FCFCGError, match="PAIR_COUNT is not set"):
        runner.main(["-c", str(conf), "-S", "0"])
    # the first value of a repeated option is kept
    with pytest.raises(FCFCGError, match="DATA_STRUCT"):
        runner.main(["-c", str(conf), "-S", "3", "-S", "0"])
    monkeypatch.chdir(tmp_path)
    with pytest.raises(FCFCGError, match="PAIR_COUNT is not set"):
        runner.main(["-b", "100", "-i", "a.txt", "-x", "[$1, $2, $3]",
                     "-B", "0", "--s-min", "0", "--s-max=10", "--s-step", "1"])


def test_estimators_checked_before_device_work(drivers, tmp_path):
    """An estimator naming a pair that is not counted, or one that does not
    parse, stops the run before any device work (FCFC's setup_cf.c:128-200)."""
    conf = tmp_path / "c.conf"
    for est in ("DR / @@ - 1", "DD / (@@ - 1"):
        conf.write_text(_pc_conf(tmp_path, 'CF_ESTIMATOR = ["%s"]\n'
                                 'CF_OUTPUT_FILE = [%s]\nOVERWRITE = 2\n'
                                 % (est, tmp_path / "xi.txt")))
        r = subprocess.run([drivers[0], "-c", str(conf)], capture_output=True,
                           text=True)
        assert r.returncode != 0 and "invalid CF_ESTIMATOR" in r.stderr, \
            (est, r.stderr)
    from fcfc_gb300 import runner
    from fcfc_gb300.capi import FCFCGError
    conf.write_text(_pc_conf(tmp_path, 'CF_ESTIMATOR = ["DR / @@ - 1"]\n'
                             'CF_OUTPUT_FILE = [%s]\nOVERWRITE = 2\n'
                             % (tmp_path / "xi.txt")))
    with pytest.raises(FCFCGError, match="invalid CF_ESTIMATOR"):
        runner.run(runner.parse_conf(conf.read_text()), "box")


def test_option_terminator_and_boolean_forms(drivers, tmp_path):
    """`--' ends the options (what follows is ignored, as in libcfg); a
    Boolean option takes T/F or stands alone for T."""
    conf = tmp_path / "c.conf"
    conf.write_text(_base_conf("DATA_STRUCT = 2\n"))
    r = subprocess.run([drivers[0], "-c", str(conf), "--", "-S", "0"],
                       capture_output=True, text=True)
    assert "DATA_STRUCT" in r.stderr, r.stderr
    for opt in (["-v", "F"], ["--verbose=T"], ["-v"], ["-u"], ["--wp", "F"]):
        r = subprocess.run([drivers[0], "-c", str(conf), "-S", "0"] + opt,
                           capture_output=True, text=True)
        assert "PAIR_COUNT" in r.stderr and "argument not found" not in \
            r.stderr, (opt, r.stderr)
