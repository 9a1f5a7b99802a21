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
