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
