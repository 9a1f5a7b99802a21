"""Full-size fixtures without a GPU: the benchmark catalogues regenerate to
the bytes FCFC counted (sha256), FCFC's files agree with the run
configurations, and the oracle reproduces FCFC's counts of the uniform box
(1e5 points, 167,540,844 unique pairs in (s, mu) 40 x 100)."""
import numpy as np
import pytest

from golden_cases import FullCase, full_case_names
from oracle import fcfc_oracle as fo

CASES = full_case_names()


def test_fixtures_present():
    assert set(CASES) >= {"c0_box_uniform", "c1_box_ns", "c1_box_ns_f32",
                          "c2_survey_ls", "c3_mocks"}


@pytest.mark.parametrize("name", CASES)
def test_catalogues_regenerate(name):
    c = FullCase(name)
    for lab, m in c.meta["cats"].items():
        a, got, want = c.catalogue(lab)
        assert got == want, "%s/%s regenerated to other bytes" % (name, lab)
        assert len(a) == m["n"]


@pytest.mark.parametrize("name", CASES)
def test_files_match_runs(name):
    c = FullCase(name)
    for run in c.runs():
        if run.get("fcfc_rejected"):
            assert "BOX_SIZE" in run["fcfc_message"] or "box" in run["fcfc_message"].lower()
            assert 2 * run["sbin"]["smax"] >= run["box"][0]
            continue
        for pair in run["pairs"]:
            f = c.pcfile(run, pair)
            assert f.bintype == run["bintype"] and f.weighted == run["weighted"]
            assert f.auto == (pair[0] == pair[1])
            assert f.periodic == c.box
            assert f.cnt.size == f.ns * max(f.n2, 1)


def test_uniform_box_total_and_oracle():
    c = FullCase("c0_box_uniform")
    run = c.runs()[0]
    ref = c.pcfile(run, "DD")
    assert int(ref.cnt.sum()) == 2 * 167540844
    x, _, _ = c.catalogue("D")
    ob = fo.Bins(False, 1, ns=40, smin=0, ds=5, nmu=100, box=1000.0)
    np.testing.assert_array_equal(2 * ob.count(x), ref.cnt)
