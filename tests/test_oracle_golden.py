"""The oracle against pair-count files written by the upstream FCFC.

Every golden case, every pair: integer counts must be identical, weighted
sums equal to 1e-12 relative (the upstream sums in thread order)."""
import numpy as np
import pytest

from golden_cases import Case, case_names
from oracle import fcfc_oracle as fo

CASES = [n for n in case_names() if not n.endswith("_cnvt")]


def _pairs(case):
    return [(p, case.meta["labels"]) for p in case.meta["pairs"]]


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("mode", [0, 1, 3])
def test_oracle_matches_reference(name, mode):
    case = Case(name)
    bins = fo.Bins(survey=not case.box, **case.bins_kwargs())
    for pair in case.meta["pairs"]:
        ref = case.pcfile(pair)
        a, wa = case.xyzw(pair[0])
        if pair[0] == pair[1]:
            got = bins.count(a, wa=wa, weighted=ref.weighted, mode=mode)
            got = got * 2
        else:
            b, wb = case.xyzw(pair[1])
            got = bins.count(a, b, wa=wa, wb=wb, weighted=ref.weighted, mode=mode)
        assert ref.cnt.shape == got.shape
        if ref.weighted:
            np.testing.assert_allclose(got, ref.cnt, rtol=1e-12, atol=0)
        else:
            assert np.array_equal(got, ref.cnt), (pair, np.nonzero(got != ref.cnt))
        if case.box:
            np.testing.assert_array_equal(bins.box(), ref.box)
