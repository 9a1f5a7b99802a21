"""The oracle against pair-count files written by the upstream FCFC.

Every golden case, every pair: integer counts must be identical, weighted
sums equal to 1e-12 relative (the upstream sums in thread order)."""
import numpy as np
import pytest

from golden_cases import Case, case_names
from oracle import fcfc_oracle as fo

CASES = case_names(convert=False)


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


def convert_with_oracle(case, label):
    """The catalogue's RA/Dec/z converted as FCFC converts it."""
    a = case.cats[label]
    zt = case.ztable()
    if zt is not None:
        xyz, bad = fo.convert_spline(a[:, :3], zt[:, 0], zt[:, 1])
        assert bad == 0
        return xyz, None
    c = case.cosmo()
    xyz, order = fo.convert_integr(a[:, :3], c["omega_m"], c["omega_l"],
                                   c["dew"], c["err"])
    return xyz, order


@pytest.mark.parametrize("name", case_names(convert=True))
def test_oracle_conversion_matches_reference(name):
    """COORD_CONVERT = T: RA/Dec/z converted by the oracle (integration or
    the Z_CMVDST_FILE spline), then counted, gives FCFC's files; the
    unweighted cases pin the converted coordinates bit for bit through the
    integer counts."""
    case = Case(name)
    bins = fo.Bins(survey=True, **case.bins_kwargs())
    conv = {l: convert_with_oracle(case, l)[0] for l in case.meta["labels"]}
    for pair in case.meta["pairs"]:
        ref = case.pcfile(pair)
        wa = case.xyzw(pair[0])[1]
        if pair[0] == pair[1]:
            got = bins.count(conv[pair[0]], wa=wa, weighted=ref.weighted,
                             mode=3) * 2
        else:
            wb = case.xyzw(pair[1])[1]
            got = bins.count(conv[pair[0]], conv[pair[1]], wa=wa, wb=wb,
                             weighted=ref.weighted, mode=3)
        if ref.weighted:
            np.testing.assert_allclose(got, ref.cnt, rtol=1e-12, atol=0)
        else:
            assert np.array_equal(got, ref.cnt), (pair, np.nonzero(got != ref.cnt))


@pytest.mark.parametrize("name", [n for n in case_names(convert=True)
                                  if Case(n).ztable() is None])
def test_oracle_conversion_orders(name):
    """The Gauss-Legendre order matches the one FCFC reported for each
    catalogue (its verbose output, recorded in the fixture)."""
    case = Case(name)
    got = [convert_with_oracle(case, l)[1] for l in case.meta["labels"]]
    assert got == case.meta["cnvt_order"]
