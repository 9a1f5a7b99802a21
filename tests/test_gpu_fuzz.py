"""Randomised configurations: geometry, binning, linear or log edges, grid
refinement (1 to 8 cells per maximum separation), clustered or uniform
catalogues, weights, auto and cross counts.  The FP32 + FP64-recheck path
must give exactly the all-FP64 path's integer counts, and its weighted sums
within 1e-10; every tenth case is also checked against the oracle.  The
adjoint is checked against the oracle's per-object gradients over random
binnings and geometries as well."""
import zlib

import numpy as np
import pytest

from oracle import fcfc_oracle as fo

pytestmark = pytest.mark.gpu

NCASE = 96


def _bins(rng, geom, bt):
    """Random binning keywords (engine) and the oracle's."""
    kw = {}
    logs = rng.random() < 0.5
    smax = float(rng.uniform(8, 40))
    if logs:
        lo = float(rng.uniform(0.05, 1.0))
        ns = int(rng.integers(4, 30))
        kw["sedges"] = np.geomspace(lo, smax, ns + 1)
    else:
        ds = float(rng.choice([0.5, 1.0, 2.0, 2.5]))
        smin = float(rng.choice([0.0, 0.0, 1.0, 2.5]))
        ns = max(1, int((smax - smin) / ds))
        kw.update(smin=smin, smax=smin + ns * ds, ds=ds)
    if bt == 1:
        kw["nmu"] = int(rng.integers(1, 40))
    if bt == 2:
        dpi = float(rng.choice([1.0, 2.0, 2.5]))
        npi = int(rng.integers(2, int(30 / dpi) + 1))   # pi_max < L/2
        kw.update(pmin=0.0, pmax=npi * dpi, dpi=dpi)
    return kw


def _oracle_kw(kw):
    from fcfc_gb300 import capi
    lib = capi.load_library()
    okw = dict(kw)
    if "sedges" in okw:
        se = okw.pop("sedges")
        okw = dict(ns=len(se) - 1, sedges=se, **okw)
    else:
        okw["ns"] = lib.fcfcg_linear_nbin(okw["smin"], okw.pop("smax"),
                                          okw["ds"])
    if "pmax" in okw:
        okw["np_"] = lib.fcfcg_linear_nbin(okw["pmin"], okw.pop("pmax"),
                                           okw["dpi"])
    return okw


@pytest.mark.parametrize("case", range(NCASE))
def test_fp32_recheck_equals_fp64(case):
    import fcfc_gb300 as fg
    from fcfc_gb300 import synth
    rng = np.random.default_rng(zlib.crc32(b"fuzz%d" % case))
    geom = "box" if rng.random() < 0.6 else "survey"
    bt = int(rng.integers(0, 3))
    kw = _bins(rng, geom, bt)
    weighted = rng.random() < 0.5
    n1, n2 = int(rng.integers(300, 5000)), int(rng.integers(300, 5000))
    if geom == "box":
        L = float(rng.uniform(90, 200))
        if rng.random() < 0.5:
            a = synth.neyman_scott(max(1, n1 // 40), L, 40, 3.0,
                                   seed=int(rng.integers(1 << 30)))
        else:
            a = synth.uniform_box(n1, L, seed=int(rng.integers(1 << 30)))
        b = synth.uniform_box(n2, L, seed=int(rng.integers(1 << 30)))
        pc = fg.PairCounter("box", bt, box=L, **kw)
    else:
        sk = dict(ra=(150.0, 162.0), dec=(10.0, 20.0), zmu=0.5, zsig=0.05,
                  zr=(0.45, 0.55))
        a = synth.radecz_to_xyz(synth.survey_radecz(
            n1, seed=int(rng.integers(1 << 30)), **sk))
        b = synth.radecz_to_xyz(synth.survey_radecz(
            n2, seed=int(rng.integers(1 << 30)), **sk))
        pc = fg.PairCounter("survey", bt, **kw)
    wa = rng.lognormal(0, 0.4, len(a)) if weighted else None
    wb = rng.uniform(0.3, 2.0, len(b)) if weighted else None
    pc.load(0, a, wa)
    pc.load(1, b, wb)
    k = int(rng.integers(1, 9))
    try:
        pc.set_cells_per_smax(k)
        for pair in ((0, None), (0, 1)):
            c32 = pc.count_pairs(*pair, weighted=weighted, precision=0)
            c64 = pc.count_pairs(*pair, weighted=weighted, precision=1)
            what = "case %d %s bt%d k%d %s %s" % (case, geom, bt, k,
                                                 "wt" if weighted else "unwt",
                                                 pair)
            if weighted:
                np.testing.assert_allclose(c32, c64, rtol=1e-10, atol=1e-12,
                                           err_msg=what)
            else:
                np.testing.assert_array_equal(c32, c64, err_msg=what)
            if case % 10 == 0:
                ob = fo.Bins(geom == "survey", bt,
                             box=None if geom == "survey" else L,
                             **_oracle_kw(kw))
                ref = (ob.count(a, wa=wa, weighted=weighted) if pair[1] is None
                       else ob.count(a, b, wa=wa, wb=wb, weighted=weighted))
                if weighted:
                    np.testing.assert_allclose(c32, ref, rtol=1e-10,
                                               atol=1e-12, err_msg=what)
                else:
                    np.testing.assert_array_equal(c32, ref, err_msg=what)
    except fg.FCFCGError as e:
        # only a fine refinement can make a stencil beyond the limit, and it
        # is refused cleanly
        assert k >= 6 and "stencil" in str(e), (k, str(e))
    finally:
        pc.close()


@pytest.mark.parametrize("case", range(16))
def test_adjoint_random_matches_oracle(case):
    """Weight gradients (fcfcg_adjoint) over random binnings and geometries,
    log bins included (the bit-pattern table variants in boxes), against the
    oracle's per-object FP64 gradients."""
    import fcfc_gb300 as fg
    from fcfc_gb300 import synth
    rng = np.random.default_rng(zlib.crc32(b"adj%d" % case))
    geom = "box" if case % 2 == 0 else "survey"
    bt = int(rng.integers(0, 3))
    kw = _bins(rng, geom, bt)
    if geom == "box":
        L = float(rng.uniform(100, 200))
        a = synth.neyman_scott(int(rng.integers(10, 60)), L, 30, 3.0,
                               seed=int(rng.integers(1 << 30)))
        b = synth.uniform_box(int(rng.integers(500, 2000)), L,
                              seed=int(rng.integers(1 << 30)))
        pc = fg.PairCounter("box", bt, box=L, **kw)
        ob = fo.Bins(False, bt, box=L, **_oracle_kw(kw))
    else:
        sk = dict(ra=(150.0, 160.0), dec=(10.0, 18.0), zmu=0.5, zsig=0.05,
                  zr=(0.45, 0.55))
        a = synth.radecz_to_xyz(synth.survey_radecz(
            int(rng.integers(500, 2500)), seed=int(rng.integers(1 << 30)),
            **sk))
        b = synth.radecz_to_xyz(synth.survey_radecz(
            int(rng.integers(500, 2500)), seed=int(rng.integers(1 << 30)),
            **sk))
        pc = fg.PairCounter("survey", bt, **kw)
        ob = fo.Bins(True, bt, **_oracle_kw(kw))
    wa = rng.lognormal(0, 0.3, len(a))
    wb = rng.uniform(0.5, 1.5, len(b))
    pc.load(0, a, wa)
    pc.load(1, b, wb)
    g = rng.normal(size=pc.ntot)
    try:
        got, _ = pc.adjoint(0, None, g)
        want, _ = ob.adjoint(a, g, wa=wa)
        np.testing.assert_allclose(got, want, rtol=1e-10,
                                   atol=1e-12 * max(1.0, np.abs(want).max()))
        got_a, got_b = pc.adjoint(0, 1, g)
        want_a, want_b = ob.adjoint(a, g, b=b, wa=wa, wb=wb)
        np.testing.assert_allclose(got_a, want_a, rtol=1e-10,
                                   atol=1e-12 * max(1.0, np.abs(want_a).max()))
        np.testing.assert_allclose(got_b, want_b, rtol=1e-10,
                                   atol=1e-12 * max(1.0, np.abs(want_b).max()))
    finally:
        pc.close()


@pytest.mark.parametrize("case", range(12))
def test_survey_wide_low_redshift(case):
    """Surveys over the whole sky at low redshift (objects a few outer radii
    from the observer, lines of sight in every direction; for (s_perp, pi)
    some within the radius where the line-of-sight prefilter is off): the
    FP32 path gives the FP64 path's counts exactly, and the oracle's on
    every other case.  Cases 0-7 bin in (s_perp, pi), 8-9 in (s, mu),
    10-11 in s."""
    import fcfc_gb300 as fg
    from fcfc_gb300 import synth
    rng = np.random.default_rng(zlib.crc32(b"wide%d" % case))
    zlo = float(rng.uniform(0.003, 0.02))
    sk = dict(ra=(0.0, 360.0), dec=(-90.0, 90.0), zmu=2 * zlo, zsig=zlo,
              zr=(zlo, 4 * zlo))
    a = synth.radecz_to_xyz(synth.survey_radecz(
        int(rng.integers(1500, 4000)), seed=int(rng.integers(1 << 30)), **sk))
    b = synth.radecz_to_xyz(synth.survey_radecz(
        int(rng.integers(1500, 4000)), seed=int(rng.integers(1 << 30)), **sk))
    weighted = bool(case % 2)
    wa = rng.uniform(0.5, 1.5, len(a)) if weighted else None
    bt = 2 if case < 8 else (1 if case < 10 else 0)
    kw = dict(smin=0.0, smax=float(rng.choice([10.0, 20.0, 30.0])), ds=1.0)
    if bt == 2:
        kw.update(pmin=0.0, pmax=float(rng.choice([5.0, 10.0, 20.0])),
                  dpi=1.0)
    if bt == 1:
        kw["nmu"] = int(rng.integers(5, 40))
    pc = fg.PairCounter("survey", bt, **kw)
    pc.load(0, a, wa)
    pc.load(1, b, None)
    try:
        for pair in ((0, None), (0, 1)):
            c32 = pc.count_pairs(*pair, weighted=weighted, precision=0)
            assert pc.stats()["precision_used"] == 0
            c64 = pc.count_pairs(*pair, weighted=weighted, precision=1)
            if weighted:
                np.testing.assert_allclose(c32, c64, rtol=1e-10, atol=1e-12)
            else:
                np.testing.assert_array_equal(c32, c64)
            if case % 2 == 0:
                ob = fo.Bins(True, bt, **_oracle_kw(kw))
                ref = (ob.count(a) if pair[1] is None else ob.count(a, b))
                np.testing.assert_array_equal(c32, ref)
    finally:
        pc.close()
