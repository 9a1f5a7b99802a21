"""GPU parity: libfcfcg.so counts against the upstream golden files and the
oracle.  Integer counts must be identical; weighted sums within 1e-10
relative (the engine accumulates weight products in 128-bit fixed point,
the reference in FP64)."""
import zlib

import numpy as np
import pytest

from golden_cases import Case, case_names
from oracle import fcfc_oracle as fo

pytestmark = pytest.mark.gpu

WT_RTOL = 1e-10

CASES = case_names(convert=False)


def engine_for(case):
    import fcfc_gb300 as fg
    kw = case.bins_kwargs()
    bt = kw.pop("bintype")
    ns = kw.pop("ns")
    args = dict(geometry="box" if case.box else "survey", bintype=bt)
    if "sedges" in kw:
        args["sedges"] = kw["sedges"]
    else:
        args.update(smin=kw["smin"], ds=kw["ds"], smax=kw["smin"] + kw["ds"] * ns)
    if bt == 1:
        args["nmu"] = kw["nmu"]
    if bt == 2:
        args.update(pmin=kw["pmin"], dpi=kw["dpi"],
                    pmax=kw["pmin"] + kw["dpi"] * kw["np_"])
    if case.box:
        args["box"] = kw["box"]
    if kw.get("with_mu_one"):
        args["with_mu_one"] = True
    return fg.PairCounter(**args)


def _assert_counts(got, ref, weighted, what):
    assert got.shape == ref.shape, what
    if weighted:
        np.testing.assert_allclose(got, ref, rtol=WT_RTOL, atol=1e-300,
                                   err_msg=what)
    else:
        bad = np.nonzero(got != ref)[0]
        assert bad.size == 0, "%s: %d bins differ, first %s: %s vs %s" % (
            what, bad.size, bad[:5], got[bad[:5]], ref[bad[:5]])


@pytest.mark.parametrize("prec", [0, 1], ids=["fp32", "fp64"])
@pytest.mark.parametrize("name", CASES)
def test_golden_counts(name, prec):
    case = Case(name)
    pc = engine_for(case)
    slots = {}
    for i, lab in enumerate(case.meta["labels"]):
        x, w = case.xyzw(lab)
        pc.load(i, x, w)
        slots[lab] = i
    for pair in case.meta["pairs"]:
        ref = case.pcfile(pair)
        a, b = slots[pair[0]], slots[pair[1]]
        got = pc.count_pairs(a, None if a == b else b, weighted=ref.weighted,
                             precision=prec)
        if a == b:
            got = got * 2
        _assert_counts(got, ref.cnt, ref.weighted, "%s %s" % (name, pair))


def _random_box(rng, n, box, clustered=False, f32=False):
    from fcfc_gb300 import synth
    if clustered:
        x = synth.neyman_scott(max(n // 50, 1), box, 50, 4.0,
                               seed=int(rng.integers(1 << 30)), float32=f32)
    else:
        x = synth.uniform_box(n, box, seed=int(rng.integers(1 << 30)))
        if f32:
            x = x.astype(np.float32).astype(np.float64)
    return x


CONFIGS = [
    # (name, geometry, bintype, binning kwargs)
    ("box_smu_lin", "box", 1, dict(smin=0, smax=40, ds=2, nmu=25)),
    ("box_smu_smin", "box", 1, dict(smin=3, smax=33, ds=1.5, nmu=7)),
    ("box_iso_lin", "box", 0, dict(smin=0, smax=35, ds=0.5)),
    ("box_spi_lin", "box", 2, dict(smin=0, smax=30, ds=3, pmin=0, pmax=20, dpi=1)),
    ("box_spi_log", "box", 2, dict(sedges=np.geomspace(0.2, 30, 16), pmin=0,
                                   pmax=25, dpi=2.5)),
    ("box_iso_log", "box", 0, dict(sedges=np.geomspace(0.05, 30, 25))),
    ("box_smu_log", "box", 1, dict(sedges=np.geomspace(0.1, 40, 30), nmu=12)),
]


@pytest.mark.parametrize("weighted", [False, True], ids=["unwt", "wt"])
@pytest.mark.parametrize("clustered", [False, True], ids=["uniform", "ns"])
@pytest.mark.parametrize("cfg", CONFIGS, ids=[c[0] for c in CONFIGS])
def test_box_vs_oracle(cfg, clustered, weighted):
    import fcfc_gb300 as fg
    name, geom, bt, kw = cfg
    rng = np.random.default_rng(zlib.crc32(("%s%d%d" % (name, clustered, weighted)).encode()))
    box = 150.0
    x = _random_box(rng, 6000, box, clustered=clustered, f32=clustered)
    w = rng.lognormal(0, 0.3, len(x)) if weighted else None
    pc = fg.PairCounter(geom, bt, box=box, **kw)
    okw = dict(kw)
    if "sedges" in okw:
        se = okw.pop("sedges")
        okw = dict(ns=len(se) - 1, sedges=se, **okw)
    else:
        okw["ns"] = fg.capi.load_library().fcfcg_linear_nbin(
            okw["smin"], okw.pop("smax"), okw["ds"])
    if bt == 2:
        okw["np_"] = fg.capi.load_library().fcfcg_linear_nbin(
            okw["pmin"], okw.pop("pmax"), okw["dpi"])
    ob = fo.Bins(False, bt, box=box, **okw)
    pc.load(0, x, w)
    ref = ob.count(x, wa=w, weighted=weighted)
    for prec in (0, 1):
        got = pc.count_pairs(0, weighted=weighted, precision=prec)
        _assert_counts(got, ref, weighted, "%s prec %d" % (name, prec))
    # cross count with a second catalogue
    y = _random_box(rng, 4000, box)
    pc.load(1, y, None)
    refx = ob.count(x, y, wa=w, weighted=weighted)
    got = pc.count_pairs(0, 1, weighted=weighted)
    _assert_counts(got, refx, weighted, "%s cross" % name)


SURVEY_CONFIGS = [
    ("sv_smu", 1, dict(smin=0, smax=40, ds=4, nmu=20)),
    ("sv_spi_lin", 2, dict(smin=0, smax=30, ds=3, pmin=0, pmax=30, dpi=3)),
    ("sv_spi_log", 2, dict(sedges=np.geomspace(0.5, 30, 12), pmin=0, pmax=30,
                           dpi=2)),
    ("sv_iso", 0, dict(smin=2, smax=40, ds=2)),
]


@pytest.mark.parametrize("weighted", [False, True], ids=["unwt", "wt"])
@pytest.mark.parametrize("cfg", SURVEY_CONFIGS, ids=[c[0] for c in SURVEY_CONFIGS])
def test_survey_vs_oracle(cfg, weighted):
    import fcfc_gb300 as fg
    from fcfc_gb300 import synth
    name, bt, kw = cfg
    kws = dict(ra=(150.0, 165.0), dec=(10.0, 22.0), zmu=0.5, zsig=0.05,
               zr=(0.45, 0.55))
    d = synth.radecz_to_xyz(synth.survey_radecz(4000, seed=5, **kws))
    r = synth.radecz_to_xyz(synth.survey_radecz(8000, seed=6, **kws))
    rng = np.random.default_rng(7)
    wd = rng.uniform(0.2, 1.0, len(d)) if weighted else None
    pc = fg.PairCounter("survey", bt, **kw)
    okw = dict(kw)
    if "sedges" in okw:
        se = okw.pop("sedges")
        okw = dict(ns=len(se) - 1, sedges=se, **okw)
    else:
        okw["ns"] = fg.capi.load_library().fcfcg_linear_nbin(
            okw["smin"], okw.pop("smax"), okw["ds"])
    if bt == 2:
        okw["np_"] = fg.capi.load_library().fcfcg_linear_nbin(
            okw["pmin"], okw.pop("pmax"), okw["dpi"])
    ob = fo.Bins(True, bt, **okw)
    pc.load(0, d, wd)
    pc.load(1, r, None)
    for prec in (0, 1):
        _assert_counts(pc.count_pairs(0, weighted=weighted, precision=prec),
                       ob.count(d, wa=wd, weighted=weighted), weighted,
                       "%s DD prec %d" % (name, prec))
        # these separations keep the FP32 windows narrow: no FP64 fallback
        assert pc.stats()["precision_used"] == prec
        _assert_counts(pc.count_pairs(0, 1, weighted=weighted, precision=prec),
                       ob.count(d, r, wa=wd, weighted=weighted), weighted,
                       "%s DR prec %d" % (name, prec))


def test_survey_spi_line_of_sight_prefilter():
    """(s_perp, pi) in a survey: the FP32 kernel drops pairs whose pi is
    beyond pi_max for sure, judging the line of sight by one point's
    direction.  Objects around the observer (where that test is switched
    off), at the origin itself, and pairs placed with pi just inside and
    just outside pi_max must give the oracle's counts."""
    import fcfc_gb300 as fg
    rng = np.random.default_rng(41)
    pmax, spmax = 30.0, 30.0
    ball = rng.normal(size=(2500, 3))
    ball *= (80.0 * rng.random(2500) ** (1 / 3) / np.linalg.norm(ball, axis=1))[:, None]
    far = rng.normal(size=(1500, 3))
    far *= (rng.uniform(250, 400, 1500) / np.linalg.norm(far, axis=1))[:, None]
    # pairs straddling pi = pi_max along their own line of sight
    n = 400
    u = rng.normal(size=(n, 3))
    u /= np.linalg.norm(u, axis=1)[:, None]
    xb = u * rng.uniform(100, 2000, n)[:, None]
    perp = rng.normal(size=(n, 3))
    perp -= (perp * u).sum(1)[:, None] * u
    perp /= np.linalg.norm(perp, axis=1)[:, None]
    dpi = pmax + rng.choice([-1e-3, -1e-7, 0.0, 1e-7, 1e-3, 0.5], n)
    dpi *= rng.choice([-1.0, 1.0], n)
    d = dpi[:, None] * u + perp * rng.uniform(0, spmax, n)[:, None]
    # x_a - x_b = d with the pair's line of sight x_a + x_b along u:
    # x_a = c + d / 2, x_b = c - d / 2 for a centre c on u
    xa2, xb2 = xb + 0.5 * d, xb - 0.5 * d
    x = np.concatenate([ball, [[0.0, 0.0, 0.0]], far, xa2, xb2])
    y = np.concatenate([rng.normal(size=(2000, 3)) * 40.0, xb2])
    w = rng.uniform(0.3, 1.7, len(x))
    kw = dict(smin=0, smax=spmax, ds=3, pmin=0, pmax=pmax, dpi=3)
    pc = fg.PairCounter("survey", 2, **kw)
    lib = fg.capi.load_library()
    ob = fo.Bins(True, 2, ns=lib.fcfcg_linear_nbin(0, spmax, 3), smin=0, ds=3,
                 np_=lib.fcfcg_linear_nbin(0, pmax, 3), pmin=0, dpi=3)
    pc.load(0, x, w)
    pc.load(1, y, None)
    for weighted in (False, True):
        _assert_counts(pc.count_pairs(0, weighted=weighted, precision=0),
                       ob.count(x, wa=w, weighted=weighted), weighted,
                       "los DD")
        assert pc.stats()["precision_used"] == 0
        _assert_counts(pc.count_pairs(0, 1, weighted=weighted, precision=0),
                       ob.count(x, y, wa=w, weighted=weighted), weighted,
                       "los DR")


def test_edge_cases():
    """Empty and single-object catalogues, duplicate points (s = 0), points
    on the box faces and on cell boundaries."""
    import fcfc_gb300 as fg
    box = 100.0
    pc = fg.PairCounter("box", 1, box=box, smin=0, smax=20, ds=2, nmu=10)
    ob = fo.Bins(False, 1, ns=10, smin=0, ds=2, nmu=10, box=box)
    pc.load(0, np.zeros((0, 3)))
    assert pc.count_pairs(0).sum() == 0
    pc.load(1, np.array([[1.0, 2.0, 3.0]]))
    assert pc.count_pairs(1).sum() == 0
    assert pc.count_pairs(0, 1).sum() == 0
    # duplicates, faces, cell edges, exact bin edges
    pts = [[0, 0, 0], [0, 0, 0], [0, 0, 10], [99.999999, 0, 0], [50, 50, 50],
           [50, 50, 52], [50, 52, 50], [52, 50, 50], [0, 0, 99.9999999999],
           [25.0, 25.0, 25.0], [25.0, 25.0, 45.0], [33.333333333333336] * 3]
    rng = np.random.default_rng(3)
    grid = np.stack(np.meshgrid(*[np.arange(0, box, 12.5)] * 3), -1).reshape(-1, 3)
    x = np.concatenate([np.array(pts, float), grid, rng.random((500, 3)) * box])
    pc.load(2, x)
    for prec in (0, 1):
        _assert_counts(pc.count_pairs(2, precision=prec), ob.count(x), False,
                       "edge prec %d" % prec)


def test_rejects_out_of_box():
    import fcfc_gb300 as fg
    pc = fg.PairCounter("box", 1, box=100.0, smin=0, smax=20, ds=2, nmu=10)
    with pytest.raises(fg.FCFCGError):
        pc.load(0, np.array([[150.0, 1.0, 1.0]]))


def test_bad_config():
    import fcfc_gb300 as fg
    with pytest.raises(fg.FCFCGError):       # s_max >= L/2
        fg.PairCounter("box", 1, box=30.0, smin=0, smax=20, ds=2, nmu=10)
