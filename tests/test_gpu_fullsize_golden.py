"""The benchmark workloads at their stated sizes against FCFC's own pair
counts (tests/golden/full, written by FCFC v1.0.1's FP64 build from the
regenerated catalogues): the FP32 + FP64-recheck path, the all-FP64 path
and the batched launch.  Integer counts must be identical; weighted sums
within 1e-10 relative (FCFC sums FP64 products in thread order, the engine
sums exact fixed-point products)."""
import numpy as np
import pytest

from golden_cases import FullCase

pytestmark = pytest.mark.gpu

WT_RTOL = 1e-10


def _check(got, ref, weighted, what):
    assert got.shape == ref.shape, what
    if weighted:
        np.testing.assert_allclose(got, ref, rtol=WT_RTOL, atol=1e-300,
                                   err_msg=what)
    else:
        bad = np.nonzero(got != ref)[0]
        assert bad.size == 0, "%s: %d bins differ, first %s: %s vs %s" % (
            what, bad.size, bad[:5], got[bad[:5]], ref[bad[:5]])


def _cat(case, lab):
    a, got, want = case.catalogue(lab)
    assert got == want, "%s/%s: catalogue regenerated to other bytes" % (
        case.name, lab)
    return a


@pytest.mark.parametrize("name", ["c0_box_uniform", "c1_box_ns",
                                  "c1_box_ns_f32"])
def test_box_full_size(name):
    import fcfc_gb300 as fg
    case = FullCase(name)
    a = _cat(case, "D")
    for run in case.runs():
        wt = run["weighted"]
        w = a[:, 3] if wt else None
        pc = fg.PairCounter(device=0, **case.engine_kwargs(run))
        pc.load(0, a[:, :3], w)
        ref = case.pcfile(run, "DD")
        for prec in (fg.PREC_FP32_RECHECK, fg.PREC_FP64):
            got = pc.count_pairs(0, weighted=wt, precision=prec) * 2
            _check(got, ref.cnt, wt, "%s %s prec %d" % (name, run["name"], prec))
            assert pc.stats()["precision_used"] == prec
        cnt, status, _ = pc.count_batch([a[:, :3]], [run["box"][0]],
                                        weights=[w] if wt else None,
                                        weighted=wt)
        assert status == [0]
        _check(cnt[0] * 2, ref.cnt, wt, "%s %s batch" % (name, run["name"]))
        if name == "c0_box_uniform":
            assert int(ref.cnt.sum()) == 2 * 167540844


def test_survey_ls_full_size():
    """1e5 data, 3e5 randoms: RA/Dec/z converted on the device (FCFC
    converted them itself), FKP weights, DD / DR / RR."""
    import fcfc_gb300 as fg
    case = FullCase("c2_survey_ls")
    d = _cat(case, "D")
    r = _cat(case, "R")
    for run in case.runs():
        wt = run["weighted"]
        pc = fg.PairCounter(device=0, **case.engine_kwargs(run))
        pc.load_radecz(0, d[:, :3], d[:, 3] if wt else None, omega_m=0.31,
                       cmvdst_err=1e-8)
        pc.load_radecz(1, r[:, :3], r[:, 3] if wt else None, omega_m=0.31,
                       cmvdst_err=1e-8)
        for pair, (sa, sb) in (("DD", (0, None)), ("DR", (0, 1)),
                               ("RR", (1, None))):
            ref = case.pcfile(run, pair)
            for prec in (fg.PREC_FP32_RECHECK, fg.PREC_FP64):
                got = pc.count_pairs(sa, sb, weighted=wt, precision=prec)
                if sb is None:
                    got = got * 2
                _check(got, ref.cnt, wt, "%s %s prec %d" % (run["name"], pair, prec))


def test_mocks_full_size():
    """Nine mocks of the batched workload in one launch: eight as FCFC
    counts them, the ninth refused as FCFC refuses it (s_max >= L / 2)."""
    import fcfc_gb300 as fg
    case = FullCase("c3_mocks")
    runs = case.runs()
    cats = [_cat(case, run["labels"][0]) for run in runs]
    boxes = [run["box"][0] for run in runs]
    refs = [None if run.get("fcfc_rejected") else case.pcfile(run, "DD")
            for run in runs]
    assert sum(r is None for r in refs) == 1
    pc = fg.PairCounter(device=0, **case.engine_kwargs(runs[0]))
    for prec in (fg.PREC_FP32_RECHECK, fg.PREC_FP64):
        cnt, status, _ = pc.count_batch(cats, boxes, precision=prec)
        for k, ref in enumerate(refs):
            if ref is None:
                assert status[k] == fg.capi.ERR_CFG
                continue
            assert status[k] == 0
            _check(cnt[k] * 2, ref.cnt, False, "mock %d prec %d" % (k, prec))
    # and one at a time through the ordinary entry point
    for k in (0, 3):
        one = fg.PairCounter(device=0, **case.engine_kwargs(runs[k]))
        one.load(0, cats[k])
        _check(one.count_pairs(0) * 2, refs[k].cnt, False, "mock %d single" % k)
