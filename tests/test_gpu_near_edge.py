"""Pairs on FCFC's bin boundaries (tests/edge_pairs.py): for each boundary
of a binning, pairs whose FP64 value, computed as FCFC computes it, is the
edge itself and the 1st, 2nd and 4th reachable values on either side (single
ulps in a box; the grid of FCFC's own S - t arithmetic for survey objects
1000-1750 Mpc/h away).  The FP32 path must flag every one of them for the
FP64 recheck, and the counts of the FP32 + recheck path, the all-FP64 path,
the batched launch (boxes) and the oracle must be identical."""
import numpy as np
import pytest

import edge_pairs as ep

pytestmark = pytest.mark.gpu

CFGS = ep.configs()


@pytest.mark.parametrize("cfg", CFGS, ids=[c[0] for c in CFGS])
def test_near_edge_pairs(cfg):
    import fcfc_gb300 as fg
    name, survey, bt, kw, L, reach, nmu = cfg
    x, B, ob, bins = ep.build(cfg)
    want = ob.count(x)
    assert want.sum() > 0
    args = dict(geometry="survey" if survey else "box", bintype=bt, device=0)
    if "sedges" in kw:
        args["sedges"] = kw["sedges"]
    else:
        args.update(smin=kw["smin"], ds=kw["ds"],
                    smax=kw["smin"] + kw["ds"] * kw["ns"])
    if bt == 1:
        args["nmu"] = kw["nmu"]
    if bt == 2:
        args.update(pmin=kw["pmin"], dpi=kw["dpi"],
                    pmax=kw["pmin"] + kw["dpi"] * kw["np_"])
    if not survey:
        args["box"] = L
    pc = fg.PairCounter(**args)
    pc.load(0, x)
    got32 = pc.count_pairs(0, precision=fg.PREC_FP32_RECHECK)
    st = pc.stats()
    assert st["precision_used"] == fg.PREC_FP32_RECHECK
    # every constructed pair (and nothing else: they are isolated) is
    # ambiguous in FP32 and goes to the FP64 recheck
    assert st["rechecked"] == len(B.a), (st["rechecked"], len(B.a))
    np.testing.assert_array_equal(got32, want)
    np.testing.assert_array_equal(pc.count_pairs(0, precision=fg.PREC_FP64), want)
    if not survey:
        cnt, status, _ = pc.count_batch([x], [L])
        assert status == [0]
        np.testing.assert_array_equal(cnt[0], want)
