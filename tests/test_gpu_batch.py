"""Batched periodic boxes (fcfcg_count_batch): many catalogues of different
sizes and boxes in one persistent FP32 launch.  Every catalogue's counts must
equal what the single-catalogue path gives for it (integer counts bit for
bit, weighted sums to 1e-10), and a few are checked against the oracle
directly; catalogues FCFC would reject (s_max not below half the box) or
that leave their box are reported per catalogue without stopping the
batch."""
import numpy as np
import pytest

from oracle import fcfc_oracle as fo

pytestmark = pytest.mark.gpu

WT_RTOL = 1e-10


def _mocks(nmock, seed, density=2.5e-4 * 8, nmin=600, nmax=6000):
    from fcfc_gb300 import synth
    rng = np.random.default_rng(seed)
    cats, boxes, wts = [], [], []
    for j in range(nmock):
        n = int(np.exp(rng.uniform(np.log(nmin), np.log(nmax))))
        L = round((n / density) ** (1 / 3), 3)
        npar = max(1, n // 20)
        x = synth.neyman_scott(npar, L, 20.0, 3.0, seed=seed * 1000 + j)
        cats.append(x)
        boxes.append(L)
        wts.append(synth.lognormal_weights(len(x), 0.3, seed=seed * 1000 + j + 500))
    return cats, boxes, wts


def _single(pc_args, x, w, L, weighted, precision):
    import fcfc_gb300 as fg
    kw = dict(pc_args)
    kw["box"] = L
    pc = fg.PairCounter("box", **kw)
    pc.load(0, x, w if weighted else None)
    return pc.count_pairs(0, weighted=weighted, precision=precision)


CONFIGS = [
    dict(bintype=1, smin=0, smax=30, ds=2.5, nmu=20),
    dict(bintype=0, smin=1, smax=28, ds=3),
    dict(bintype=2, sedges=np.geomspace(0.5, 25, 11), pmin=0, pmax=20, dpi=2),
]


@pytest.mark.parametrize("cfg", range(len(CONFIGS)))
@pytest.mark.parametrize("weighted", [False, True])
def test_batch_matches_single_catalogue_path(cfg, weighted):
    import fcfc_gb300 as fg
    args = dict(CONFIGS[cfg])
    cats, boxes, wts = _mocks(14, seed=40 + cfg)
    # one catalogue too small for the bins (s_max >= L/2), one empty, one
    # with a point outside its box
    cats.append(cats[0][:50] * (40.0 / boxes[0]))
    boxes.append(40.0)
    wts.append(wts[0][:50])
    cats.append(np.zeros((0, 3)))
    boxes.append(200.0)
    wts.append(np.zeros(0))
    bad = cats[1].copy()
    bad[7, 0] = boxes[1] * 1.01
    cats.append(bad)
    boxes.append(boxes[1])
    wts.append(wts[1])
    pc = fg.PairCounter("box", box=max(boxes), device=0, **args)
    for prec in (fg.PREC_FP32_RECHECK, fg.PREC_FP64):
        got, status, sumw = pc.count_batch(cats, boxes, wts, weighted=weighted,
                                           precision=prec)
        assert status[-3] == fg.capi.ERR_CFG
        assert status[-2] == 0 and not np.any(got[-2])
        assert status[-1] == fg.capi.ERR_DATA
        for j in range(len(cats) - 3):
            assert status[j] == 0, (j, status[j])
            want = _single(args, cats[j], wts[j], boxes[j], weighted,
                           fg.PREC_FP32_RECHECK)
            if weighted:
                np.testing.assert_allclose(got[j], want, rtol=WT_RTOL, atol=1e-300)
                assert sumw[j] == pytest.approx(float(np.sum(wts[j])), rel=1e-12)
            else:
                assert np.array_equal(got[j], want), (j, prec)
                assert sumw[j] == len(cats[j])
        if prec == fg.PREC_FP32_RECHECK:
            st = pc.stats()
            assert st["precision_used"] == fg.PREC_FP32_RECHECK
            assert st["in_range"] > 0


def test_batch_against_oracle_and_device_inputs():
    import torch
    import fcfc_gb300 as fg
    args = dict(CONFIGS[0])
    cats, boxes, wts = _mocks(6, seed=77, nmin=1000, nmax=4000)
    pc = fg.PairCounter("box", box=max(boxes), device=0, **args)
    dev = torch.device("cuda", 0)
    tens = []
    dcats, dw = [], []
    for x, w in zip(cats, wts):
        cols = [torch.from_numpy(np.ascontiguousarray(x[:, k])).to(dev) for k in range(3)]
        wt = torch.from_numpy(np.ascontiguousarray(w)).to(dev)
        tens += cols + [wt]
        dcats.append((cols[0].data_ptr(), cols[1].data_ptr(), cols[2].data_ptr(), len(x)))
        dw.append(wt.data_ptr())
    got_u, st_u, _ = pc.count_batch(dcats, boxes, dw, weighted=False, on_device=True)
    got_w, st_w, _ = pc.count_batch(dcats, boxes, dw, weighted=True, on_device=True)
    assert not any(st_u) and not any(st_w)
    for j in range(len(cats)):
        ob = fo.Bins(False, 1, ns=12, smin=0, ds=2.5, nmu=20, box=boxes[j])
        assert np.array_equal(got_u[j], ob.count(cats[j], mode=3))
        np.testing.assert_allclose(got_w[j], ob.count(cats[j], wa=wts[j], mode=3),
                                   rtol=WT_RTOL, atol=1e-300)


def test_batch_autotune_keeps_counts():
    import fcfc_gb300 as fg
    args = dict(CONFIGS[0])
    cats, boxes, wts = _mocks(8, seed=91, nmin=2000, nmax=8000)
    pc = fg.PairCounter("box", box=max(boxes), device=0, **args)
    ref, _, _ = pc.count_batch(cats, boxes)
    k, ms = pc.autotune_batch(cats, boxes)
    assert 1 <= k <= 5 and ms > 0
    got, _, _ = pc.count_batch(cats, boxes)
    assert pc.stats()["cells_per_smax"] == k
    for a, b in zip(ref, got):
        assert np.array_equal(a, b)


def test_batch_accepts_column_arrays():
    """Host catalogues given as (x, y, z) columns count as the N x 3 arrays."""
    import fcfc_gb300 as fg
    cats, boxes, wts = _mocks(6, seed=77)
    pc = fg.PairCounter("box", **dict(CONFIGS[0], box=max(boxes)))
    a, st_a, _ = pc.count_batch(cats, boxes, wts, weighted=True)
    cols = [tuple(np.ascontiguousarray(c[:, k]) for k in range(3)) for c in cats]
    b, st_b, _ = pc.count_batch(cols, boxes, wts, weighted=True)
    assert list(st_a) == list(st_b)
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)
