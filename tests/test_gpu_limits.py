"""Configurations at FCFC's limits and malformed inputs.

* ns up to FCFC_MAX_NSBIN (10000) and nmu up to FCFC_MAX_NMU (255): the
  histogram then no longer fits in shared memory (global accumulators) and,
  beyond 4094 s bins, the FP32 edge tables do not exist (FP64 path) -- the
  counts must still equal the oracle's.
* Non-finite coordinates or weights are rejected with FCFCG_ERR_DATA."""
import numpy as np
import pytest

from oracle import fcfc_oracle as fo

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("ns,nmu,ds", [(4000, 255, 0.005), (10000, 2, 0.002),
                                       (300, 255, 0.1)])
def test_large_bin_counts(ns, nmu, ds):
    import fcfc_gb300 as fg
    from fcfc_gb300 import synth
    L = 100.0
    x = synth.neyman_scott(30, L, 40, 2.0, seed=5)
    w = synth.lognormal_weights(len(x), 0.3, seed=6)
    smax = ns * ds
    pc = fg.PairCounter("box", fg.BIN_SMU, box=L, smin=0, smax=smax, ds=ds,
                        nmu=nmu)
    assert pc.ns == ns and pc.ntot == ns * nmu
    ob = fo.Bins(False, 1, ns=ns, smin=0, ds=ds, nmu=nmu, box=L)
    pc.load(0, x, w)
    for prec in (0, 1):
        np.testing.assert_array_equal(pc.count_pairs(0, precision=prec),
                                      ob.count(x, mode=1))
        np.testing.assert_allclose(pc.count_pairs(0, weighted=True, precision=prec),
                                   ob.count(x, wa=w, mode=1), rtol=1e-10,
                                   atol=1e-300)


def test_non_finite_inputs_rejected():
    import fcfc_gb300 as fg
    pc = fg.PairCounter("survey", fg.BIN_ISO, smin=0, smax=10, ds=1)
    x = np.random.default_rng(1).random((100, 3)) * 50
    for bad in (np.nan, np.inf, -np.inf):
        y = x.copy()
        y[17, 1] = bad
        with pytest.raises(fg.FCFCGError) as e:
            pc.load(0, y)
        assert e.value.code == fg.capi.ERR_DATA
        w = np.ones(len(x))
        w[3] = bad
        with pytest.raises(fg.FCFCGError) as e:
            pc.load(0, x, w)
        assert e.value.code == fg.capi.ERR_DATA
    pc.load(0, x)
    assert pc.count_pairs(0).sum() > 0


def test_recheck_queue_overflow():
    """Ambiguous pairs that find the FP64 recheck queue full are binned in
    the counting kernel itself (plain, weighted, batched and adjoint
    kernels): the results must not change with the queue's capacity."""
    import fcfc_gb300 as fg
    from fcfc_gb300 import synth
    kws = dict(ra=(150.0, 158.0), dec=(10.0, 17.0), zmu=0.5, zsig=0.04,
               zr=(0.46, 0.54))
    d = synth.radecz_to_xyz(synth.survey_radecz(3000, seed=81, **kws))
    r = synth.radecz_to_xyz(synth.survey_radecz(4000, seed=82, **kws))
    wd = synth.lognormal_weights(len(d), 0.3, seed=83)
    pc = fg.PairCounter("survey", fg.BIN_SMU, smin=0, smax=40, ds=0.5, nmu=60)
    ob = fo.Bins(True, 1, ns=80, smin=0, ds=0.5, nmu=60)
    pc.load(0, d, wd)
    pc.load(1, r)
    want = ob.count(d, r, mode=1)
    want_w = ob.count(d, r, wa=wd, mode=1)
    g = np.random.default_rng(84).normal(size=pc.ntot)
    pc.set_queue_capacity(1 << 30)          # clamped to the allocation
    ref_dw, ref_dr = pc.adjoint(0, 1, g)
    for cap in (0, 5):
        pc.set_queue_capacity(cap)
        np.testing.assert_array_equal(pc.count_pairs(0, 1), want)
        st = pc.stats()
        assert st["precision_used"] == fg.PREC_FP32_RECHECK
        assert st["rechecked"] > cap and st["recheck_inline"] == st["rechecked"] - cap
        np.testing.assert_allclose(pc.count_pairs(0, 1, weighted=True), want_w,
                                   rtol=1e-10, atol=1e-300)
        dw, dr = pc.adjoint(0, 1, g)
        np.testing.assert_allclose(dw, ref_dw, rtol=1e-11, atol=1e-11 * np.abs(ref_dw).max())
        np.testing.assert_allclose(dr, ref_dr, rtol=1e-11, atol=1e-11 * np.abs(ref_dr).max())
    # batched boxes share the queue
    bx = fg.PairCounter("box", fg.BIN_SMU, box=300.0, smin=0, smax=40, ds=0.5,
                        nmu=60)
    cats = [synth.neyman_scott(30, 300.0, 40, 3.0, seed=85 + k) for k in range(3)]
    bx.set_queue_capacity(3)
    cnt, status, _ = bx.count_batch(cats, [300.0] * 3)
    assert not any(status)
    for k in range(3):
        obk = fo.Bins(False, 1, ns=80, smin=0, ds=0.5, nmu=60, box=300.0)
        np.testing.assert_array_equal(cnt[k], obk.count(cats[k], mode=1))


@pytest.mark.parametrize("weighted", [False, True], ids=["unwt", "wt"])
def test_warp_queue_sizes(weighted):
    """The FP32 kernel's per-warp candidate queue (256, 512, 1024 entries or
    automatic) changes when candidates are binned, never the counts; dense
    clusters fill a small queue several times per neighbour block."""
    import fcfc_gb300 as fg
    from fcfc_gb300 import synth
    x = synth.neyman_scott(40, 200.0, 300, 1.5, seed=91)
    w = synth.lognormal_weights(len(x), 0.3, seed=92) if weighted else None
    pc = fg.PairCounter("box", fg.BIN_SMU, box=200.0, smin=0, smax=30, ds=1,
                        nmu=30)
    pc.load(0, x, w)
    ob = fo.Bins(False, 1, ns=30, smin=0, ds=1, nmu=30, box=200.0)
    want = ob.count(x, wa=w, weighted=weighted)
    seen = set()
    for q in (256, 512, 1024, 0):
        pc.set_warp_queue(q)
        got = pc.count_pairs(0, weighted=weighted)
        st = pc.stats()
        assert st["precision_used"] == fg.PREC_FP32_RECHECK
        if q:
            assert st["warp_queue"] == q
        seen.add(st["warp_queue"])
        if weighted:
            np.testing.assert_allclose(got, want, rtol=1e-10, atol=1e-300)
        else:
            np.testing.assert_array_equal(got, want)
    with pytest.raises(fg.FCFCGError):
        pc.set_warp_queue(300)
    # the autotuner times the queue sizes and keeps one
    pc.set_warp_queue(0)
    pc.autotune(0, weighted=weighted)
    pc.count_pairs(0, weighted=weighted)
    assert pc.stats()["warp_queue"] in (256, 512, 1024)


def test_shared_histogram_handover():
    """Unweighted FP32 counts: a CTA's 32-bit shared bins take their adds
    unchecked and are handed to the global counters before the pairs added
    since the last hand-over could pass the threshold
    (fcfcg_set_hist_handover, default 2^32 - 1); a chunk that alone could
    pass it counts in global memory.  Small thresholds force both paths --
    every chunk global (1), a mix (5000), frequent hand-overs (10^6) --
    for one catalogue and for a batch: the counts never change."""
    import fcfc_gb300 as fg
    from fcfc_gb300 import synth
    x = synth.neyman_scott(40, 200.0, 300, 1.5, seed=93)
    pc = fg.PairCounter("box", fg.BIN_SMU, box=200.0, smin=0, smax=30, ds=1,
                        nmu=30)
    pc.load(0, x)
    want = fo.Bins(False, 1, ns=30, smin=0, ds=1, nmu=30,
                   box=200.0).count(x, mode=1)
    np.testing.assert_array_equal(pc.count_pairs(0), want)
    cats = [synth.neyman_scott(30, 200.0, 200, 2.0, seed=94 + k)
            for k in range(3)]
    ref, status, _ = pc.count_batch(cats, [200.0] * 3)
    assert list(status) == [0, 0, 0]
    for limit in (1, 5000, 10 ** 6, 0):
        pc.set_hist_handover(limit)
        np.testing.assert_array_equal(pc.count_pairs(0), want)
        assert pc.stats()["precision_used"] == fg.PREC_FP32_RECHECK
        got, status, _ = pc.count_batch(cats, [200.0] * 3)
        for g, r in zip(got, ref):
            np.testing.assert_array_equal(g, r)
    with pytest.raises(fg.FCFCGError):
        pc.set_hist_handover(2 ** 32)
