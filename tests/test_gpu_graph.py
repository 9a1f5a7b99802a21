"""Count graphs (fcfcg_graph_create / fcfcg_graph_run): DD, DR and RR
captured once as a CUDA graph and replayed.  Every replay must give exactly
what fcfcg_count gives for each item (integer counts bit for bit; FP32-path
weighted sums bit for bit too, since both are the same exact fixed-point sums
of symmetric products; FP64-path weighted sums to 1e-12), also
after plain counts that re-sort the catalogues into other grids between
replays, after a catalogue is reloaded with other data (the graph captures
itself again), and for empty catalogues."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _survey(nd, nr, seed):
    from fcfc_gb300 import synth
    d = synth.radecz_to_xyz(synth.survey_radecz(nd, seed=seed))
    r = synth.radecz_to_xyz(synth.survey_radecz(nr, seed=seed + 1))
    wd = synth.lognormal_weights(nd, 0.3, seed=seed + 2)
    wr = synth.lognormal_weights(nr, 0.3, seed=seed + 3)
    return d, r, wd, wr


def _plain(pc, pairs, precision):
    out = []
    for a, b, wt in pairs:
        out.append(pc.count_pairs(a, b, weighted=wt, precision=precision))
    return out


def _same(got, want, fp64=False):
    """Integer counts bit for bit; FP32-path weighted sums bit for bit too
    (exact fixed-point sums of symmetric products); the FP64 path's weighted
    sums are FP64 atomics in no fixed order: 1e-12 relative."""
    assert len(got) == len(want)
    for g, w in zip(got, want):
        assert g.dtype == w.dtype
        if fp64 and g.dtype == np.float64:
            np.testing.assert_allclose(g, w, rtol=1e-12, atol=0)
        else:
            np.testing.assert_array_equal(g, w)


SURVEY_BINS = [
    dict(bintype=1, smin=0, smax=60, ds=5, nmu=20),
    dict(bintype=2, sedges=np.geomspace(0.5, 40, 13), pmin=0, pmax=30, dpi=3),
]


@pytest.mark.parametrize("cfg", range(len(SURVEY_BINS)))
@pytest.mark.parametrize("precision", [0, 1])
def test_survey_dd_dr_rr_graph_matches_plain_counts(cfg, precision):
    import fcfc_gb300 as fg
    d, r, wd, wr = _survey(6000, 30000, seed=70 + cfg)
    pc = fg.PairCounter("survey", **SURVEY_BINS[cfg])
    pc.load(0, d, wd)
    pc.load(1, r, wr)
    pairs = [(0, None, True), (0, 1, True), (1, None, True),
             (0, None, False), (0, 1, False), (1, None, False)]
    g = pc.count_graph(pairs, precision=precision)
    want = _plain(pc, pairs, precision)
    fp64 = precision == 1
    for _ in range(2):
        _same(g.run(), want, fp64)
    # a plain count in another grid (a cross count with the slots swapped)
    # between replays: the graph sorts what it needs itself
    pc.count_pairs(1, 0, weighted=False, precision=precision)
    _same(g.run(), want, fp64)
    _same(_plain(pc, pairs, precision), want, fp64)
    g.close()
    pc.close()


def test_box_graph_and_reload():
    import fcfc_gb300 as fg
    from fcfc_gb300 import synth
    L = 300.0
    pc = fg.PairCounter("box", 1, box=L, smin=0, smax=40, ds=2, nmu=25)
    x1 = synth.neyman_scott(400, L, 20.0, 4.0, seed=5)
    w1 = synth.lognormal_weights(len(x1), 0.3, seed=6)
    x2 = synth.uniform_box(9000, L, seed=7)
    pc.load(0, x1, w1)
    pc.load(1, x2)
    pairs = [(0, None, False), (0, 1, True), (1, None, False)]
    g = pc.count_graph(pairs)
    _same(g.run(), _plain(pc, pairs, 0))
    assert g.info()[0] == 1 and g.info()[1] > 0
    # the same catalogue loaded again plans the same: a replay, no capture
    pc.load(0, x1, w1)
    _same(g.run(), _plain(pc, pairs, 0))
    assert g.info()[0] == 1
    # other data of the same size: counted correctly (captured again only
    # when the plan differs)
    x3 = synth.uniform_box(len(x1), L, seed=8)
    pc.load(0, x3, w1[::-1].copy())
    _same(g.run(), _plain(pc, pairs, 0))
    # a larger catalogue (buffers reallocated): captured again
    x4 = synth.neyman_scott(900, L, 20.0, 4.0, seed=9)
    pc.load(0, x4, synth.lognormal_weights(len(x4), 0.3, seed=10))
    n0 = g.info()[0]
    got = g.run()
    assert g.info()[0] == n0 + 1
    _same(got, _plain(pc, pairs, 0))
    assert got[0].sum() > 0
    # an empty catalogue: zeros, and the other items still count
    pc.load(1, np.zeros((0, 3)))
    got = g.run()
    assert not got[1].any() and not got[2].any()
    _same(got[:1], _plain(pc, pairs[:1], 0))
    pc.close()           # closes the graph first
    assert g.h is None


def test_graph_arguments():
    import fcfc_gb300 as fg
    pc = fg.PairCounter("box", 0, box=100.0, smin=0, smax=20, ds=4)
    pc.load(0, np.random.default_rng(1).random((100, 3)) * 100)
    with pytest.raises(fg.FCFCGError):      # slot 3 not loaded
        pc.count_graph([(0, 3, False)])
    with pytest.raises(fg.FCFCGError):      # auto count of two slots
        from fcfc_gb300 import capi
        import ctypes as C
        items = (capi.CountItem * 1)()
        items[0].slot_a, items[0].slot_b, items[0].isauto = 0, 1, 1
        out = np.zeros(pc.ntot, np.int64)
        items[0].icnt = out.ctypes.data_as(C.POINTER(C.c_int64))
        h = C.c_void_p()
        pc._check(pc.lib.fcfcg_graph_create(pc.h, items, 1, 0, C.byref(h)))
    pc.close()
