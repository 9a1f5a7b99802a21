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
