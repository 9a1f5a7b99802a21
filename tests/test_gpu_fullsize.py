"""Full-size workloads, checked through properties that hold at any size:
the FP32 + FP64-recheck path must give exactly the all-FP64 path's integer
counts (and weighted sums within 1e-10), on the clustered 2e6-object box of
the benchmark and on a 1e6-object survey converted from RA/Dec/z; the
counts of an auto count sum to the number of in-range pairs the kernel
reports."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_box_2e6_fp32_equals_fp64():
    import fcfc_gb300 as fg
    from fcfc_gb300 import synth
    x = synth.neyman_scott(20000, 2000.0, 100.0, 5.0, seed=1)
    w = synth.lognormal_weights(len(x), 0.3, seed=2)
    pc = fg.PairCounter("box", fg.BIN_SMU, box=2000.0, smin=0, smax=200, ds=5,
                        nmu=100, device=0)
    pc.load(0, x, w)
    c32 = pc.count_pairs(0)
    st = pc.stats()
    assert st["precision_used"] == fg.PREC_FP32_RECHECK
    assert int(c32.sum()) == st["in_range"]
    c64 = pc.count_pairs(0, precision=fg.PREC_FP64)
    np.testing.assert_array_equal(c32, c64)
    w32 = pc.count_pairs(0, weighted=True)
    w64 = pc.count_pairs(0, weighted=True, precision=fg.PREC_FP64)
    np.testing.assert_allclose(w32, w64, rtol=1e-10, atol=0)


def test_survey_1e6_fp32_equals_fp64():
    import fcfc_gb300 as fg
    from fcfc_gb300 import synth
    rdz = synth.survey_radecz(1000000, seed=11)
    wd = synth.fkp_weights(rdz)
    for bt, kw in ((fg.BIN_SMU, dict(smin=0, smax=200, ds=5, nmu=100)),
                   (fg.BIN_SPI, dict(sedges=np.geomspace(0.1, 100.0, 41),
                                     pmin=0, pmax=40, dpi=1))):
        pc = fg.PairCounter("survey", bt, device=0, **kw)
        pc.load_radecz(0, rdz, wd, omega_m=0.31)
        c32 = pc.count_pairs(0)
        assert pc.stats()["precision_used"] == fg.PREC_FP32_RECHECK
        c64 = pc.count_pairs(0, precision=fg.PREC_FP64)
        np.testing.assert_array_equal(c32, c64)
        w32 = pc.count_pairs(0, weighted=True)
        w64 = pc.count_pairs(0, weighted=True, precision=fg.PREC_FP64)
        np.testing.assert_allclose(w32, w64, rtol=1e-10, atol=0)
