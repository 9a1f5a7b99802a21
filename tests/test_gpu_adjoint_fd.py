"""Weight gradients of a Landy-Szalay loss at survey scale against central
finite differences.

Data 5e5 objects with lognormal(0, 0.3) weights and randoms 5e6 (unit
weights) from the survey generator; L = sum_b g_b xi_LS(b) over (s, mu)
40 x 100 bins, s < 200 Mpc/h, g ~ N(0, 1);
xi = (DD_n - 2 DR_n + RR_n) / RR_n with DD_n = 2 DD / (W (W - 1)),
DR_n = DR / (W Wr), RR_n = 2 RR / (Wr (Wr - 1)) (FCFC's normalisations,
src/fcfc/2pt/eval_cf.c:125-149).

The gradient: fcfcg_adjoint of DD and of DR (through the C ABI) with the
chain rule, plus the normalisations' dependence on W.  The check, for 64
random data weights: the central difference (L(w + h e_i) - L(w - h e_i)) /
2h, h = 1e-6, taken exactly.  A step in w_i changes DD_b by h a_b and DR_b
by h c_b, where a_b and c_b sum the partner weights of the pairs touching
object i in bin b -- found here with FCFC's FP64 per-pair formula
(src/fcfc/2pt/metric_common.c:142-260, restated in tests/edge_pairs.py) --
and W by h; the difference of the two losses is then formed bin by bin in
closed form, so no cancellation limits it.  Agreement to 1e-8 relative.
"""
import numpy as np
import pytest

import edge_pairs as ep

pytestmark = pytest.mark.gpu

ND, NR = 500000, 5000000
SMAX, DS, NMU = 200.0, 5.0, 100
H = 1e-6


def _touching(i, xd, wd, xr, fac, s2e):
    """(a, c): per bin, the partner weights of object i's pairs with the
    other data objects and with the randoms, binned by FCFC's formula."""
    ns = len(s2e) - 1
    out = []
    for x, w, skip in ((xd, wd, i), (xr, None, -1)):
        near = np.all(np.abs(x - xd[i]) < SMAX * 1.001, axis=1)
        if skip >= 0:
            near[skip] = False
        idx = np.nonzero(near)[0]
        a = np.repeat(xd[i][None, :], len(idx), axis=0)
        v = ep.survey_values(a, x[idx], fac, NMU)
        s2, q2 = v["s2"], v["q2"]
        si = np.searchsorted(s2e, s2, side="right") - 1
        ok = (si >= 0) & (si < ns)
        p = np.floor(q2)
        ok &= (s2 >= np.finfo(float).eps) & (p < NMU * NMU) | \
            (s2 < np.finfo(float).eps) & ok
        p = np.where(s2 < np.finfo(float).eps, 0, p)
        mi = np.floor(np.sqrt(np.clip(p, 0, None))).astype(np.int64)
        mi = np.where(mi * mi > p, mi - 1, mi)
        bins = (si + mi * ns)[ok]
        ww = np.ones(len(idx)) if w is None else w[idx]
        acc = np.zeros(ns * NMU)
        np.add.at(acc, bins, ww[ok])
        out.append(acc)
    return out


def test_landy_szalay_gradient_finite_differences():
    import fcfc_gb300 as fg
    from fcfc_gb300 import synth
    from oracle import fcfc_oracle as fo
    xd = synth.radecz_to_xyz(synth.survey_radecz(ND, seed=41))
    xr = synth.radecz_to_xyz(synth.survey_radecz(NR, seed=42))
    wd = synth.lognormal_weights(ND, 0.3, seed=43)
    pc = fg.PairCounter("survey", fg.BIN_SMU, smin=0, smax=SMAX, ds=DS,
                        nmu=NMU, device=0)
    pc.load(0, xd, wd)
    pc.load(1, xr)
    DD = pc.count_pairs(0, weighted=True)
    DR = pc.count_pairs(0, 1, weighted=True)
    RR = pc.count_pairs(1, weighted=True)
    g = np.random.default_rng(44).normal(size=pc.ntot)
    W, Wr = float(np.sum(wd)), float(NR)
    nDD, nDR, nRR = W * (W - 1), W * Wr, Wr * (Wr - 1)
    rrn = 2 * RR / nRR
    live = rrn > 0
    gr = np.where(live, g / np.where(live, rrn, 1), 0.0)
    # gradient: the adjoint kernels and the chain rule
    a1, _ = pc.adjoint(0, None, gr * 2 / nDD)
    a2, _ = pc.adjoint(0, 1, -gr * 2 / nDR)
    dW = (-(gr * 2 * DD).sum() * (2 * W - 1) / nDD ** 2 +
          (gr * 2 * DR).sum() * Wr / nDR ** 2)
    grad = a1 + a2 + dW

    ob = fo.Bins(True, 1, ns=int(SMAX / DS), smin=0, ds=DS, nmu=NMU)
    _, _, s2e, _ = ob.tables()
    fac = ob.rescale
    idx = np.random.default_rng(45).choice(ND, 64, replace=False)
    worst = 0.0
    for i in idx:
        a, c = _touching(i, xd, wd, xr, fac, s2e)
        # xi_b(w +- h e_i) with DD + -h a, DR +- h c, W +- h: the difference
        # of the two losses in closed form (the h in every term cancels)
        Wp, Wm = W + H, W - H
        nDDp, nDDm = Wp * (Wp - 1), Wm * (Wm - 1)
        nDRp, nDRm = Wp * Wr, Wm * Wr
        # 2 DD/nDD: [(DD + h a) nDDm - (DD - h a) nDDp] / (nDDp nDDm)
        #   = h [a (nDDp + nDDm) - DD 2 (2 W - 1)] / (nDDp nDDm)
        tdd = 2 * (a * (nDDp + nDDm) - DD * 2 * (2 * W - 1)) / (nDDp * nDDm)
        # DR/nDR: [(DR + h c) nDRm - (DR - h c) nDRp] / (nDRp nDRm)
        #   = h [c (nDRp + nDRm) - DR 2 Wr] / (nDRp nDRm)
        tdr = (c * (nDRp + nDRm) - DR * 2 * Wr) / (nDRp * nDRm)
        fd = float(np.sum(gr * (tdd - 2 * tdr))) / 2
        err = abs(fd - grad[i]) / max(abs(fd), 1e-300)
        worst = max(worst, err)
        assert err <= 1e-8, (int(i), fd, grad[i], err)
    print("worst relative difference %.3g" % worst)
