"""Adjoint of the weighted counts (fcfcg_adjoint) and its torch.autograd
wrapper.

* Per object against the oracle's FP64 brute-force gradient
  dL/dw_i = sum_j w_j g[bin(i, j)]: the bins are the same pairs' bins, so
  the only difference is FP64 summation order (1e-11 relative).
* Against central finite differences of the counts themselves, step 1e-6:
  C is bilinear in the weights (no w_i^2 term), so the central difference
  is exact up to the quantisation of the products (2^-51 of the largest
  weight product), and must agree to 1e-8 relative.
* The Landy-Szalay loss L = sum_b g_b xi_LS(b) through autograd against the
  chain rule on the oracle's per-object gradients (1e-10), and against
  central differences of L (step 1e-6; the FP64 rounding of L itself,
  ~1e-16 |L| / 2e-6, bounds that agreement to 1e-6 relative)."""
import numpy as np
import pytest

from oracle import fcfc_oracle as fo

pytestmark = pytest.mark.gpu


def _survey(nd, nr, seed):
    from fcfc_gb300 import synth
    kw = dict(ra=(150.0, 160.0), dec=(10.0, 20.0), zmu=0.5, zsig=0.05,
              zr=(0.45, 0.55))
    d = synth.radecz_to_xyz(synth.survey_radecz(nd, seed=seed, **kw))
    r = synth.radecz_to_xyz(synth.survey_radecz(nr, seed=seed + 1, **kw))
    wd = synth.lognormal_weights(nd, 0.3, seed=seed + 2)
    return d, r, wd


@pytest.mark.parametrize("case", ["box_smu_auto", "survey_smu_cross",
                                  "survey_spi_auto"])
def test_adjoint_matches_oracle(case):
    import fcfc_gb300 as fg
    from fcfc_gb300 import synth
    rng = np.random.default_rng(5)
    if case == "box_smu_auto":
        L = 300.0
        x = synth.neyman_scott(60, L, 40, 4.0, seed=3)
        w = synth.lognormal_weights(len(x), 0.3, seed=4)
        pc = fg.PairCounter("box", fg.BIN_SMU, box=L, smin=0, smax=40, ds=4,
                            nmu=10, device=0)
        ob = fo.Bins(False, 1, ns=10, smin=0, ds=4, nmu=10, box=L)
        pc.load(0, x, w)
        g = rng.normal(size=pc.ntot)
        got, _ = pc.adjoint(0, None, g)
        want, _ = ob.adjoint(x, g, wa=w)
    elif case == "survey_smu_cross":
        d, r, wd = _survey(2000, 3000, 11)
        wr = synth.lognormal_weights(len(r), 0.2, seed=14)
        pc = fg.PairCounter("survey", fg.BIN_SMU, smin=0, smax=30, ds=3,
                            nmu=10, device=0)
        ob = fo.Bins(True, 1, ns=10, smin=0, ds=3, nmu=10)
        pc.load(0, d, wd)
        pc.load(1, r, wr)
        g = rng.normal(size=pc.ntot)
        got, got_b = pc.adjoint(0, 1, g)
        want, want_b = ob.adjoint(d, g, b=r, wa=wd, wb=wr)
        np.testing.assert_allclose(got_b, want_b, rtol=1e-11, atol=1e-12)
    else:
        d, r, wd = _survey(3000, 10, 21)
        edges = np.geomspace(0.5, 25, 9)
        pc = fg.PairCounter("survey", fg.BIN_SPI, sedges=edges, pmin=0,
                            pmax=20, dpi=2, device=0)
        ob = fo.Bins(True, 2, ns=8, sedges=edges, np_=10, pmin=0, dpi=2)
        pc.load(0, d, wd)
        g = rng.normal(size=pc.ntot)
        got, _ = pc.adjoint(0, None, g)
        want, _ = ob.adjoint(d, g, wa=wd)
    assert np.any(want != 0)
    np.testing.assert_allclose(got, want, rtol=1e-11, atol=1e-12)


def test_adjoint_matches_count_differences():
    """C is bilinear in the weights, so a central difference of sum_b g_b C_b
    is exact for any step: with a step of 1e-2 the adjoint must match to
    1e-10.  With the step of 1e-6 the difference is limited by the FP64
    rounding of the returned counts (|C_b| 2^-53 per bin, over 2e-6), so the
    agreement is 1e-8 relative or that rounding bound, whichever is larger."""
    import fcfc_gb300 as fg
    d, r, wd = _survey(2500, 10, 31)
    pc = fg.PairCounter("survey", fg.BIN_SMU, smin=0, smax=30, ds=3, nmu=10,
                        device=0)
    g = np.random.default_rng(6).normal(size=pc.ntot)
    pc.load(0, d, wd)
    grad, _ = pc.adjoint(0, None, g)
    idx = np.random.default_rng(7).choice(len(d), 64, replace=False)
    for h, rtol in ((1e-2, 1e-10), (1e-6, 1e-8)):
        for i in idx:
            w1 = wd.copy()
            w1[i] += h
            pc.load(0, d, w1)
            cp = pc.count_pairs(0, weighted=True)
            w1[i] -= 2 * h
            pc.load(0, d, w1)
            cm = pc.count_pairs(0, weighted=True)
            fd = float(np.dot(g, cp - cm)) / (2 * h)
            rounding = float(np.dot(np.abs(g), np.maximum(np.abs(cp), np.abs(cm)))
                             ) * 2.0 ** -52 / (2 * h)
            tol = max(rtol * max(abs(grad[i]), 1e-3), rounding)
            assert abs(fd - grad[i]) <= tol, (h, i, fd, grad[i], tol)


def test_autograd_landy_szalay():
    import torch
    import fcfc_gb300 as fg
    from fcfc_gb300.autograd import weighted_pair_counts, xi_ls
    d, r, wd_np = _survey(1500, 4000, 41)
    pc = fg.PairCounter("survey", fg.BIN_SMU, smin=0, smax=30, ds=3, nmu=10,
                        device=0)
    g = torch.from_numpy(np.random.default_rng(8).normal(size=pc.ntot))
    wr = torch.ones(len(r), dtype=torch.float64)

    def loss(w):
        dd = weighted_pair_counts(pc, d, w)
        dr = weighted_pair_counts(pc, d, w, r, wr)
        rr = weighted_pair_counts(pc, r, wr)
        return (g * xi_ls(dd, dr, rr, w.sum(), wr.sum())).sum()

    wd = torch.from_numpy(wd_np.copy()).requires_grad_(True)
    Lv = loss(wd)
    Lv.backward()
    grad = wd.grad.numpy()

    # chain rule on the oracle's per-object gradients and counts
    ob = fo.Bins(True, 1, ns=10, smin=0, ds=3, nmu=10)
    DD = ob.count(d, wa=wd_np, weighted=True)
    DR = ob.count(d, r, wa=wd_np, wb=np.ones(len(r)), weighted=True)
    RR = ob.count(r, wa=np.ones(len(r)), weighted=True)
    W, Wr = wd_np.sum(), float(len(r))
    nDD, nDR, nRR = W * (W - 1), W * Wr, Wr * (Wr - 1)
    gn = g.numpy()
    rrn = 2 * RR / nRR
    # xi = (2DD/nDD - 2 DR/nDR + rrn) / rrn
    gdd = gn * 2 / nDD / rrn                      # dL/dDD per bin
    gdr = -gn * 2 / nDR / rrn                     # dL/dDR per bin
    dW = (-(gn * 2 * DD / rrn).sum() * (2 * W - 1) / nDD ** 2 +
          (gn * 2 * DR / rrn).sum() * Wr / nDR ** 2)
    a1, _ = ob.adjoint(d, gdd, wa=wd_np)
    a2, _ = ob.adjoint(d, gdr, b=r, wa=wd_np, wb=np.ones(len(r)))
    want = a1 + a2 + dW
    np.testing.assert_allclose(grad, want, rtol=1e-10, atol=1e-12 * np.abs(want).max())

    # central differences of L itself on 64 weights
    h = 1e-6
    idx = np.random.default_rng(9).choice(len(d), 64, replace=False)
    with torch.no_grad():
        for i in idx:
            w1 = torch.from_numpy(wd_np.copy())
            w1[i] += h
            lp = float(loss(w1))
            w1[i] -= 2 * h
            lm = float(loss(w1))
            fd = (lp - lm) / (2 * h)
            tol = 1e-6 * abs(grad[i]) + 4e-16 * abs(float(Lv)) / h
            assert abs(fd - grad[i]) <= tol, (i, fd, grad[i])
