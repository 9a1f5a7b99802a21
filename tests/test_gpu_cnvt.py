"""RA/Dec/z -> comoving coordinates on the GPU (FCFC_2PT's COORD_CONVERT).

* Through the engine, the conversion golden cases reproduce FCFC's pair
  counts: the unweighted ones bit for bit, which pins the converted
  coordinates (a one-ulp change moves pairs across bin edges only rarely,
  but FCFC's and the engine's counts agree exactly on every case here).
* Against the oracle (the C library's cos/sin/pow in the reference's
  operation order) on 2e5 random objects: the same Gauss-Legendre order, and
  coordinates within 8 ulp relative.  CUDA's double sin/cos/pow carry at most
  2 ulp of error and the C library's under 1, so each factor of
  d cos(dec) cos(ra) differs by at most 3 ulp; every other operation is an
  identically rounded IEEE operation in the same order.
* Errors as FCFC raises them: negative redshift, a cosmology check_cosmo
  rejects, redshifts outside the Z_CMVDST_FILE table, a box context."""
import numpy as np
import pytest

from golden_cases import Case, case_names
from oracle import fcfc_oracle as fo

pytestmark = pytest.mark.gpu

ULP_BOUND = 8 * 2.0 ** -52


def _cosmo_kw(case):
    zt = case.ztable()
    if zt is not None:
        return dict(ztable=zt)
    m = case.meta
    kw = dict(omega_m=m.get("omega_m", 0.31))
    if "omega_l" in m:
        kw["omega_l"] = m["omega_l"]
    if "dew" in m:
        kw["dew"] = m["dew"]
    if "cmvdst_err" in m:
        kw["cmvdst_err"] = m["cmvdst_err"]
    return kw


@pytest.mark.parametrize("name", case_names(convert=True))
@pytest.mark.parametrize("precision", [0, 1])
def test_converted_counts_match_reference(name, precision):
    from test_gpu_parity import engine_for
    case = Case(name)
    pc = engine_for(case)
    ck = _cosmo_kw(case)
    slots = {}
    for i, lab in enumerate(case.meta["labels"]):
        a = case.cats[lab]
        pc.load_radecz(i, a[:, :3], a[:, 3] if a.shape[1] > 3 else None, **ck)
        slots[lab] = i
    for pair in case.meta["pairs"]:
        ref = case.pcfile(pair)
        sa, sb = slots[pair[0]], slots[pair[1]]
        if sa == sb:
            got = pc.count_pairs(sa, weighted=ref.weighted, precision=precision) * 2
        else:
            got = pc.count_pairs(sa, sb, weighted=ref.weighted, precision=precision)
        if ref.weighted:
            np.testing.assert_allclose(got, ref.cnt, rtol=1e-10, atol=0)
        else:
            assert np.array_equal(got, ref.cnt), (pair, np.nonzero(got != ref.cnt))


def _device_convert(pc, rdz, **ck):
    import torch
    dev = torch.device("cuda", 0)
    cols = [torch.from_numpy(np.ascontiguousarray(rdz[:, k])).to(dev) for k in range(3)]
    out = [torch.empty_like(cols[0]) for _ in range(3)]
    order = pc.convert_device(len(rdz), *[c.data_ptr() for c in cols],
                              *[o.data_ptr() for o in out], **ck)
    torch.cuda.synchronize()
    return np.stack([o.cpu().numpy() for o in out], axis=1), order


def _random_radecz(n, seed, zr=(0.01, 3.0)):
    rng = np.random.default_rng(seed)
    return np.stack([rng.uniform(0, 360, n), rng.uniform(-90, 90, n),
                     rng.uniform(*zr, n)], axis=1)


@pytest.mark.parametrize("cosmo", [
    dict(omega_m=0.31),
    dict(omega_m=0.3, omega_l=0.65, dew=-0.9, cmvdst_err=1e-10),
    dict(omega_m=0.25, omega_l=0.8, dew=-1.2),
])
def test_integration_matches_oracle(cosmo):
    import fcfc_gb300 as fg
    pc = fg.PairCounter("survey", fg.BIN_ISO, smin=0, smax=10, ds=1, device=0)
    rdz = _random_radecz(200000, seed=31)
    got, order = _device_convert(pc, rdz, **cosmo)
    want, want_order = fo.convert_integr(rdz, cosmo["omega_m"],
                                         cosmo.get("omega_l"),
                                         cosmo.get("dew", -1.0),
                                         cosmo.get("cmvdst_err", 1e-8))
    assert order == want_order
    err = np.abs(got - want)
    assert np.all(err <= ULP_BOUND * np.abs(want) + 1e-300), err.max()
    # most results are bit-identical (the libraries agree on most inputs)
    assert np.mean(got == want) > 0.5


def test_spline_matches_oracle_and_rejects_outside():
    import fcfc_gb300 as fg
    from fcfc_gb300 import synth
    pc = fg.PairCounter("survey", fg.BIN_ISO, smin=0, smax=10, ds=1, device=0)
    zt = np.linspace(0.0, 2.0, 301)
    tab = np.c_[zt, synth.comoving_distance(zt, 0.3)]
    tab = tab[np.random.default_rng(5).permutation(len(tab))]
    rdz = _random_radecz(100000, seed=32, zr=(0.0, 1.999))
    got, order = _device_convert(pc, rdz, ztable=tab)
    want, bad = fo.convert_spline(rdz, tab[:, 0], tab[:, 1])
    assert order == 0 and bad == 0
    err = np.abs(got - want)
    assert np.all(err <= ULP_BOUND * np.abs(want) + 1e-300), err.max()
    # a redshift at the table's upper end is outside [z0, z_last)
    rdz[5, 2] = 2.0
    with pytest.raises(fg.FCFCGError) as e:
        _device_convert(pc, rdz, ztable=tab)
    assert e.value.code == fg.capi.ERR_CNVT
    with pytest.raises(fg.FCFCGError) as e:
        _device_convert(pc, rdz[:10], ztable=tab[:1])
    assert e.value.code == fg.capi.ERR_CNVT


def test_conversion_errors():
    import fcfc_gb300 as fg
    pc = fg.PairCounter("survey", fg.BIN_ISO, smin=0, smax=10, ds=1, device=0)
    rdz = _random_radecz(1000, seed=33)
    rdz[17, 2] = -0.01
    with pytest.raises(fg.FCFCGError) as e:
        pc.load_radecz(0, rdz)
    assert e.value.code == fg.capi.ERR_DATA
    rdz[17, 2] = 0.5
    for bad in (dict(omega_m=0.0), dict(omega_m=1.5), dict(omega_m=0.3, dew=-0.2),
                dict(omega_m=0.3, omega_l=-0.1), dict(omega_m=0.3, cmvdst_err=1e-20)):
        with pytest.raises(fg.FCFCGError) as e:
            pc.load_radecz(0, rdz, **bad)
        assert e.value.code == fg.capi.ERR_CFG, bad
    box = fg.PairCounter("box", fg.BIN_ISO, box=100, smin=0, smax=10, ds=1, device=0)
    with pytest.raises(fg.FCFCGError) as e:
        box.load_radecz(0, rdz)
    assert e.value.code == fg.capi.ERR_ARG
    # a good load after the failures
    pc.load_radecz(0, rdz)
    assert pc.catalog_info(0)[0] == 1000
