"""CPU-side checks of libfcfcg.so: it loads, exports every entry point the
public header declares, and its host-only bin set-up matches the oracle (and
through it the upstream FCFC) table for table."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from golden_cases import Case, case_names
from oracle import fcfc_oracle as fo

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "fcfcg.h")


def header_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(fcfcg_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    import fcfc_gb300 as fg
    lib = fg.load_library()
    names = header_functions()
    assert len(names) > 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    # and the ctypes prototypes cover exactly the header
    assert set(names) == set(fg.capi.PROTOTYPES), (
        set(names) ^ set(fg.capi.PROTOTYPES))


def test_no_gpu_context_fails_loudly():
    import torch
    import fcfc_gb300 as fg
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(fg.FCFCGError) as e:
        fg.PairCounter("box", 1, box=100.0, smin=0, smax=20, ds=5, nmu=10)
    assert e.value.code == fg.capi.ERR_CUDA


def _engine_host(case):
    import fcfc_gb300 as fg
    kw = case.bins_kwargs()
    bt = kw.pop("bintype")
    ns = kw.pop("ns")
    args = dict(geometry="box" if case.box else "survey", bintype=bt,
                host_only=True)
    if "sedges" in kw:
        args["sedges"] = kw["sedges"]
    else:
        args.update(smin=kw["smin"], ds=kw["ds"], smax=kw["smin"] + kw["ds"] * ns)
    if bt == 1:
        args["nmu"] = kw["nmu"]
    if bt == 2:
        args.update(pmin=kw["pmin"], dpi=kw["dpi"],
                    pmax=kw["pmin"] + kw["dpi"] * kw["np_"])
    if case.box:
        args["box"] = kw["box"]
    return fg.PairCounter(**args)


def _compare_tables(pc, ob):
    st, pt, s2, pb = pc.tables()
    ost, opt, os2, opb = ob.tables()
    assert pc.rescale == ob.rescale
    np.testing.assert_array_equal(st, ost)
    np.testing.assert_array_equal(s2, os2)
    if pb is not None:
        np.testing.assert_array_equal(pt, opt)
        np.testing.assert_array_equal(pb, opb)


@pytest.mark.parametrize("name", case_names())
def test_bins_match_oracle_on_golden_cases(name):
    case = Case(name)
    pc = _engine_host(case)
    ob = fo.Bins(survey=not case.box, **case.bins_kwargs())
    _compare_tables(pc, ob)
    ref = case.pcfile(case.meta["pairs"][0])
    np.testing.assert_array_equal(pc.sbin, ref.sbin)
    if case.box:
        np.testing.assert_array_equal(pc.info.box_rescaled[:], ref.box)


def _random_configs(n, seed=0):
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n):
        survey = bool(rng.integers(2))
        bt = int(rng.integers(3))
        kind = rng.integers(3)
        if kind == 0:      # linear, decimal steps
            smin = float(rng.choice([0, 0, 0.5, 1, 2.5, 3]))
            ds = float(rng.choice([0.5, 1, 2, 2.5, 4, 5, 0.25, 0.1, 1.5]))
            ns = int(rng.integers(3, 60))
            s = dict(smin=smin, ds=ds, ns=ns)
        elif kind == 1:    # linear, awkward step -> hybrid
            s = dict(smin=0.0, ds=float(rng.uniform(0.05, 3.0)),
                     ns=int(rng.integers(3, 40)))
        else:              # file bins (log)
            lo = float(rng.uniform(0.05, 2))
            e = np.geomspace(lo, lo * rng.uniform(10, 200), int(rng.integers(4, 40)))
            s = dict(sedges=e, ns=len(e) - 1)
        p = {}
        if bt == 2:
            pk = rng.integers(2)
            if pk == 0:
                p = dict(pmin=float(rng.choice([0, 0, 1, 2])),
                         dpi=float(rng.choice([0.5, 1, 2, 2.5])),
                         np_=int(rng.integers(2, 40)))
            else:
                e = np.sort(rng.uniform(0, 60, int(rng.integers(3, 20))))
                e[0] = 0.0
                p = dict(pedges=np.unique(e), np_=len(np.unique(e)) - 1)
        smax_ = s["sedges"][-1] if "sedges" in s else s["smin"] + s["ds"] * s["ns"]
        pmax_ = 0
        if bt == 2:
            pmax_ = p["pedges"][-1] if "pedges" in p else p["pmin"] + p["dpi"] * p["np_"]
        box = 2.2 * max(smax_, pmax_) + 1
        out.append((survey, bt, s, p, int(rng.integers(2, 120)), box))
    return out


@pytest.mark.parametrize("cfg", _random_configs(120), ids=lambda c: "cfg")
def test_bins_match_oracle_random(cfg):
    import fcfc_gb300 as fg
    survey, bt, s, p, nmu, box = cfg
    args = dict(geometry="survey" if survey else "box", bintype=bt,
                host_only=True, nmu=nmu, box=None if survey else box)
    okw = dict(ns=s["ns"], nmu=nmu, box=None if survey else box)
    if "sedges" in s:
        args["sedges"] = s["sedges"]
        okw["sedges"] = s["sedges"]
    else:
        args.update(smin=s["smin"], ds=s["ds"], smax=s["smin"] + s["ds"] * s["ns"])
        okw.update(smin=s["smin"], ds=s["ds"])
    if bt == 2:
        okw["np_"] = p["np_"]
        if "pedges" in p:
            args["pedges"] = p["pedges"]
            okw["pedges"] = p["pedges"]
        else:
            args.update(pmin=p["pmin"], dpi=p["dpi"],
                        pmax=p["pmin"] + p["dpi"] * p["np_"])
            okw.update(pmin=p["pmin"], dpi=p["dpi"])
    try:
        ob = fo.Bins(survey, bt, **okw)
    except ValueError:
        with pytest.raises(fg.FCFCGError):
            fg.PairCounter(**args)
        return
    pc = fg.PairCounter(**args)
    _compare_tables(pc, ob)


def test_linear_nbin_matches_conf_verify():
    import fcfc_gb300 as fg
    lib = fg.load_library()
    # conf_verify counts steps while v < max - 1e-10
    for mn, mx, st in [(0, 200, 5), (0, 40, 1), (0.1, 0.9, 0.2), (5, 45, 4),
                       (0, 12.3457 * 2, 0.123457 * 2), (0, 1, 0.3)]:
        v, n = mn, 0
        while v < mx - 1e-10:
            v += st
            n += 1
        assert lib.fcfcg_linear_nbin(mn, mx, st) == n


def test_config_errors():
    import fcfc_gb300 as fg
    bad = [
        dict(geometry="box", bintype=1, box=30.0, smin=0, smax=20, ds=2, nmu=10),
        dict(geometry="box", bintype=1, box=100.0, smin=0, smax=20, ds=2, nmu=1),
        dict(geometry="box", bintype=1, box=100.0, smin=0, smax=20, ds=2, nmu=300),
        dict(geometry="box", bintype=7, box=100.0, smin=0, smax=20, ds=2),
        dict(geometry="box", bintype=2, box=100.0, smin=0, smax=20, ds=2,
             pmin=0, pmax=60, dpi=1),
    ]
    for kw in bad:
        with pytest.raises(fg.FCFCGError) as e:
            fg.PairCounter(host_only=True, **kw)
        assert e.value.code == fg.capi.ERR_CFG


def test_fp32_table_kind():
    """Log s bins in a box get a bit-pattern FP32 window table (a fixed
    number of cells per octave, at most one edge per cell); linear bins and
    surveys keep the uniform table."""
    import fcfc_gb300 as fg
    log = np.geomspace(0.1, 50, 31)
    cases = [
        (dict(geometry="box", bintype=0, box=200.0, sedges=log), True),
        (dict(geometry="box", bintype=1, box=200.0, sedges=log, nmu=10), True),
        (dict(geometry="box", bintype=2, box=200.0, sedges=log, pmin=0,
              pmax=20, dpi=1), True),
        (dict(geometry="survey", bintype=2, sedges=log, pmin=0, pmax=20,
              dpi=1), False),
        (dict(geometry="box", bintype=1, box=200.0, smin=0, smax=50, ds=5,
              nmu=10), False),
    ]
    for kw, want in cases:
        pc = fg.PairCounter(host_only=True, **kw)
        cpo = pc.info.ftab_cells_per_octave
        assert (cpo > 0) == want, (kw, cpo)
        if want:
            # edges a factor 1.23 apart: 16 cells per octave resolve them
            assert 16 <= cpo <= 1 << 15
        pc.close()


def test_grid_sub_bits_bounds():
    """The grid sort's sub-cell choice (prep.cu:fcfcg_grid_sub_bits): 4x4x4
    sub-cells where cells hold many objects, 2x2x2 or none as they thin out,
    the fine counters at most ~4 per object (or 2^22), and the fine index
    (cell << bits | sub-cell) always within 32 bits."""
    import fcfc_gb300 as fg
    lib = fg.load_library()
    f = lib.fcfcg_grid_sub_bits
    f.restype = C.c_int
    f.argtypes = [C.c_size_t, C.c_size_t]
    assert f(64000, 2000000) == 6            # ~31 objects per cell
    assert f(1800000, 55000000) == 6
    assert f(2000000, 4000000) == 3          # ~2 objects per cell
    assert f(2000000, 2000000) == 0          # ~1: no sub-cells
    assert f(40000000, 2000000) == 0
    assert f(1000, 0) == 6                   # small grids: 2^22 counters
    for nc in (1, 10 ** 3, 10 ** 5, 6 * 10 ** 7, 10 ** 8, 2 ** 31):
        for n in (0, 10 ** 4, 10 ** 6, 10 ** 8, 4 * 10 ** 9):
            sb = f(nc, n)
            assert sb in (0, 3, 6)
            if sb:
                assert (nc << sb) < 0xFFFFFFF0
                assert (nc << sb) <= max(4 * n, 1 << 22)
