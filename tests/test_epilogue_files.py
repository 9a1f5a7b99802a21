"""Post-processing and file formats against the upstream outputs, on the CPU:
starting from the counts in the golden pair-count files, the C library must
write byte-identical pair-count files (binary and ASCII) and byte-identical
xi / multipole / w_p files."""
import os

import numpy as np
import pytest

from golden_cases import Case, case_names

CASES = case_names()


def host_counter(case):
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
        args["box"] = case.meta["box"] * 3 if len(case.meta["box"]) == 1 \
            else case.meta["box"]
    if kw.get("with_mu_one"):
        args["with_mu_one"] = True
    return fg.PairCounter(**args)


@pytest.mark.parametrize("name", CASES)
def test_paircount_files_byte_identical(name, tmp_path):
    case = Case(name)
    pc = host_counter(case)
    for pair in case.meta["pairs"]:
        ref = case.pcfile(pair)
        auto = pair[0] == pair[1]
        ntr = [int(v) for v in ref.tracers] if not ref.weighted else [0, 0]
        wtr = list(ref.tracers) if ref.weighted else None
        if ref.weighted:
            # the file keeps only the weighted numbers; counts of objects are
            # not written for weighted pairs
            ntr = [len(case.cats[pair[0]]), len(case.cats[pair[1]])]
        out = str(tmp_path / (pair + ".bin"))
        pc.write_paircount(out, 0, auto, ref.weighted, ntr, wtr, ref.norm,
                           ref.ncnt, ref.cnt)
        want = open(os.path.join(case.dir, pair + ".bin"), "rb").read()
        got = open(out, "rb").read()
        assert got == want
        # and read back
        r = pc.read_paircount(out)
        assert r["auto"] == auto and r["weighted"] == ref.weighted
        np.testing.assert_array_equal(r["cnt"], ref.cnt)
        asc = os.path.join(case.dir, pair + ".txt")
        if os.path.exists(asc):
            out2 = str(tmp_path / (pair + ".txt"))
            pc.write_paircount(out2, 1, auto, ref.weighted, ntr, wtr, ref.norm,
                               ref.ncnt, ref.cnt)
            assert open(out2).read() == open(asc).read()


@pytest.mark.parametrize("name", CASES)
def test_norms(name):
    case = Case(name)
    pc = host_counter(case)
    for pair in case.meta["pairs"]:
        ref = case.pcfile(pair)
        auto = pair[0] == pair[1]
        if ref.weighted:
            n1 = ref.tracers[0]
            n2 = ref.tracers[-1]
        else:
            n1 = float(ref.tracers[0])
            n2 = float(ref.tracers[-1])
        cnt = ref.cnt // 2 if (auto and not ref.weighted) else (
            ref.cnt / 2 if auto else ref.cnt)
        c2, norm, ncnt = pc.normalise(cnt, auto, ref.weighted, n1, n2)
        assert norm == ref.norm
        np.testing.assert_array_equal(c2, ref.cnt)
        np.testing.assert_array_equal(ncnt, ref.ncnt)


@pytest.mark.parametrize("name", CASES)
def test_cf_multipoles_wp_byte_identical(name, tmp_path):
    import fcfc_gb300 as fg
    case = Case(name)
    pc = host_counter(case)
    pairs = case.meta["pairs"]
    nc = np.stack([case.pcfile(p).ncnt for p in pairs])
    rr = pc.analytic_rr() if case.box else None
    lib = fg.load_library()
    for e in case.meta["cf"]:
        xi = np.zeros(pc.ntot)
        rc = lib.fcfcg_cf_eval(e.encode(), len(pairs), "".join(pairs).encode(),
                               fg.capi.ptr(np.ascontiguousarray(nc)),
                               fg.capi.ptr(rr) if rr is not None else None,
                               pc.ntot, fg.capi.ptr(xi))
        assert rc == 0
        out = str(tmp_path / "xi.txt")
        pc.write_cf(out, xi)
        assert open(out).read() == open(os.path.join(case.dir, "xi.txt")).read()
        if case.meta.get("poles") and case.meta["bintype"] == 1:
            mp = pc.multipoles(xi, case.meta["poles"])
            out = str(tmp_path / "mp.txt")
            pc.write_multipoles(out, case.meta["poles"], mp)
            assert open(out).read() == open(os.path.join(case.dir, "mp.txt")).read()
        if case.meta.get("wp") and case.meta["bintype"] == 2:
            wp = pc.wp(xi)
            out = str(tmp_path / "wp.txt")
            pc.write_wp(out, wp)
            assert open(out).read() == open(os.path.join(case.dir, "wp.txt")).read()


def test_estimator_syntax():
    import fcfc_gb300 as fg
    lib = fg.load_library()
    nc = np.ascontiguousarray([[1.0, 2.0], [4.0, 8.0]])
    out = np.zeros(2)

    def ev(s):
        rc = lib.fcfcg_cf_eval(s.encode(), 2, b"DDRR", fg.capi.ptr(nc), None,
                               2, fg.capi.ptr(out))
        return rc, out.copy()

    assert ev("DD/RR - 1")[1].tolist() == [1 / 4 - 1, 2 / 8 - 1]
    assert ev("(DD - 2*DD + RR)/RR")[1].tolist() == [(1 - 2 + 4) / 4, (2 - 4 + 8) / 8]
    assert ev("-DD**2")[1].tolist() == [1.0, 4.0]
    assert ev("sqrt(RR) + abs(-DD)")[1].tolist() == [3.0, 2 ** 1.5 + 2]
    assert ev("DD / @@")[0] != 0          # no analytic RR given
    assert ev("DX")[0] != 0               # unknown label
    assert ev("DD +")[0] != 0


@pytest.mark.parametrize("name", case_names(single_prec=True))
def test_reads_single_precision_files(name):
    """A pair-count file written by a SINGLE_PREC build of FCFC (float box
    and bin edges) reads back, as FCFC's double build reads it
    (src/fcfc/2pt_box/read_res.c:256-420)."""
    case = Case(name)
    pc = host_counter(case)
    for pair in case.meta["pairs"]:
        fn = os.path.join(case.dir, pair + ".bin")
        r = pc.read_paircount(fn)
        ref = case.pcfile(pair)
        assert r["auto"] == (pair[0] == pair[1])
        np.testing.assert_array_equal(r["cnt"], ref.cnt)
        np.testing.assert_array_equal(r["ncnt"], ref.ncnt)
        assert r["norm"] == ref.norm
