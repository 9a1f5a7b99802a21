#!/usr/bin/env python3
"""Generate the golden fixtures in tests/golden/ by running the upstream FCFC.

The upstream executables are compiled from their own sources by
``make -f oracle/Makefile.ref`` (scalar FP64 + OpenMP, i.e. the build an
aarch64 host gets) into oracle/_ref/.  This script can only run where the
FCFC sources were available to build them; the fixtures it writes are
committed and are all the tests need.

Each case directory holds
  meta.json        the configuration (FCFC keys) and catalogue list
  <label>.npy      the catalogue, float64, columns x y z [w]
  <PAIR>.bin       FCFC binary pair-count file (OUTPUT_FORMAT = 0)
  <PAIR>.txt       FCFC ASCII pair-count file (OUTPUT_FORMAT = 1), some cases
  xi.txt / mp.txt / wp.txt   FCFC correlation-function outputs

Usage: python tests/golden/make_golden.py [case ...]
"""
from __future__ import annotations

import json
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from fcfc_gb300 import synth  # noqa: E402

REF = os.path.join(ROOT, "oracle", "_ref")


def box_cases():
    c = {}
    x = synth.uniform_box(3000, 300.0, seed=11)
    c["box_iso_auto"] = dict(
        box=[300.0], bintype=0, cats={"D": x}, pairs=["DD"],
        cf=["DD / @@ - 1"], sbin=dict(smin=0, smax=40, ds=2))
    c["box_smu_auto"] = dict(
        box=[300.0], bintype=1, cats={"D": x}, pairs=["DD"],
        cf=["DD / @@ - 1"], poles=[0, 2, 4], nmu=20,
        sbin=dict(smin=0, smax=50, ds=5), ascii=True)
    ns = synth.neyman_scott(40, 400.0, mean_children=60, sigma=5.0, seed=12,
                            float32=True)
    w = synth.lognormal_weights(len(ns), 0.3, seed=13)
    c["box_smu_wt_ns32"] = dict(
        box=[400.0], bintype=1, cats={"D": np.c_[ns, w]}, pairs=["DD"],
        cf=["DD / @@ - 1"], poles=[0, 2, 4], nmu=15,
        sbin=dict(smin=0, smax=60, ds=2.5), ascii=True)
    logb = np.geomspace(0.1, 50.0, 13)
    c["box_spi_log_wt"] = dict(
        box=[400.0], bintype=2, cats={"D": np.c_[ns, w]}, pairs=["DD"],
        cf=["DD / @@ - 1"], wp=True, sfile=np.c_[logb[:-1], logb[1:]],
        pbin=dict(pmin=0, pmax=30, dpi=1))
    d = synth.uniform_box(2000, 250.0, seed=14)
    r = synth.uniform_box(3000, 250.0, seed=15)
    wd = synth.lognormal_weights(2000, 0.3, seed=16)
    c["box_spi_lin_cross"] = dict(
        box=[250.0], bintype=2, cats={"D": np.c_[d, wd], "R": r},
        pairs=["DD", "DR"], cf=["DD / DR - 1"], wp=True,
        sbin=dict(smin=2, smax=40, ds=2), pbin=dict(pmin=5, pmax=25, dpi=2.5))
    d2 = synth.uniform_box(2500, [300.0, 240.0, 270.0], seed=17)
    r2 = synth.uniform_box(2500, [300.0, 240.0, 270.0], seed=18)
    c["box_smu_cuboid_smin"] = dict(
        box=[300.0, 240.0, 270.0], bintype=1, cats={"D": d2, "R": r2},
        pairs=["DD", "DR", "RR"], cf=["(DD - 2*DR + RR) / RR"],
        poles=[0, 2], nmu=10, sbin=dict(smin=5, smax=45, ds=4))
    c["box_iso_hybrid"] = dict(
        box=[300.0], bintype=0, cats={"D": x}, pairs=["DD"],
        cf=["DD / @@ - 1"], sfile=np.c_[np.geomspace(0.5, 40, 21)[:-1],
                                        np.geomspace(0.5, 40, 21)[1:]])
    c["box_smu_oddstep"] = dict(
        box=[300.0], bintype=1, cats={"D": x}, pairs=["DD"],
        cf=["DD / @@ - 1"], poles=[0, 2], nmu=8,
        sbin=dict(smin=0, smax=12.3457 * 2, ds=0.123457 * 2))
    return c


def survey_cases():
    c = {}
    kw = dict(ra=(100.0, 112.0), dec=(0.0, 12.0), zmu=0.45, zsig=0.05,
              zr=(0.4, 0.5))
    rd = synth.survey_radecz(1500, seed=21, **kw)
    rr = synth.survey_radecz(4500, seed=22, **kw)
    xd = synth.radecz_to_xyz(rd)
    xr = synth.radecz_to_xyz(rr)
    wd = synth.fkp_weights(rd, ra=kw["ra"], dec=kw["dec"])
    # FCFC_2PT crashes when only some catalogues carry weights (its unit
    # weight path), so randoms get an explicit column of ones here.
    xr1 = np.c_[xr, np.ones(len(xr))]
    ls = ["(DD - 2*DR + RR) / RR"]
    c["survey_smu_ls"] = dict(
        bintype=1, cats={"D": np.c_[xd, wd], "R": xr1}, pairs=["DD", "DR", "RR"],
        cf=ls, poles=[0, 2, 4], nmu=20, sbin=dict(smin=0, smax=50, ds=5),
        ascii=True)
    logb = np.geomspace(0.5, 50.0, 11)
    c["survey_spi_log_ls"] = dict(
        bintype=2, cats={"D": np.c_[xd, wd], "R": xr1}, pairs=["DD", "DR", "RR"],
        cf=ls, wp=True, sfile=np.c_[logb[:-1], logb[1:]],
        pbin=dict(pmin=0, pmax=40, dpi=2))
    c["survey_spi_lin_ls"] = dict(
        bintype=2, cats={"D": np.c_[xd, wd], "R": xr1}, pairs=["DD", "DR", "RR"],
        cf=ls, wp=True, sbin=dict(smin=0, smax=40, ds=4),
        pbin=dict(pmin=0, pmax=30, dpi=3))
    c["survey_iso_cross"] = dict(
        bintype=0, cats={"D": xd, "R": xr}, pairs=["DR"], cf=["DR"],
        sbin=dict(smin=1, smax=41, ds=2))
    c["survey_smu_unwt"] = dict(
        bintype=1, cats={"D": xd, "R": xr}, pairs=["DD", "DR", "RR"],
        cf=ls, poles=[0, 2], nmu=12, sbin=dict(smin=2, smax=42, ds=4))
    # RA/Dec/z input converted by FCFC itself (COORD_CONVERT = T).
    c["survey_smu_cnvt"] = dict(
        bintype=1, cats={"D": np.c_[rd, wd]}, pairs=["DD"], cf=["DD"],
        poles=[0], nmu=10, sbin=dict(smin=0, smax=50, ds=5), convert=True,
        omega_m=0.31)
    # Unweighted, so the integer counts pin the conversion bit for bit:
    # a curved wCDM cosmology (Omega_k != 0, w != -1: the pow branch) ...
    kw2 = dict(ra=(150.0, 160.0), dec=(20.0, 30.0), zmu=0.6, zsig=0.08,
               zr=(0.5, 0.7))
    rd2 = synth.survey_radecz(2000, seed=23, **kw2)
    rr2 = synth.survey_radecz(5000, seed=24, **kw2)
    c["survey_smu_cnvt_wcdm"] = dict(
        bintype=1, cats={"D": rd2, "R": rr2}, pairs=["DD", "DR", "RR"],
        cf=ls, poles=[0, 2], nmu=10, sbin=dict(smin=0, smax=40, ds=4),
        convert=True, omega_m=0.3, omega_l=0.65, dew=-0.9, cmvdst_err=1e-10)
    # ... and a (z, comoving distance) table given by Z_CMVDST_FILE, rows out
    # of order, with a comment and a blank line.
    zt = np.linspace(0.45, 0.75, 61)
    dt = synth.comoving_distance(zt, 0.29)
    perm = np.random.default_rng(25).permutation(len(zt))
    c["survey_spi_cnvt_spline"] = dict(
        bintype=2, cats={"D": rd2, "R": rr2}, pairs=["DD", "DR", "RR"],
        cf=ls, wp=True, sbin=dict(smin=0, smax=30, ds=3),
        pbin=dict(pmin=0, pmax=30, dpi=3), convert=True,
        ztab=np.c_[zt[perm], dt[perm]])
    return c


def variant_cases():
    """Cases for the compile-time variants of FCFC: WITH_MU_ONE (mu = 1 in
    the last mu bin) and SINGLE_PREC (float coordinates: its pair-count file
    format)."""
    from fcfc_gb300 import synth
    c = {}
    # a lattice: many pairs along z, i.e. mu = 1 exactly
    g = np.arange(0.0, 200.0, 12.5)
    lat = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
    x = np.concatenate([lat, synth.uniform_box(2000, 200.0, seed=51)])
    c["box_smu_muone"] = dict(
        box=[200.0], bintype=1, cats={"D": x}, pairs=["DD"],
        cf=["DD / @@ - 1"], poles=[0, 2], nmu=10,
        sbin=dict(smin=0, smax=50, ds=5), exe="FCFC_2PT_BOX_muone")
    # survey: objects on common lines of sight (same RA, Dec)
    kw = dict(ra=(120.0, 125.0), dec=(5.0, 10.0), zmu=0.45, zsig=0.05,
              zr=(0.4, 0.5))
    rd = synth.survey_radecz(1200, seed=52, **kw)
    rd[600:, :2] = rd[:600, :2]          # pairs along the line of sight
    xs = synth.radecz_to_xyz(rd)
    c["survey_smu_muone"] = dict(
        bintype=1, cats={"D": xs}, pairs=["DD"], cf=["DD"], poles=[0],
        nmu=10, sbin=dict(smin=0, smax=40, ds=4), exe="FCFC_2PT_muone")
    c["box_smu_sp"] = dict(
        box=[200.0], bintype=1, cats={"D": synth.uniform_box(1500, 200.0,
                                                            seed=53)},
        pairs=["DD"], cf=["DD / @@ - 1"], nmu=10,
        sbin=dict(smin=0, smax=50, ds=5), exe="FCFC_2PT_BOX_sp", fmt="%f")
    return c


def expr_case():
    """Catalogue columns combined by POSITION / WEIGHT expressions and
    filtered by SELECTION (numbers, an integer flag, a string tag)."""
    from fcfc_gb300 import synth
    rng = np.random.default_rng(61)
    x = synth.uniform_box(4000, 300.0, seed=62)
    w = synth.lognormal_weights(len(x), 0.3, seed=63)
    flag = rng.integers(0, 3, len(x))
    tag = rng.choice(["A", "B"], len(x))
    lines = ["# x/2 y-1.5 z w1 w2 flag tag"]
    for i in range(len(x)):
        lines.append("%.17g %.17g %.17g %.17g %.17g %d %s" % (
            x[i, 0] / 2, x[i, 1] - 1.5, x[i, 2], w[i], 1.0 / (1 + i % 7),
            flag[i], tag[i]))
    return dict(
        box=[300.0], bintype=1, pairs=["DD"], cf=["DD / @@ - 1"], poles=[0, 2],
        nmu=10, sbin=dict(smin=0, smax=40, ds=4),
        text={"D": "\n".join(lines) + "\n"},
        keys={"ASCII_FORMATTER": '"%lf %lf %lf %lf %lf %d %s"',
              "ASCII_COMMENT": "['#']", "ASCII_SKIP": "[0]",
              "POSITION": "[$1*2, ${2} + 1.5, $3]",
              "WEIGHT": "[$4 * $5]",
              "SELECTION": """'$6 >= 1 && ($7 == "A" || $5 > 0.3)'"""})


def run_expr_case(name, case, exe):
    out = os.path.join(HERE, name)
    if os.path.isdir(out):
        shutil.rmtree(out)
    os.makedirs(out)
    with tempfile.TemporaryDirectory() as tmp:
        fn = os.path.join(tmp, "D.txt")
        open(fn, "w").write(case["text"]["D"])
        lines = ["CATALOG = [%s]" % fn, "CATALOG_LABEL = [D]",
                 "BOX_SIZE = [%r]" % case["box"][0],
                 "BINNING_SCHEME = %d" % case["bintype"],
                 "PAIR_COUNT = [DD]",
                 "PAIR_COUNT_FILE = [%s]" % os.path.join(tmp, "DD.bin"),
                 "CF_ESTIMATOR = [\"%s\"]" % case["cf"][0],
                 "CF_OUTPUT_FILE = [%s]" % os.path.join(tmp, "xi.txt"),
                 "MULTIPOLE = [0, 2]",
                 "MULTIPOLE_FILE = [%s]" % os.path.join(tmp, "mp.txt"),
                 "SEP_BIN_MIN = 0", "SEP_BIN_MAX = 40", "SEP_BIN_SIZE = 4",
                 "MU_BIN_NUM = 10", "OUTPUT_FORMAT = 0", "OVERWRITE = 2",
                 "VERBOSE = F"]
        lines += ["%s = %s" % kv for kv in case["keys"].items()]
        conf = os.path.join(tmp, "run.conf")
        open(conf, "w").write("\n".join(lines) + "\n")
        env = dict(os.environ, OMP_NUM_THREADS="4")
        subprocess.run([exe, "-c", conf], check=True, env=env,
                       stdout=subprocess.DEVNULL)
        for fnm in ("DD.bin", "xi.txt", "mp.txt"):
            shutil.copy(os.path.join(tmp, fnm), os.path.join(out, fnm))
    open(os.path.join(out, "D.txt"), "w").write(case["text"]["D"])
    meta = {k: v for k, v in case.items() if k != "text"}
    meta.update(labels=["D"], geometry="box", build=os.path.basename(exe),
                catalog_text={"D": "D.txt"}, weighted={"D": True},
                reader={"formatter": "%lf %lf %lf %lf %lf %d %s",
                        "position": ["$1*2", "${2} + 1.5", "$3"],
                        "weight": "$4 * $5",
                        "selection": '$6 >= 1 && ($7 == "A" || $5 > 0.3)',
                        "comment": "#"})
    with open(os.path.join(out, "meta.json"), "w") as f:
        json.dump(meta, f, indent=1, sort_keys=True)
    print("wrote", name)


def write_conf(case, tmp, exe_box):
    labels = list(case["cats"].keys())
    lines = []
    cats = []
    for lab in labels:
        a = case["cats"][lab]
        fn = os.path.join(tmp, lab + ".txt")
        np.savetxt(fn, a, fmt="%.17g")
        cats.append(fn)
    tok = case.get("fmt", "%lf")    # a SINGLE_PREC build reads floats
    fmt = ", ".join('"%s"' % " ".join([tok] * case["cats"][l].shape[1])
                    for l in labels)
    lines.append("CATALOG = [%s]" % ", ".join(cats))
    lines.append("CATALOG_LABEL = [%s]" % ", ".join(labels))
    lines.append("ASCII_FORMATTER = [%s]" % fmt)
    pos = []
    for _ in labels:
        pos += ["$1", "$2", "$3"]
    lines.append("POSITION = [%s]" % ", ".join(pos))
    wts = [("$4" if case["cats"][l].shape[1] > 3 else "1") for l in labels]
    if any(case["cats"][l].shape[1] > 3 for l in labels):
        lines.append("WEIGHT = [%s]" % ", ".join(wts))
    if exe_box:
        lines.append("BOX_SIZE = [%s]" % ", ".join(repr(v) for v in case["box"]))
    else:
        cnv = "T" if case.get("convert") else "F"
        lines.append("COORD_CONVERT = [%s]" % ", ".join([cnv] * len(labels)))
        lines.append("OMEGA_M = %r" % case.get("omega_m", 0.31))
        if "omega_l" in case:
            lines.append("OMEGA_LAMBDA = %r" % case["omega_l"])
        if "dew" in case:
            lines.append("DE_EOS_W = %r" % case["dew"])
        if "cmvdst_err" in case:
            lines.append("CMVDST_ERR = %r" % case["cmvdst_err"])
        if "ztab" in case:
            fn = os.path.join(tmp, "zcmv.txt")
            with open(fn, "w") as f:
                f.write("# z  comoving distance (Mpc/h)\n\n")
                for zz, dd in case["ztab"]:
                    f.write("%.17g %.17g\n" % (zz, dd))
            lines.append("Z_CMVDST_FILE = %s" % fn)
    lines.append("BINNING_SCHEME = %d" % case["bintype"])
    lines.append("PAIR_COUNT = [%s]" % ", ".join(case["pairs"]))
    lines.append("PAIR_COUNT_FILE = [%s]" % ", ".join(
        os.path.join(tmp, p + ".bin") for p in case["pairs"]))
    lines.append("CF_ESTIMATOR = [%s]" % ", ".join('"%s"' % e for e in case["cf"]))
    lines.append("CF_OUTPUT_FILE = [%s]" % os.path.join(tmp, "xi.txt"))
    if case.get("poles"):
        lines.append("MULTIPOLE = [%s]" % ", ".join(map(str, case["poles"])))
        lines.append("MULTIPOLE_FILE = [%s]" % os.path.join(tmp, "mp.txt"))
    if case.get("wp"):
        lines.append("PROJECTED_CF = T")
        lines.append("PROJECTED_FILE = [%s]" % os.path.join(tmp, "wp.txt"))
    if "sfile" in case:
        fn = os.path.join(tmp, "sbins.txt")
        np.savetxt(fn, case["sfile"], fmt="%.17g")
        lines.append("SEP_BIN_FILE = %s" % fn)
    else:
        s = case["sbin"]
        lines += ["SEP_BIN_MIN = %r" % s["smin"], "SEP_BIN_MAX = %r" % s["smax"],
                  "SEP_BIN_SIZE = %r" % s["ds"]]
    if case["bintype"] == 1:
        lines.append("MU_BIN_NUM = %d" % case.get("nmu", 10))
    if case["bintype"] == 2:
        p = case["pbin"]
        lines += ["PI_BIN_MIN = %r" % p["pmin"], "PI_BIN_MAX = %r" % p["pmax"],
                  "PI_BIN_SIZE = %r" % p["dpi"]]
    lines += ["OVERWRITE = 2", "VERBOSE = F"]
    return lines


def run_case(name, case, exe):
    out = os.path.join(HERE, name)
    if os.path.isdir(out):
        shutil.rmtree(out)
    os.makedirs(out)
    box = "BOX" in os.path.basename(exe)
    with tempfile.TemporaryDirectory() as tmp:
        for ofmt in ([0, 1] if case.get("ascii") else [0]):
            lines = write_conf(case, tmp, box) + ["OUTPUT_FORMAT = %d" % ofmt]
            conf = os.path.join(tmp, "run.conf")
            with open(conf, "w") as f:
                f.write("\n".join(lines) + "\n")
            env = dict(os.environ, OMP_NUM_THREADS="4")
            subprocess.run([exe, "-c", conf], check=True, env=env,
                           stdout=subprocess.DEVNULL)
            for p in case["pairs"]:
                shutil.copy(os.path.join(tmp, p + ".bin"),
                            os.path.join(out, p + (".bin" if ofmt == 0 else ".txt")))
        orders = []
        if case.get("convert") and "ztab" not in case:
            # the Gauss-Legendre order FCFC picks, from its verbose output
            lines = [l for l in write_conf(case, tmp, box)
                     if not l.startswith("VERBOSE")]
            lines += ["OUTPUT_FORMAT = 0", "VERBOSE = T"]
            with open(conf, "w") as f:
                f.write("\n".join(lines) + "\n")
            log = subprocess.run([exe, "-c", conf], check=True, env=env,
                                 capture_output=True, text=True).stdout
            tag = "Legendre-Gauss integration with order"
            orders = [int(l.split(tag)[1]) for l in log.splitlines() if tag in l]
        for fn in ("xi.txt", "mp.txt", "wp.txt"):
            if os.path.exists(os.path.join(tmp, fn)):
                shutil.copy(os.path.join(tmp, fn), os.path.join(out, fn))
        if "sfile" in case:
            shutil.copy(os.path.join(tmp, "sbins.txt"), os.path.join(out, "sbins.txt"))
        if "ztab" in case:
            shutil.copy(os.path.join(tmp, "zcmv.txt"), os.path.join(out, "zcmv.txt"))
    for lab, a in case["cats"].items():
        np.save(os.path.join(out, lab + ".npy"), np.ascontiguousarray(a))
    meta = {k: v for k, v in case.items()
            if k not in ("cats", "sfile", "ztab", "exe")}
    meta["build"] = case.get("exe", os.path.basename(exe))
    if "ztab" in case:
        meta["zfile"] = "zcmv.txt"
    if orders:
        meta["cnvt_order"] = orders   # one per catalogue, in label order
    meta["labels"] = list(case["cats"].keys())
    meta["weighted"] = {l: bool(a.shape[1] > 3) for l, a in case["cats"].items()}
    meta["geometry"] = "box" if box else "survey"
    if "sfile" in case:
        meta["sfile"] = "sbins.txt"
    with open(os.path.join(out, "meta.json"), "w") as f:
        json.dump(meta, f, indent=1, sort_keys=True)
    print("wrote", name)


def main(argv):
    allc = {}
    for name, c in box_cases().items():
        allc[name] = (c, os.path.join(REF, "FCFC_2PT_BOX"))
    for name, c in survey_cases().items():
        allc[name] = (c, os.path.join(REF, "FCFC_2PT"))
    for name, c in variant_cases().items():
        allc[name] = (c, os.path.join(REF, c["exe"]))
    special = {"box_smu_expr": (expr_case, "FCFC_2PT_BOX")}
    names = argv or sorted(list(allc) + list(special))
    for n in names:
        if n in special:
            mk, exe = special[n]
            run_expr_case(n, mk(), os.path.join(REF, exe))
        else:
            run_case(n, *allc[n])


if __name__ == "__main__":
    main(sys.argv[1:])
