"""Loading of the golden fixtures written by tests/golden/make_golden.py."""
from __future__ import annotations

import json
import os

import numpy as np

from fcfc_gb300 import pcfile

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def case_names(convert=None, single_prec=False):
    """Golden case names; convert=True / False keeps only the cases whose
    catalogues are RA/Dec/z (COORD_CONVERT) / Cartesian.  Cases written by a
    SINGLE_PREC build of FCFC (float arithmetic: other counts, another file
    layout) come only with single_prec=True (only them) or None (all)."""
    out = []
    for d in sorted(os.listdir(GOLDEN)):
        fn = os.path.join(GOLDEN, d, "meta.json")
        if not os.path.isfile(fn):
            continue
        with open(fn) as f:
            m = json.load(f)
        if convert is not None and bool(m.get("convert")) != convert:
            continue
        sp = m.get("build", "").endswith("_sp")
        if single_prec is not None and sp != single_prec:
            continue
        out.append(d)
    return out


class Case:
    def __init__(self, name):
        self.name = name
        self.dir = os.path.join(GOLDEN, name)
        with open(os.path.join(self.dir, "meta.json")) as f:
            self.meta = json.load(f)
        if self.meta.get("catalog_text"):
            # an ASCII catalogue read through FCFC's column expressions
            from fcfc_gb300 import ascii
            r = self.meta["reader"]
            self.cats = {}
            for l, fn in self.meta["catalog_text"].items():
                xyz, w = ascii.read_ascii(os.path.join(self.dir, fn),
                                          r["formatter"], r["position"],
                                          r.get("weight"), r.get("selection"),
                                          0, r.get("comment"))
                self.cats[l] = xyz if w is None else np.c_[xyz, w]
        else:
            self.cats = {l: np.load(os.path.join(self.dir, l + ".npy"))
                         for l in self.meta["labels"]}
        self.box = self.meta.get("geometry") == "box"
        self.sedges = None
        if self.meta.get("sfile"):
            t = np.loadtxt(os.path.join(self.dir, self.meta["sfile"]), ndmin=2)
            # read_bins: lower edges, with the midpoint of a discontinuity
            e = np.empty(len(t) + 1)
            e[0] = t[0, 0]
            for i in range(1, len(t)):
                e[i] = t[i, 0] if t[i, 0] == t[i - 1, 1] else 0.5 * (t[i, 0] + t[i - 1, 1])
            e[-1] = t[-1, 1]
            self.sedges = e

    def pcfile(self, pair):
        return pcfile.read_binary(os.path.join(self.dir, pair + ".bin"))

    def bins_kwargs(self):
        m = self.meta
        kw = dict(bintype=m["bintype"])
        if self.sedges is not None:
            kw.update(ns=len(self.sedges) - 1, sedges=self.sedges)
        else:
            s = m["sbin"]
            n, v = 0, s["smin"]
            while v < s["smax"] - 1e-10:
                v += s["ds"]
                n += 1
            kw.update(ns=n, smin=s["smin"], ds=s["ds"])
        if m["bintype"] == 1:
            kw["nmu"] = m.get("nmu", 10)
        if m["bintype"] == 2:
            p = m["pbin"]
            n, v = 0, p["pmin"]
            while v < p["pmax"] - 1e-10:
                v += p["dpi"]
                n += 1
            kw.update(np_=n, pmin=p["pmin"], dpi=p["dpi"])
        if self.box:
            kw["box"] = (m["box"] * 3)[:3] if len(m["box"]) == 1 else m["box"]
        if self.mu_one:
            kw["with_mu_one"] = True
        return kw

    @property
    def mu_one(self):
        """Written by a WITH_MU_ONE build (mu = 1 in the last mu bin)."""
        return self.meta.get("build", "").endswith("_muone")

    @property
    def convert(self):
        return bool(self.meta.get("convert"))

    def cosmo(self):
        """OMEGA_M, OMEGA_LAMBDA (None: flat), DE_EOS_W, CMVDST_ERR."""
        m = self.meta
        return dict(omega_m=m.get("omega_m", 0.31), omega_l=m.get("omega_l"),
                    dew=m.get("dew", -1.0), err=m.get("cmvdst_err", 1e-8))

    def ztable(self):
        """Z_CMVDST_FILE rows (z, d) in file order, or None."""
        if not self.meta.get("zfile"):
            return None
        rows = []
        with open(os.path.join(self.dir, self.meta["zfile"])) as f:
            for line in f:
                t = line.strip()
                if t and not t.startswith("#"):
                    rows.append([float(v) for v in t.split()[:2]])
        return np.array(rows)

    def xyzw(self, label):
        a = self.cats[label]
        return a[:, :3], (a[:, 3] if a.shape[1] > 3 else None)


# --------------------------------------------------------------------------
# Full-size fixtures (tests/golden/full, written by make_golden_full.py):
# FCFC's pair-count files for the benchmark workloads at their stated sizes.
# The catalogues are regenerated from their specs and checked by sha256.

FULL = os.path.join(GOLDEN, "full")


def full_case_names():
    if not os.path.isdir(FULL):
        return []
    return sorted(d for d in os.listdir(FULL)
                  if os.path.isfile(os.path.join(FULL, d, "meta.json")))


class FullCase:
    _cache: dict = {}

    def __init__(self, name):
        self.name = name
        self.dir = os.path.join(FULL, name)
        with open(os.path.join(self.dir, "meta.json")) as f:
            self.meta = json.load(f)
        self.box = self.meta["geometry"] == "box"

    def catalogue(self, label):
        """(N x 3 or 4 array, sha256 as generated, sha256 recorded)."""
        from fcfc_gb300 import synth
        c = self.meta["cats"][label]
        key = json.dumps(c["spec"], sort_keys=True)
        if key not in FullCase._cache:
            a = synth.catalogue(c["spec"])
            FullCase._cache.clear()          # hold one catalogue set at most
            FullCase._cache[key] = (a, synth.catalogue_sha256(a))
        a, h = FullCase._cache[key]
        return a, h, c["sha256"]

    def runs(self):
        return self.meta["runs"]

    def pcfile(self, run, pair):
        return pcfile.read_binary(os.path.join(self.dir, "%s_%s.bin" % (
            run["name"], pair)))

    def sedges(self, run):
        if not run.get("sfile"):
            return None
        t = np.loadtxt(os.path.join(self.dir, run["sfile"]), ndmin=2)
        e = np.empty(len(t) + 1)
        e[0] = t[0, 0]
        for i in range(1, len(t)):
            e[i] = t[i, 0] if t[i, 0] == t[i - 1, 1] else 0.5 * (t[i, 0] + t[i - 1, 1])
        e[-1] = t[-1, 1]
        return e

    def engine_kwargs(self, run):
        """PairCounter keyword arguments of a run's binning."""
        kw = dict(geometry="box" if self.box else "survey",
                  bintype=run["bintype"])
        se = self.sedges(run)
        if se is not None:
            kw["sedges"] = se
        else:
            s = run["sbin"]
            kw.update(smin=s["smin"], smax=s["smax"], ds=s["ds"])
        if run["bintype"] == 1:
            kw["nmu"] = run["nmu"]
        if run["bintype"] == 2:
            p = run["pbin"]
            kw.update(pmin=p["pmin"], pmax=p["pmax"], dpi=p["dpi"])
        if self.box:
            kw["box"] = run["box"][0]
        return kw
