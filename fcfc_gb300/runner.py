"""FCFC-compatible run flow on the GB300 engine.

Takes FCFC's configuration keys (a libcfg-style file or a dict), counts the
pairs listed in PAIR_COUNT on the GPU, writes PAIR_COUNT_FILE, evaluates
CF_ESTIMATOR into CF_OUTPUT_FILE, and the Legendre multipoles / projected
correlation function into MULTIPOLE_FILE / PROJECTED_FILE -- the sequence of
FCFC's eval_cf (src/fcfc/2pt_box/eval_cf.c:405, survey src/fcfc/2pt/eval_cf.c).
Outputs are checked first, as FCFC's check_output does
(src/fcfc/2pt_box/load_conf.c:582-650): OVERWRITE = 0 refuses existing
files, 1 reads existing pair-count files back instead of recounting them.

    python -m fcfc_gb300.runner --box -c fcfc_2pt_box.conf
    python -m fcfc_gb300.runner --survey -c fcfc_2pt.conf
"""
from __future__ import annotations

import argparse
import ctypes as C
import os
import re
import shlex
import sys

import numpy as np

from . import ascii, capi
from .capi import BIN_SMU, BIN_SPI, FCFCGError
from .engine import PairCounter


# --------------------------------------------------------------------------
# configuration

def parse_conf(text: str) -> dict:
    """libcfg syntax: KEY = value or [a, b, ...]; '#' comments; '\\' joins
    lines; values may be quoted.  A key given twice keeps its first value,
    as libcfg does (src/lib/libcfg.c:1219-1232)."""
    out = {}
    text = re.sub(r"\\\s*\n", " ", text)
    for line in text.splitlines():
        s = line.strip()
        if not s or s.startswith("#"):
            continue
        if "=" not in s:
            continue
        k, v = s.split("=", 1)
        k = k.strip()
        v = _strip_comment(v).strip()
        if not v or k in out:
            continue
        if v.startswith("["):
            inner = v[1:v.rindex("]")] if "]" in v else v[1:]
            lex = shlex.shlex(inner, posix=True)
            lex.whitespace = ","
            lex.whitespace_split = True
            lex.commenters = ""
            out[k] = [t.strip() for t in lex]
        else:
            out[k] = _unquote(v)
    return out


def _strip_comment(v):
    q = None
    for i, ch in enumerate(v):
        if ch in "'\"":
            q = None if q == ch else (ch if q is None else q)
        elif ch == "#" and q is None:
            return v[:i]
    return v


def _unquote(v):
    v = v.strip()
    if len(v) >= 2 and v[0] == v[-1] and v[0] in "'\"":
        return v[1:-1]
    return v


def _arr(conf, key, n=None, default=None, cast=str):
    v = conf.get(key, default)
    if v is None:
        return None
    if not isinstance(v, list):
        v = [v]
    v = [cast(x) if not isinstance(x, str) or cast is str else cast(_unquote(x))
         for x in v]
    if n is not None and len(v) == 1 and n > 1:
        v = v * n
    return v


def _bool(x):
    return str(x).strip().upper() in ("T", "TRUE", "1", "Y", "YES")


# --------------------------------------------------------------------------
# catalogues

def read_catalog(path, formatter=None, position=("$1", "$2", "$3"),
                 weight=None, skip=0, comment=None, selection=None):
    """A catalogue as FCFC reads it: ASCII with ASCII_FORMATTER, POSITION /
    WEIGHT column expressions and SELECTION (see ascii.py); .npy arrays
    (columns x y z [w]) are read directly."""
    if path.endswith(".npy"):
        a = np.load(path)
        w = a[:, 3] if (weight is not None and a.shape[1] > 3) else None
        return a[:, :3].astype(np.float64), w
    if not formatter:
        ncol = max(int(c) for c in re.findall(r"\$\{?(\d+)",
                                              " ".join(list(position) +
                                                       [weight or "",
                                                        selection or ""])))
        formatter = " ".join(["%lf"] * ncol)
    return ascii.read_ascii(path, formatter, list(position), weight, selection,
                            int(skip or 0), comment if comment else None)


def read_ztable(path):
    """Z_CMVDST_FILE: two numbers (z, comoving distance) per line; '#' lines
    and blank lines are skipped, as read_ascii_table does
    (src/io/read_ascii.c:398-500)."""
    rows = []
    with open(path) as f:
        for line in f:
            t = line.lstrip()
            if not t or t.startswith("#"):
                continue
            v = t.split()
            try:
                rows.append((float(v[0]), float(v[1])))
            except (IndexError, ValueError):
                raise FCFCGError(capi.ERR_FILE, "failed to read line: %s" % t)
    return np.array(rows, np.float64).reshape(-1, 2)


def cosmo_from_conf(conf):
    """The conversion keys of FCFC_2PT (load_conf.c:532-536): OMEGA_M,
    OMEGA_LAMBDA, DE_EOS_W, CMVDST_ERR, or Z_CMVDST_FILE."""
    if conf.get("Z_CMVDST_FILE"):
        return dict(ztable=read_ztable(conf["Z_CMVDST_FILE"]))
    if "OMEGA_M" not in conf:
        raise FCFCGError(capi.ERR_CFG, "OMEGA_M is not set")
    c = dict(omega_m=float(conf["OMEGA_M"]))
    if "OMEGA_LAMBDA" in conf:
        c["omega_l"] = float(conf["OMEGA_LAMBDA"])
    if "DE_EOS_W" in conf:
        c["dew"] = float(conf["DE_EOS_W"])
    if "CMVDST_ERR" in conf:
        c["cmvdst_err"] = float(conf["CMVDST_ERR"])
    return c


def read_bins_file(path):
    """Edges as FCFC's read_bins builds them (setup_cf.c:74-119)."""
    t = np.loadtxt(path, comments="#", ndmin=2)
    e = np.empty(len(t) + 1)
    e[0] = t[0, 0]
    for i in range(1, len(t)):
        if abs(t[i, 0] - t[i - 1, 1]) > 1e-10:
            raise FCFCGError(capi.ERR_FILE, "discontinuous separation bins")
        e[i] = t[i, 0] if t[i, 0] == t[i - 1, 1] else 0.5 * (t[i, 0] + t[i - 1, 1])
    e[-1] = t[-1, 1]
    return e


# --------------------------------------------------------------------------

def check_output(fname, key, ovw, force, ask=input):
    """FCFC's check_output (src/fcfc/2pt_box/load_conf.c:582-650): False to
    write the file, True to read it back (an existing pair-count file with
    0 < OVERWRITE < force); FCFC's refusals raise.  force: 2 for
    PAIR_COUNT_FILE, 1 for the correlation function outputs.  A negative
    OVERWRITE asks (``ask``) up to |OVERWRITE| times."""
    if not fname:
        raise FCFCGError(capi.ERR_CFG, "the output file %s is not set" % key)
    if os.path.exists(fname):
        if ovw < 0:
            for _ in range(-ovw):
                try:
                    a = ask("%s exists: `%s'; overwrite it? (y/n): "
                            % (key, fname))[:1]
                except EOFError:
                    continue
                if a in ("n", "N"):
                    ovw = force - 1
                    break
                if a in ("y", "Y"):
                    ovw = force
                    break
            else:
                raise FCFCGError(capi.ERR_FILE, "too many failed inputs")
        if ovw <= 0:
            raise FCFCGError(capi.ERR_FILE, "abort to avoid overwriting %s: "
                             "`%s'" % (key, fname))
        if ovw < force:
            if not os.access(fname, os.R_OK):
                raise FCFCGError(capi.ERR_FILE, "cannot access %s: `%s'"
                                 % (key, fname))
            return True
        if not os.access(fname, os.W_OK):
            raise FCFCGError(capi.ERR_FILE, "cannot write to file: `%s'"
                             % fname)
    else:
        d = os.path.dirname(fname)
        if d and not os.access(d, os.X_OK):
            raise FCFCGError(capi.ERR_FILE, "cannot access the directory `%s'"
                             % d)
    return False


def run(conf: dict, geometry: str = "box", device: int = -1,
        precision: int = capi.PREC_FP32_RECHECK, verbose: bool = False,
        with_mu_one: bool = False, graph: bool = True):
    """Run one FCFC job.  Returns a dict with counts, xi, multipoles, wp.
    with_mu_one: behave as FCFC built with -DWITH_MU_ONE.  graph: when the
    catalogues fit the 8 slots, count every pair through one CUDA graph
    (the same counts as one at a time)."""
    box = geometry == "box"
    files = _arr(conf, "CATALOG")
    ncat = len(files)
    labels = _arr(conf, "CATALOG_LABEL") or [chr(ord("A") + i) for i in range(ncat)]
    # capital letters, each once (load_conf.c:675-705)
    labels = [l[:1] for l in labels]
    for i, l in enumerate(labels):
        if not ("A" <= l <= "Z"):
            raise FCFCGError(capi.ERR_CFG, "invalid CATALOG_LABEL: %r" % l)
        if l in labels[:i]:
            raise FCFCGError(capi.ERR_CFG, "duplicate CATALOG_LABEL: %s" % l)
    fmtr = _arr(conf, "ASCII_FORMATTER", ncat)
    pos = _arr(conf, "POSITION")
    wts = _arr(conf, "WEIGHT", ncat)
    skip = _arr(conf, "ASCII_SKIP", ncat, default=[0] * ncat)
    cmt = _arr(conf, "ASCII_COMMENT", ncat)
    sel = _arr(conf, "SELECTION", ncat)
    # DATA_STRUCT: k-d tree (0) or ball tree (1), both the cell grid here;
    # other values rejected as FCFC does (load_conf.c:825-834)
    if int(conf.get("DATA_STRUCT", 0)) not in (0, 1):
        raise FCFCGError(capi.ERR_CFG, "invalid DATA_STRUCT: %s"
                         % conf["DATA_STRUCT"])
    bintype = int(conf.get("BINNING_SCHEME", 0))
    pairs = _arr(conf, "PAIR_COUNT")
    pcout = _arr(conf, "PAIR_COUNT_FILE")
    if not pairs:
        raise FCFCGError(capi.ERR_CFG, "PAIR_COUNT is not set")
    if not pcout or len(pcout) < len(pairs):
        raise FCFCGError(capi.ERR_CFG, "PAIR_COUNT_FILE needs one file per pair")
    est = _arr(conf, "CF_ESTIMATOR") or []
    cfout = _arr(conf, "CF_OUTPUT_FILE") or []
    # sorted, without duplicates, 0 to 6 (load_conf.c:915-941)
    poles = sorted({int(p) for p in (_arr(conf, "MULTIPOLE") or [])})
    if poles and (poles[0] < 0 or poles[-1] > 6):
        raise FCFCGError(capi.ERR_CFG, "MULTIPOLE must be between 0 and 6")
    mpout = _arr(conf, "MULTIPOLE_FILE") or []
    do_wp = _bool(conf.get("PROJECTED_CF", "F"))
    wpout = _arr(conf, "PROJECTED_FILE") or []
    ofmt = int(conf.get("OUTPUT_FORMAT", 0))
    ovw = int(conf.get("OVERWRITE", 0))
    cnvt = [False] * ncat
    cosmo = None
    if not box:
        # one value for all catalogues, else at least one per catalogue
        # (load_conf.c:885-906)
        cv = _arr(conf, "COORD_CONVERT", ncat)
        if cv:
            if len(cv) < ncat:
                raise FCFCGError(capi.ERR_CFG, "too few elements of COORD_CONVERT")
            cnvt = [_bool(v) for v in cv[:ncat]]
        if any(cnvt):
            cosmo = cosmo_from_conf(conf)

    # the outputs, checked as FCFC does before any counting: existing
    # pair-count files with OVERWRITE = 1 are read back, the others counted
    readback = [check_output(pcout[k] if k < len(pcout) else None,
                             "PAIR_COUNT_FILE", ovw, 2)
                for k in range(len(pairs))]
    if est:
        outs = [("CF_OUTPUT_FILE", cfout)]
        if poles and bintype == BIN_SMU:
            outs.append(("MULTIPOLE_FILE", mpout))
        if do_wp and bintype == BIN_SPI:
            outs.append(("PROJECTED_FILE", wpout))
        for key, files_ in outs:
            if len(files_) < len(est):
                raise FCFCGError(capi.ERR_CFG, "too few elements of %s" % key)
            for k in range(len(est)):
                check_output(files_[k], key, ovw, 1)
    # each estimator parses and names only counted pairs (setup_cf.c:
    # 128-200): evaluated once on zero counts before any device work
    if est:
        lib = capi.load_library()
        z = np.zeros(len(pairs))
        zrr = np.zeros(1)
        one = np.zeros(1)
        for e in est:
            if lib.fcfcg_cf_eval(e.encode(), len(pairs), "".join(pairs).encode(),
                                 capi.ptr(z), capi.ptr(zrr) if box else None,
                                 1, capi.ptr(one)):
                raise FCFCGError(capi.ERR_CFG, "invalid CF_ESTIMATOR %r (a "
                                 "syntax error, or a pair not in PAIR_COUNT)"
                                 % e)
    kw = dict(geometry=geometry, bintype=bintype, device=device)
    if box:
        b = [float(v) for v in _arr(conf, "BOX_SIZE")]
        kw["box"] = b * 3 if len(b) == 1 else b
    if conf.get("SEP_BIN_FILE"):
        kw["sedges"] = read_bins_file(conf["SEP_BIN_FILE"])
    else:
        kw.update(smin=float(conf["SEP_BIN_MIN"]), smax=float(conf["SEP_BIN_MAX"]),
                  ds=float(conf["SEP_BIN_SIZE"]))
    if bintype == BIN_SMU:
        kw["nmu"] = int(conf["MU_BIN_NUM"])
    if bintype == BIN_SPI:
        if conf.get("PI_BIN_FILE"):
            kw["pedges"] = read_bins_file(conf["PI_BIN_FILE"])
        else:
            kw.update(pmin=float(conf["PI_BIN_MIN"]), pmax=float(conf["PI_BIN_MAX"]),
                      dpi=float(conf["PI_BIN_SIZE"]))

    pc = PairCounter(with_mu_one=with_mu_one, **kw)

    def load_cat(i, slot):
        p3 = pos[3 * i: 3 * i + 3]
        w = wts[i] if wts and wts[i] not in (None, "", "''", '""', "1") \
            else None
        x, ww = read_catalog(files[i], fmtr[i] if fmtr else None, p3, w,
                             skip[i], cmt[i] if cmt else None,
                             sel[i] if sel and sel[i] not in ("", "''", '""')
                             else None)
        if cnvt[i]:
            pc.load_radecz(slot, x, ww, **cosmo)
        else:
            pc.load(slot, x, ww)

    # an empty weight or "1" means no weights (load_conf.c:780-789)
    weighted_cat = {}
    for i, lab in enumerate(labels):
        w = wts[i] if wts else None
        weighted_cat[lab] = w not in (None, "", "''", '""', "1")

    done, todo = {}, []
    for k, pair in enumerate(pairs):
        if readback[k]:
            done[k] = pc.read_paircount(pcout[k])
        else:
            todo.append(k)
    need = []            # catalogues the counts use, in order of first use
    for k in todo:
        for lab in pairs[k][:2]:
            i = labels.index(lab)
            if i not in need:
                need.append(i)
    counts, slots = {}, {}
    if todo and len(need) <= 8 and graph:
        # every count at once: DD, DR, RR, ... replayed from one CUDA graph
        slot = {i: s for s, i in enumerate(need)}
        for i in need:
            load_cat(i, slot[i])
        items = []
        for k in todo:
            a, bl = pairs[k][0], pairs[k][1]
            sa, sb = slot[labels.index(a)], slot[labels.index(bl)]
            slots[k] = (sa, sb)
            items.append((sa, None if a == bl else sb,
                          weighted_cat[a] or weighted_cat[bl]))
        g = pc.count_graph(items, precision=precision)
        try:
            for k, c in zip(todo, g.run()):
                counts[k] = c
        finally:
            g.close()
    else:
        # one count at a time, catalogue i in slot i % 8
        loaded = {}
        for k in todo:
            a, bl = pairs[k][0], pairs[k][1]
            for lab in (a, bl):
                i = labels.index(lab)
                if loaded.get(i % 8) != i:
                    load_cat(i, i % 8)
                    loaded[i % 8] = i
            ia, ib = labels.index(a), labels.index(bl)
            if loaded.get(ia % 8) != ia or loaded.get(ib % 8) != ib:
                raise FCFCGError(capi.ERR_CFG, "catalogues %s and %s share a "
                                 "slot: at most 8 catalogues per pair set"
                                 % (a, bl))
            sa, sb = ia % 8, ib % 8
            slots[k] = (sa, sb)
            counts[k] = pc.count_pairs(sa, None if a == bl else sb,
                                       weighted=weighted_cat[a] or
                                       weighted_cat[bl], precision=precision)

    ncnt_all = []
    out = {"counts": {}, "norm": {}}
    for k, pair in enumerate(pairs):
        if k in done:
            r = done[k]
            ncnt_all.append(r["ncnt"])
            out["counts"][pair] = r["cnt"]
            out["norm"][pair] = r["norm"]
            continue
        a, bl = pair[0], pair[1]
        isauto = a == bl
        weighted = weighted_cat[a] or weighted_cat[bl]
        sa, sb = slots[k]
        na, wa = pc.catalog_info(sa)
        nb, wb = pc.catalog_info(sb)
        if weighted:
            n1, n2 = wa, wb
        else:
            n1, n2 = float(na), float(nb)
        cnt2, norm, ncnt = pc.normalise(counts[k], isauto, weighted, n1, n2)
        pc.write_paircount(pcout[k], ofmt, isauto, weighted,
                           [na] if isauto else [na, nb],
                           [wa] if isauto else [wa, wb], norm, ncnt, cnt2)
        ncnt_all.append(ncnt)
        out["counts"][pair] = cnt2
        out["norm"][pair] = norm
        if verbose:
            print("counted %s" % pair)

    rr = pc.analytic_rr() if box else None
    if est:
        lab = "".join(pairs).encode()
        nc = np.ascontiguousarray(np.stack(ncnt_all), np.float64)
        out["xi"] = []
        out["mp"] = []
        out["wp"] = []
        for k, e in enumerate(est):
            xi = np.zeros(pc.ntot)
            rc = pc.lib.fcfcg_cf_eval(
                e.encode(), len(pairs), lab, capi.ptr(nc),
                capi.ptr(rr) if rr is not None else None, pc.ntot,
                capi.ptr(xi))
            if rc:
                raise FCFCGError(rc, "CF_ESTIMATOR %r" % e)
            pc.write_cf(cfout[k], xi)
            out["xi"].append(xi)
            if poles and bintype == BIN_SMU:
                mp = pc.multipoles(xi, poles)
                pc.write_multipoles(mpout[k], poles, mp)
                out["mp"].append(mp)
            elif do_wp and bintype == BIN_SPI:
                wp = pc.wp(xi)
                pc.write_wp(wpout[k], wp)
                out["wp"].append(wp)
    return out


# FCFC's command line options and the keys they set (short, long, key,
# Boolean), src/fcfc/2pt_box/load_conf.c:477-515, src/fcfc/2pt/load_conf.c:
# 512-553; box-only and survey-only entries are marked
OPTIONS = [
    ("i", "input", "CATALOG", 0), ("l", "label", "CATALOG_LABEL", 0),
    ("T", "type", "CATALOG_TYPE", 0), (None, "skip", "ASCII_SKIP", 0),
    (None, "comment", "ASCII_COMMENT", 0), ("f", "formatter", "ASCII_FORMATTER", 0),
    ("x", "position", "POSITION", 0), ("w", "weight", "WEIGHT", 0),
    ("s", "select", "SELECTION", 0), ("b", "box", "BOX_SIZE", "box-opt"),
    (None, "convert", "COORD_CONVERT", "survey-bool"),
    ("d", "omega-m", "OMEGA_M", "survey"), (None, "omega-l", "OMEGA_LAMBDA", "survey"),
    (None, "eos-w", "DE_EOS_W", "survey"), (None, "cmvdst-err", "CMVDST_ERR", "survey"),
    (None, "cmvdst-file", "Z_CMVDST_FILE", "survey"),
    ("S", "data-struct", "DATA_STRUCT", 0), ("B", "bin", "BINNING_SCHEME", 0),
    ("p", "pair", "PAIR_COUNT", 0), ("P", "pair-output", "PAIR_COUNT_FILE", 0),
    ("e", "cf", "CF_ESTIMATOR", 0), ("E", "cf-output", "CF_OUTPUT_FILE", 0),
    ("m", "multipole", "MULTIPOLE", 0), ("M", "mp-output", "MULTIPOLE_FILE", 0),
    ("u", "wp", "PROJECTED_CF", "bool"), ("U", "wp-output", "PROJECTED_FILE", 0),
    (None, "s-file", "SEP_BIN_FILE", 0), (None, "s-min", "SEP_BIN_MIN", 0),
    (None, "s-max", "SEP_BIN_MAX", 0), (None, "s-step", "SEP_BIN_SIZE", 0),
    (None, "mu-num", "MU_BIN_NUM", 0), (None, "pi-file", "PI_BIN_FILE", 0),
    (None, "pi-min", "PI_BIN_MIN", 0), (None, "pi-max", "PI_BIN_MAX", 0),
    (None, "pi-step", "PI_BIN_SIZE", 0), ("F", "out-format", "OUTPUT_FORMAT", 0),
    ("O", "overwrite", "OVERWRITE", 0),
]


class _FirstValue(argparse.Action):
    """Keep an option's first value, as libcfg does (a repeated option is
    reported and dropped, src/lib/libcfg.c:1106-1112)."""

    def __call__(self, parser, namespace, values, option_string=None):
        if getattr(namespace, self.dest, None) is not None:
            print("Warning: omitting duplicate entry of parameter `%s'"
                  % self.dest, file=sys.stderr)
            return
        setattr(namespace, self.dest, values)


def main(argv=None):
    """FCFC's command line: every option sets its key over the configuration
    file's value; the file defaults to FCFC's name for the geometry, and a
    missing one leaves the command line's keys alone."""
    ap = argparse.ArgumentParser(description="FCFC run flow on the GB300 engine")
    # --survey: FCFC_2PT's flow; FCFC_2PT_BOX's otherwise.  --box alone
    # selects the box flow too, --box VALUE (or -b) is FCFC's BOX_SIZE.
    ap.add_argument("--survey", action="store_true", help="FCFC_2PT keys")
    ap.add_argument("-c", "--conf", default=None)
    ap.add_argument("--fp64", action="store_true", help="all-FP64 GPU path")
    ap.add_argument("--with-mu-one", action="store_true",
                    help="mu = 1 in the last mu bin, as FCFC built with "
                         "-DWITH_MU_ONE")
    ap.add_argument("--no-graph", action="store_true",
                    help="one count per pair instead of one CUDA graph")
    ap.add_argument("-v", "--verbose", nargs="?", const="T", default=None)
    survey = argv is not None and "--survey" in argv or \
        argv is None and "--survey" in sys.argv[1:]
    for short, long_, key, kind in OPTIONS:
        if kind in ("survey", "survey-bool") and not survey:
            continue
        names = (["-" + short] if short else []) + ["--" + long_]
        if kind == "box-opt":
            ap.add_argument(*names, dest=key, nargs="?", const="", default=None,
                            action=_FirstValue)
        elif kind in ("bool", "survey-bool"):
            ap.add_argument(*names, dest=key, nargs="?", const="T", default=None,
                            action=_FirstValue)
        else:
            ap.add_argument(*names, dest=key, default=None, action=_FirstValue)
    a = ap.parse_args(argv)
    path = a.conf or ("fcfc_2pt.conf" if a.survey else "fcfc_2pt_box.conf")
    if os.access(path, os.R_OK):
        conf = parse_conf(open(path).read())
    else:
        print("Warning: cannot access the configuration file: `%s'" % path,
              file=sys.stderr)
        conf = {}
    for _, _, key, _ in OPTIONS:
        v = getattr(a, key, None)
        if v:
            conf.update(parse_conf("%s = %s" % (key, v)))
    verbose = a.verbose if a.verbose is not None else conf.get("VERBOSE", "T")
    run(conf, "survey" if a.survey else "box",
        precision=capi.PREC_FP64 if a.fp64 else capi.PREC_FP32_RECHECK,
        verbose=_bool(verbose), with_mu_one=a.with_mu_one,
        graph=not a.no_graph)
    return 0


if __name__ == "__main__":
    sys.exit(main())
