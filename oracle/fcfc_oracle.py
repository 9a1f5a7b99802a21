"""ctypes front end of the FCFC oracle (oracle/fcfc_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by the smoke check and by the
CPU-baseline leg of bench.py.  The product (fcfc_gb300/) never imports it.

The oracle restates FCFC's binning set-up and per-pair formulas in plain C
(see the header of fcfc_oracle.c for the file:line of every part it
follows); tests/test_oracle_golden.py pins it against pair-count files written
by the upstream executables.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SRC = os.path.join(_HERE, "fcfc_oracle.c")
_LIBDIR = os.path.join(_HERE, "lib")
_LIB = os.path.join(_LIBDIR, "libfcfc_oracle.so")
_DEPS = [_SRC, os.path.join(os.path.dirname(_HERE), "fcfc_gb300", "csrc",
                            "legauss_tab.h")]

BIN_ISO, BIN_SMU, BIN_SPI = 0, 1, 2


def build(force: bool = False) -> str:
    """Compile the oracle into oracle/lib/ (gcc, OpenMP, no FMA contraction)."""
    if not force and os.path.exists(_LIB) and \
            all(os.path.getmtime(_LIB) >= os.path.getmtime(d) for d in _DEPS):
        return _LIB
    os.makedirs(_LIBDIR, exist_ok=True)
    tmp = _LIB + ".tmp%d" % os.getpid()
    subprocess.check_call(["gcc", "-O3", "-std=c99", "-ffp-contract=off",
                           "-fno-fast-math", "-fopenmp", "-shared", "-fPIC",
                           "-o", tmp, _SRC, "-lm"])
    os.replace(tmp, _LIB)
    return _LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(build())
        L = _lib
        P = C.c_void_p
        D = C.c_double
        dp = C.POINTER(C.c_double)
        L.fco_bins_new.restype = P
        L.fco_bins_new.argtypes = [C.c_int, C.c_int, C.c_int, D, D, C.c_int, dp,
                                   C.c_int, C.c_int, D, D, C.c_int, dp, dp]
        L.fco_bins_free.argtypes = [P]
        L.fco_bins_set_mu_one.argtypes = [P, C.c_int]
        L.fco_bins_rescale.restype = D
        L.fco_bins_rescale.argtypes = [P]
        for f in ("fco_bins_tabtype",):
            getattr(L, f).restype = C.c_int
            getattr(L, f).argtypes = [P]
        for f in ("fco_bins_ntot", "fco_bins_nstab", "fco_bins_nptab"):
            getattr(L, f).restype = C.c_long
            getattr(L, f).argtypes = [P]
        L.fco_bins_tables.argtypes = [P, P, P, P, P]
        L.fco_bins_box.argtypes = [P, P]
        L.fco_count.restype = C.c_int
        L.fco_count.argtypes = [P, C.c_size_t, P, P, P, P, C.c_size_t, P, P, P, P,
                                C.c_int, C.c_int, C.c_int, C.c_int, P, P]
        L.fco_adjoint.restype = C.c_int
        L.fco_adjoint.argtypes = [P, C.c_size_t, P, P, P, P, C.c_size_t, P, P,
                                  P, P, C.c_int, P, P, P]
        L.fco_cnvt_order.restype = C.c_int
        L.fco_cnvt_order.argtypes = [D, D, D, D, D, C.c_size_t, P]
        L.fco_cnvt_integr.argtypes = [D, D, D, D, C.c_int, C.c_size_t, P, P, P,
                                      P, P, P]
        L.fco_cnvt_spline.restype = C.c_size_t
        L.fco_cnvt_spline.argtypes = [C.c_size_t, P, P, C.c_size_t, P, P, P, P,
                                      P, P]
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _dptr(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_double))


class Bins:
    """Reference bin set-up: rescale factor, edges and lookup tables.

    ``sedges``/``pedges`` (ns+1 / np+1 raw edges) select file-defined bins;
    otherwise linear bins come from (smin, ds, ns) / (pmin, dpi, np).
    """

    def __init__(self, survey: bool, bintype: int, ns: int, smin=0.0, ds=1.0,
                 sedges=None, nmu=1, np_=0, pmin=0.0, dpi=1.0, pedges=None,
                 box=None, with_mu_one=False):
        L = lib()
        self._keep = []
        se = None if sedges is None else np.ascontiguousarray(sedges, np.float64)
        pe = None if pedges is None else np.ascontiguousarray(pedges, np.float64)
        bx = None if box is None else np.ascontiguousarray(
            np.broadcast_to(np.asarray(box, np.float64), (3,)))
        self._keep += [se, pe, bx]
        self.survey, self.bintype = bool(survey), int(bintype)
        self.ns, self.nmu, self.np = int(ns), int(nmu), int(np_)
        h = L.fco_bins_new(int(survey), int(bintype), int(se is None),
                           float(smin), float(ds), int(ns), _dptr(se), int(nmu),
                           int(pe is None), float(pmin), float(dpi), int(np_),
                           _dptr(pe), _dptr(bx))
        if not h:
            raise ValueError("oracle bin set-up failed")
        self.h = h
        L.fco_bins_set_mu_one(h, int(bool(with_mu_one)))

    def __del__(self):
        h = getattr(self, "h", None)
        if h and _lib is not None:
            _lib.fco_bins_free(h)
            self.h = None

    @property
    def rescale(self) -> float:
        return lib().fco_bins_rescale(self.h)

    @property
    def tabtype(self) -> int:
        return lib().fco_bins_tabtype(self.h)

    @property
    def ntot(self) -> int:
        return lib().fco_bins_ntot(self.h)

    def tables(self):
        L = lib()
        st = np.zeros(L.fco_bins_nstab(self.h), np.uint16)
        pt = np.zeros(max(L.fco_bins_nptab(self.h), 0), np.uint16)
        s2 = np.zeros(self.ns + 1)
        p = np.zeros(self.np + 1) if self.bintype == BIN_SPI else None
        L.fco_bins_tables(self.h, _ptr(st), _ptr(pt), _ptr(s2), _ptr(p))
        return st, pt, s2, p

    def box(self):
        out = np.zeros(3)
        lib().fco_bins_box(self.h, _ptr(out))
        return out

    def count(self, a, b=None, wa=None, wb=None, weighted=None, mode=0,
              nthread=0):
        """Pair counts of catalogue ``a`` (N x 3) with ``b`` (auto if None).

        Returns int64 counts (unweighted) or float64 sums (weighted), flat,
        index s + ns * (mu or pi); auto counts are unordered pairs (undoubled).
        """
        isauto = b is None
        a = np.ascontiguousarray(a, np.float64)
        cols_a = [np.ascontiguousarray(a[:, k]) for k in range(3)]
        wa_ = None if wa is None else np.ascontiguousarray(wa, np.float64)
        if weighted is None:
            weighted = (wa is not None) or (wb is not None)
        if isauto:
            cols_b, wb_, nb = [None] * 3, None, 0
        else:
            b = np.ascontiguousarray(b, np.float64)
            cols_b = [np.ascontiguousarray(b[:, k]) for k in range(3)]
            wb_ = None if wb is None else np.ascontiguousarray(wb, np.float64)
            nb = len(b)
        ntot = self.ntot
        icnt = np.zeros(ntot, np.int64)
        wcnt = np.zeros(ntot, np.float64)
        rc = lib().fco_count(self.h, len(a), *[_ptr(c) for c in cols_a], _ptr(wa_),
                             nb, *[_ptr(c) for c in cols_b], _ptr(wb_),
                             int(isauto), int(bool(weighted)), int(mode),
                             int(nthread), _ptr(icnt), _ptr(wcnt))
        if rc:
            raise MemoryError("oracle count failed")
        return wcnt if weighted else icnt

    def adjoint(self, a, g, b=None, wa=None, wb=None):
        """Gradient of sum_b g_b C_b over the weights, C the weighted count
        (brute force, FP64): (dwa, dwb); dwb is None for auto counts."""
        isauto = b is None
        a = np.ascontiguousarray(a, np.float64)
        cols_a = [np.ascontiguousarray(a[:, k]) for k in range(3)]
        wa_ = None if wa is None else np.ascontiguousarray(wa, np.float64)
        g = np.ascontiguousarray(g, np.float64)
        dwa = np.zeros(len(a))
        dwb = None
        if isauto:
            cols_b, wb_, nb = [None] * 3, None, 0
        else:
            b = np.ascontiguousarray(b, np.float64)
            cols_b = [np.ascontiguousarray(b[:, k]) for k in range(3)]
            wb_ = None if wb is None else np.ascontiguousarray(wb, np.float64)
            nb = len(b)
            dwb = np.zeros(nb)
        rc = lib().fco_adjoint(self.h, len(a), *[_ptr(c) for c in cols_a],
                               _ptr(wa_), nb, *[_ptr(c) for c in cols_b],
                               _ptr(wb_), int(isauto), _ptr(g), _ptr(dwa),
                               _ptr(dwb))
        if rc:
            raise MemoryError("oracle adjoint failed")
        return dwa, dwb


def cosmo_params(omega_m, omega_l=None, dew=-1.0):
    """(Omega_m, Omega_Lambda, Omega_k, widx) as check_cosmo and cnvt_coord
    derive them (src/fcfc/2pt/load_conf.c:700-735, cnvt_coord.c:416)."""
    if omega_l is None:
        ol, ok = 1.0 - omega_m, 0.0
    else:
        ol, ok = float(omega_l), 1.0 - omega_m - omega_l
    widx = 0.0 if dew == -1 else 3 * (1 + dew)
    return float(omega_m), ol, ok, widx


def convert_integr(radecz, omega_m, omega_l=None, dew=-1.0, err=1e-8):
    """FCFC's COORD_CONVERT by Gauss-Legendre integration: (xyz, order)."""
    a = np.ascontiguousarray(radecz, np.float64)
    cols = [np.ascontiguousarray(a[:, k]) for k in range(3)]
    p = cosmo_params(omega_m, omega_l, dew)
    L = lib()
    order = L.fco_cnvt_order(*p, float(err), len(a), _ptr(cols[2]))
    if order < 0:
        raise ValueError("integration does not converge")
    out = [np.empty(len(a)) for _ in range(3)]
    L.fco_cnvt_integr(*p, order, len(a), *[_ptr(c) for c in cols],
                      *[_ptr(o) for o in out])
    return np.stack(out, axis=1), order


def convert_spline(radecz, zs, ds):
    """FCFC's COORD_CONVERT through Z_CMVDST_FILE: the table is sorted stably
    by z first (read_sample's timsort); returns (xyz, n_outside)."""
    zs = np.asarray(zs, np.float64)
    ds = np.asarray(ds, np.float64)
    o = np.argsort(zs, kind="stable")
    zs = np.ascontiguousarray(zs[o])
    ds = np.ascontiguousarray(ds[o])
    a = np.ascontiguousarray(radecz, np.float64)
    cols = [np.ascontiguousarray(a[:, k]) for k in range(3)]
    out = [np.empty(len(a)) for _ in range(3)]
    bad = lib().fco_cnvt_spline(len(zs), _ptr(zs), _ptr(ds), len(a),
                                *[_ptr(c) for c in cols], *[_ptr(x) for x in out])
    return np.stack(out, axis=1), int(bad)
