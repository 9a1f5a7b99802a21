"""ctypes binding of libfcfcg.so (include/fcfcg.h).

The shared library is the product: every count runs on the GPU through it.
Importing this module does not need a GPU; creating a device context does,
and fails with FCFCGError(FCFCG_ERR_CUDA) when there is none.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libfcfcg.so")

OK = 0
ERR_MEMORY, ERR_ARG, ERR_FILE, ERR_CFG = -1, -2, -3, -4
ERR_DATA, ERR_CNVT, ERR_CF, ERR_SAVE, ERR_UNKNOWN = -21, -22, -24, -25, -99
ERR_CUDA, ERR_TIMEOUT, ERR_UNSUPPORTED = -100, -101, -102
BIN_ISO, BIN_SMU, BIN_SPI = 0, 1, 2
GEOM_BOX, GEOM_SURVEY = 0, 1
PREC_FP32_RECHECK, PREC_FP64 = 0, 1
TAB_INT, TAB_HYBRID = 0, 1

_dp = C.POINTER(C.c_double)


class Binning(C.Structure):
    _fields_ = [("geometry", C.c_int), ("bintype", C.c_int),
                ("box", C.c_double * 3), ("ns", C.c_int), ("smin", C.c_double),
                ("ds", C.c_double), ("sedges", _dp), ("nmu", C.c_int),
                ("np", C.c_int), ("pmin", C.c_double), ("dpi", C.c_double),
                ("pedges", _dp), ("with_mu_one", C.c_int)]


class BinsInfo(C.Structure):
    _fields_ = [("ns", C.c_int), ("nmu", C.c_int), ("np", C.c_int),
                ("ntot", C.c_int64), ("tabtype", C.c_int),
                ("rescale", C.c_double), ("box_rescaled", C.c_double * 3),
                ("nstab", C.c_int64), ("nptab", C.c_int64),
                ("ftab_cells_per_octave", C.c_int)]


class Cosmo(C.Structure):
    """fcfcg_cosmo: OMEGA_M, OMEGA_LAMBDA, DE_EOS_W, CMVDST_ERR and the
    Z_CMVDST_FILE table of FCFC_2PT's coordinate conversion."""
    _fields_ = [("omega_m", C.c_double), ("omega_l", C.c_double),
                ("has_omega_l", C.c_int), ("dew", C.c_double),
                ("cmvdst_err", C.c_double), ("nsample", C.c_size_t),
                ("z_sample", _dp), ("d_sample", _dp)]


def make_cosmo(omega_m=0.31, omega_l=None, dew=-1.0, cmvdst_err=0.0,
               ztable=None):
    """Cosmo struct plus the arrays it points to (keep both alive).
    ztable: (z, d) rows of a Z_CMVDST_FILE, which replaces integration."""
    c = Cosmo()
    c.omega_m = float(omega_m)
    c.has_omega_l = omega_l is not None
    c.omega_l = float(omega_l) if omega_l is not None else 0.0
    c.dew = float(dew)
    c.cmvdst_err = float(cmvdst_err)
    keep = []
    if ztable is not None:
        t = np.asarray(ztable, np.float64)
        zs = np.ascontiguousarray(t[:, 0])
        ds = np.ascontiguousarray(t[:, 1])
        keep = [zs, ds]
        c.nsample = len(zs)
        c.z_sample = zs.ctypes.data_as(_dp)
        c.d_sample = ds.ctypes.data_as(_dp)
    return c, keep


class Job(C.Structure):
    """fcfcg_job: one periodic-box catalogue of a batch."""
    _fields_ = [("n", C.c_size_t), ("x", _dp), ("y", _dp), ("z", _dp),
                ("w", _dp), ("box", C.c_double * 3),
                ("icnt", C.POINTER(C.c_int64)), ("wcnt", _dp),
                ("sumw", C.c_double), ("status", C.c_int)]


class CountItem(C.Structure):
    """fcfcg_count_item: one count of a count graph."""
    _fields_ = [("slot_a", C.c_int), ("slot_b", C.c_int),
                ("isauto", C.c_int), ("withwt", C.c_int),
                ("icnt", C.POINTER(C.c_int64)), ("wcnt", _dp)]


class Stats(C.Structure):
    _fields_ = [("candidates", C.c_uint64), ("in_range", C.c_uint64),
                ("rechecked", C.c_uint64), ("recheck_inline", C.c_uint64),
                ("ms_grid", C.c_double), ("ms_count", C.c_double),
                ("ms_recheck", C.c_double), ("ms_total", C.c_double),
                ("cells_per_smax", C.c_int), ("ncell", C.c_int * 3),
                ("nstencil", C.c_int), ("nchunks", C.c_uint64),
                ("precision_used", C.c_int), ("launches", C.c_uint64),
                ("warp_queue", C.c_int)]

    def as_dict(self):
        d = {k: getattr(self, k) for k, _ in self._fields_}
        d["ncell"] = list(self.ncell)
        return d


class FCFCGError(RuntimeError):
    def __init__(self, code, msg=""):
        super().__init__("%s (%d)%s" % (strerror(code), code,
                                         (": " + msg) if msg else ""))
        self.code = code


# Every exported entry point with its prototype: (restype, argtypes).
P = C.c_void_p
PROTOTYPES = {
    "fcfcg_strerror": (C.c_char_p, [C.c_int]),
    "fcfcg_last_error": (C.c_char_p, [P]),
    "fcfcg_linear_nbin": (C.c_int, [C.c_double, C.c_double, C.c_double]),
    "fcfcg_create": (C.c_int, [C.POINTER(Binning), C.c_int, C.POINTER(P)]),
    "fcfcg_create_host": (C.c_int, [C.POINTER(Binning), C.POINTER(P)]),
    "fcfcg_destroy": (None, [P]),
    "fcfcg_bins_info_get": (C.c_int, [P, C.POINTER(BinsInfo)]),
    "fcfcg_bins_edges": (C.c_int, [P, P, P]),
    "fcfcg_bins_tables": (C.c_int, [P, P, P, P, P]),
    "fcfcg_load_catalog": (C.c_int, [P, C.c_int, C.c_size_t, P, P, P, P]),
    "fcfcg_load_catalog_device": (C.c_int, [P, C.c_int, C.c_size_t, P, P, P, P]),
    "fcfcg_adjoint": (C.c_int, [P, C.c_int, C.c_int, C.c_int, P, P, P]),
    "fcfcg_count_batch": (C.c_int, [P, C.POINTER(Job), C.c_int, C.c_int,
                                    C.c_int, C.c_int]),
    "fcfcg_autotune_batch": (C.c_int, [P, C.POINTER(Job), C.c_int, C.c_int,
                                       C.c_int, C.POINTER(C.c_int),
                                       C.POINTER(C.c_double)]),
    "fcfcg_cnvt_coord": (C.c_int, [P, C.c_size_t, P, P, P, P, P, P,
                                   C.POINTER(Cosmo), C.POINTER(C.c_int)]),
    "fcfcg_load_catalog_radecz": (C.c_int, [P, C.c_int, C.c_size_t, P, P, P, P,
                                            C.POINTER(Cosmo)]),
    "fcfcg_load_catalog_radecz_device": (C.c_int, [P, C.c_int, C.c_size_t, P, P,
                                                   P, P, C.POINTER(Cosmo)]),
    "fcfcg_catalog_info": (C.c_int, [P, C.c_int, C.POINTER(C.c_size_t),
                                     C.POINTER(C.c_double)]),
    "fcfcg_count": (C.c_int, [P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                              P, P]),
    "fcfcg_stats_get": (C.c_int, [P, C.POINTER(Stats)]),
    "fcfcg_graph_create": (C.c_int, [P, C.POINTER(CountItem), C.c_int,
                                     C.c_int, C.POINTER(P)]),
    "fcfcg_graph_run": (C.c_int, [P]),
    "fcfcg_graph_info": (C.c_int, [P, C.POINTER(C.c_int),
                                   C.POINTER(C.c_uint64)]),
    "fcfcg_graph_destroy": (None, [P]),
    "fcfcg_set_cells_per_smax": (C.c_int, [P, C.c_int]),
    "fcfcg_set_queue_capacity": (C.c_int, [P, C.c_size_t]),
    "fcfcg_set_hist_handover": (C.c_int, [P, C.c_ulonglong]),
    "fcfcg_set_warp_queue": (C.c_int, [P, C.c_int]),
    "fcfcg_probe_smem_atomics": (C.c_int, [C.c_int, C.POINTER(C.c_double)]),
    "fcfcg_autotune": (C.c_int, [P, C.c_int, C.c_int, C.c_int, C.c_int,
                                 C.POINTER(C.c_int), C.POINTER(C.c_double)]),
    "fcfcg_norm": (C.c_double, [C.c_int, C.c_int, C.c_double, C.c_double]),
    "fcfcg_analytic_rr": (C.c_int, [P, P]),
    "fcfcg_multipoles": (C.c_int, [P, P, C.c_int, P, P]),
    "fcfcg_wp": (C.c_int, [P, P, P]),
    "fcfcg_write_paircount": (C.c_int, [P, C.c_char_p, C.c_int, C.c_int,
                                        C.c_int, P, P, C.c_double, P, P, P]),
    "fcfcg_read_paircount": (C.c_int, [P, C.c_char_p, P, P, P, P, P, P, P,
                                       P]),
    "fcfcg_cf_eval": (C.c_int, [C.c_char_p, C.c_int, C.c_char_p, P, P,
                                C.c_long, P]),
    "fcfcg_count_noalloc": (C.c_int, [P, C.c_int, C.c_size_t, P, P, P,
                                      C.c_size_t, P, P, P, P, P]),
    "fcfcg_write_cf": (C.c_int, [P, C.c_char_p, P]),
    "fcfcg_write_multipoles": (C.c_int, [P, C.c_char_p, C.c_int, P, P]),
    "fcfcg_write_wp": (C.c_int, [P, C.c_char_p, P]),
}

_lib = None


def load_library(path: str | None = None):
    """Load libfcfcg.so (building it first if it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        from . import build
        build.build()
    lib = C.CDLL(path)
    for name, (res, args) in PROTOTYPES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def strerror(code: int) -> str:
    return load_library().fcfcg_strerror(code).decode()


def ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def make_binning(geometry, bintype, box=None, ns=None, smin=0.0, ds=1.0,
                 sedges=None, nmu=1, np_=0, pmin=0.0, dpi=1.0, pedges=None,
                 smax=None, pmax=None, with_mu_one=False):
    """Binning struct plus the arrays it points to (keep both alive)."""
    lib = load_library()
    keep = []
    b = Binning()
    b.geometry, b.bintype = int(geometry), int(bintype)
    bx = [0.0, 0.0, 0.0] if box is None else list(
        np.broadcast_to(np.asarray(box, float), (3,)))
    b.box = (C.c_double * 3)(*bx)
    if sedges is not None:
        se = np.ascontiguousarray(sedges, np.float64)
        keep.append(se)
        b.sedges = se.ctypes.data_as(_dp)
        b.ns = len(se) - 1
    else:
        if ns is None:
            ns = lib.fcfcg_linear_nbin(smin, smax, ds)
        b.ns, b.smin, b.ds = int(ns), float(smin), float(ds)
    b.nmu = int(nmu)
    if pedges is not None:
        pe = np.ascontiguousarray(pedges, np.float64)
        keep.append(pe)
        b.pedges = pe.ctypes.data_as(_dp)
        b.np = len(pe) - 1
    else:
        if bintype == BIN_SPI and not np_:
            np_ = lib.fcfcg_linear_nbin(pmin, pmax, dpi)
        b.np, b.pmin, b.dpi = int(np_), float(pmin), float(dpi)
    b.with_mu_one = int(bool(with_mu_one))
    return b, keep
