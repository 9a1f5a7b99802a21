"""Python front end of the GB300 pair-counting engine.

``PairCounter`` holds one binning set-up (what FCFC's cf_setup builds,
src/fcfc/2pt_box/setup_cf.c:547-848) on one GPU, takes catalogues, and counts
pairs through the C ABI exactly where FCFC calls
``count_pairs(tree1, tree2, cf, cnt, isauto, withwt)``
(src/fcfc/2pt_box/count_func.h:54-59): auto counts come back undoubled, as
count_pairs leaves them, and ``normalise`` applies eval_pairs' doubling and
norms (src/fcfc/2pt_box/eval_cf.c:117-167).

There is no CPU path: every count runs in libfcfcg.so on the device, and a
missing GPU or library raises FCFCGError.
"""
from __future__ import annotations

import ctypes as C
import weakref

import numpy as np

from . import capi
from .capi import (BIN_ISO, BIN_SMU, BIN_SPI, GEOM_BOX, GEOM_SURVEY,
                   PREC_FP32_RECHECK, PREC_FP64, FCFCGError)


def _columns(a):
    """Three contiguous FP64 host columns of an N x 3 array, or of an
    (x, y, z) tuple of columns (not copied when already contiguous FP64)."""
    if isinstance(a, (tuple, list)) and len(a) == 3:
        cols = [np.ascontiguousarray(v, np.float64) for v in a]
        if not (len(cols[0]) == len(cols[1]) == len(cols[2])):
            raise ValueError("columns of different lengths")
        return cols
    a = np.asarray(a, np.float64)
    return [np.ascontiguousarray(a[:, k]) for k in range(3)]


class PairCounter:
    """One binning set-up on one GPU.

    geometry: "box" (FCFC_2PT_BOX, periodic) or "survey" (FCFC_2PT).
    bintype: BINNING_SCHEME (0 iso, 1 (s,mu), 2 (s_perp,pi)).
    Separation bins: linear (smin, smax, ds) or ``sedges`` (ns+1 edges as
    read_bins gives them); pi bins likewise; ``nmu`` for (s, mu).
    """

    def __init__(self, geometry="box", bintype=BIN_SMU, box=None, smin=0.0,
                 smax=None, ds=None, sedges=None, nmu=1, pmin=0.0, pmax=None,
                 dpi=None, pedges=None, device=-1, host_only=False,
                 with_mu_one=False):
        lib = capi.load_library()
        self.lib = lib
        geom = GEOM_BOX if geometry in ("box", GEOM_BOX) else GEOM_SURVEY
        self.geometry = geom
        self.bintype = int(bintype)
        self._b, self._keep = capi.make_binning(
            geom, bintype, box=box, smin=smin, ds=ds if ds is not None else 1.0,
            smax=smax, sedges=sedges, nmu=nmu, pmin=pmin, pmax=pmax,
            dpi=dpi if dpi is not None else 1.0, pedges=pedges,
            with_mu_one=with_mu_one)
        h = C.c_void_p()
        if host_only:
            rc = lib.fcfcg_create_host(C.byref(self._b), C.byref(h))
        else:
            rc = lib.fcfcg_create(C.byref(self._b), int(device), C.byref(h))
        self.h = h
        if rc:
            msg = lib.fcfcg_last_error(h).decode() if h else ""
            lib.fcfcg_destroy(h)
            self.h = None
            raise FCFCGError(rc, msg)
        info = capi.BinsInfo()
        self._check(lib.fcfcg_bins_info_get(self.h, C.byref(info)))
        self.info = info
        self.ns, self.nmu, self.np, self.ntot = info.ns, info.nmu, info.np, info.ntot
        self.rescale = info.rescale
        self.box_raw = None if box is None else np.broadcast_to(
            np.asarray(box, float), (3,)).copy()
        self.sbin = np.zeros(self.ns + 1)
        self.pbin = np.zeros(self.np + 1) if self.bintype == BIN_SPI else None
        self._check(lib.fcfcg_bins_edges(self.h, capi.ptr(self.sbin),
                                         capi.ptr(self.pbin)))
        self._n = {}
        self._graphs = weakref.WeakValueDictionary()

    # -- plumbing -----------------------------------------------------------
    def _check(self, rc):
        if rc:
            msg = self.lib.fcfcg_last_error(self.h).decode() if self.h else ""
            raise FCFCGError(rc, msg)

    def close(self):
        # count graphs refer to the context: they go first
        for g in list(getattr(self, "_graphs", {}).values()):
            g.close()
        if getattr(self, "h", None):
            self.lib.fcfcg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- tables -------------------------------------------------------------
    def tables(self):
        st = np.zeros(self.info.nstab, np.uint16)
        pt = np.zeros(self.info.nptab, np.uint16)
        s2 = np.zeros(self.ns + 1)
        pb = np.zeros(self.np + 1) if self.bintype == BIN_SPI else None
        self._check(self.lib.fcfcg_bins_tables(self.h, capi.ptr(st),
                                               capi.ptr(pt), capi.ptr(s2),
                                               capi.ptr(pb)))
        return st, pt, s2, pb

    # -- catalogues ---------------------------------------------------------
    def load(self, slot: int, xyz, w=None):
        """Copy a catalogue (N x 3 FP64 host array or (x, y, z) host columns,
        coordinates as read, and optional weights) to the device slot."""
        cols = _columns(xyz)
        ww = None if w is None else np.ascontiguousarray(w, np.float64)
        self._check(self.lib.fcfcg_load_catalog(
            self.h, int(slot), len(cols[0]), *[capi.ptr(c) for c in cols],
            capi.ptr(ww)))
        self._n[slot] = (len(cols[0]), w is not None)

    def load_device(self, slot: int, x_ptr: int, y_ptr: int, z_ptr: int,
                    n: int, w_ptr: int | None = None):
        """Catalogue already on the device (FP64 pointers, e.g. from torch)."""
        self._check(self.lib.fcfcg_load_catalog_device(
            self.h, int(slot), int(n), C.c_void_p(x_ptr), C.c_void_p(y_ptr),
            C.c_void_p(z_ptr), C.c_void_p(w_ptr) if w_ptr else None))
        self._n[slot] = (int(n), w_ptr is not None)

    def load_radecz(self, slot: int, radecz, w=None, omega_m=0.31,
                    omega_l=None, dew=-1.0, cmvdst_err=0.0, ztable=None):
        """Load a catalogue given as RA, Dec (degrees) and redshift (N x 3
        host array, or three host columns), converted to comoving
        coordinates on the device as
        FCFC_2PT's COORD_CONVERT does: Gauss-Legendre integration in the given
        cosmology, or the spline through ``ztable`` rows (z, d)."""
        cols = _columns(radecz)
        ww = None if w is None else np.ascontiguousarray(w, np.float64)
        cs, keep = capi.make_cosmo(omega_m, omega_l, dew, cmvdst_err, ztable)
        self._check(self.lib.fcfcg_load_catalog_radecz(
            self.h, int(slot), len(cols[0]), *[capi.ptr(c) for c in cols],
            capi.ptr(ww), C.byref(cs)))
        del keep
        self._n[slot] = (len(cols[0]), w is not None)

    def load_radecz_device(self, slot: int, ra_ptr: int, dec_ptr: int,
                           z_ptr: int, n: int, w_ptr: int | None = None,
                           omega_m=0.31, omega_l=None, dew=-1.0,
                           cmvdst_err=0.0, ztable=None):
        """load_radecz from device FP64 arrays (the inputs are not changed)."""
        cs, keep = capi.make_cosmo(omega_m, omega_l, dew, cmvdst_err, ztable)
        vp = C.c_void_p
        self._check(self.lib.fcfcg_load_catalog_radecz_device(
            self.h, int(slot), int(n), vp(ra_ptr), vp(dec_ptr), vp(z_ptr),
            vp(w_ptr) if w_ptr else None, C.byref(cs)))
        del keep
        self._n[slot] = (int(n), w_ptr is not None)

    def convert_device(self, n: int, ra_ptr: int, dec_ptr: int, z_ptr: int,
                       x_ptr: int, y_ptr: int, zc_ptr: int, omega_m=0.31,
                       omega_l=None, dew=-1.0, cmvdst_err=0.0, ztable=None):
        """fcfcg_cnvt_coord on device arrays; returns the Gauss-Legendre order
        (0 for the spline)."""
        cs, keep = capi.make_cosmo(omega_m, omega_l, dew, cmvdst_err, ztable)
        order = C.c_int()
        vp = C.c_void_p
        self._check(self.lib.fcfcg_cnvt_coord(
            self.h, int(n), vp(ra_ptr), vp(dec_ptr), vp(z_ptr), vp(x_ptr),
            vp(y_ptr), vp(zc_ptr), C.byref(cs), C.byref(order)))
        del keep
        return order.value

    def catalog_info(self, slot: int):
        n = C.c_size_t()
        sw = C.c_double()
        self._check(self.lib.fcfcg_catalog_info(self.h, int(slot), C.byref(n),
                                                C.byref(sw)))
        return n.value, sw.value

    def set_cells_per_smax(self, k: int):
        self._check(self.lib.fcfcg_set_cells_per_smax(self.h, int(k)))

    def set_warp_queue(self, entries: int):
        """Entries of the FP32 kernel's per-warp candidate queue (256, 512,
        1024; 0 automatic)."""
        self._check(self.lib.fcfcg_set_warp_queue(self.h, int(entries)))

    def set_hist_handover(self, pairs: int):
        """Hand-over threshold of the FP32 kernel's unweighted shared
        histogram (1..2^32 - 1; 0 default); the counts do not change."""
        self._check(self.lib.fcfcg_set_hist_handover(self.h, int(pairs)))

    def set_queue_capacity(self, cap: int):
        """Limit the FP64 recheck queue (pairs beyond are binned inside the
        counting kernel; the counts do not change)."""
        self._check(self.lib.fcfcg_set_queue_capacity(self.h, int(cap)))

    def autotune(self, a: int, b: int | None = None, weighted=False):
        """Time the FP32 count at 1..8 cells per maximum separation, then
        the warp queue sizes at the fastest, and keep both for catalogues of
        this density; returns (k, ms)."""
        isauto = b is None or b == a
        k = C.c_int()
        ms = C.c_double()
        self._check(self.lib.fcfcg_autotune(self.h, a, a if b is None else b,
                                            int(isauto), int(bool(weighted)),
                                            C.byref(k), C.byref(ms)))
        return k.value, ms.value

    # -- counting -----------------------------------------------------------
    def count_pairs(self, a: int, b: int | None = None, weighted=False,
                    precision=PREC_FP32_RECHECK, out=None):
        """count_pairs: unordered pairs once for auto (b None or == a)."""
        isauto = b is None or b == a
        b = a if b is None else b
        if weighted:
            res = out if out is not None else np.zeros(self.ntot, np.float64)
            self._check(self.lib.fcfcg_count(self.h, a, b, int(isauto), 1,
                                             int(precision), None,
                                             capi.ptr(res)))
        else:
            res = out if out is not None else np.zeros(self.ntot, np.int64)
            self._check(self.lib.fcfcg_count(self.h, a, b, int(isauto), 0,
                                             int(precision), capi.ptr(res),
                                             None))
        return res

    def count_graph(self, pairs, precision=PREC_FP32_RECHECK):
        """Capture counts as one CUDA graph (fcfcg_graph_create).  pairs:
        (a, b, weighted) per count, b None or == a for an auto count; e.g.
        DD, DR, RR of a survey.  Returns a CountGraph whose run() replays
        them and returns the histograms, the same as count_pairs."""
        return CountGraph(self, pairs, precision)

    # -- batches of periodic boxes -----------------------------------------
    def _jobs(self, cats, boxes, weights, weighted, on_device):
        n = len(cats)
        jobs = (capi.Job * max(n, 1))()
        keep = []
        outs = []
        for j in range(n):
            J = jobs[j]
            b = np.broadcast_to(np.asarray(boxes[j], np.float64), (3,))
            for k in range(3):
                J.box[k] = float(b[k])
            if on_device:
                x, y, z = cats[j][:3]
                J.n = int(cats[j][3])
                J.x, J.y, J.z = (C.cast(C.c_void_p(p), capi._dp) for p in (x, y, z))
                if weighted:
                    J.w = C.cast(C.c_void_p(weights[j]), capi._dp)
            else:
                cols = _columns(cats[j])
                keep += cols
                J.n = len(cols[0])
                J.x, J.y, J.z = (c.ctypes.data_as(capi._dp) for c in cols)
                if weighted:
                    w = np.ascontiguousarray(weights[j], np.float64)
                    keep.append(w)
                    J.w = w.ctypes.data_as(capi._dp)
            if weighted:
                o = np.zeros(self.ntot)
                J.wcnt = o.ctypes.data_as(capi._dp)
            else:
                o = np.zeros(self.ntot, np.int64)
                J.icnt = o.ctypes.data_as(C.POINTER(C.c_int64))
            outs.append(o)
        return jobs, keep, outs

    def count_batch(self, cats, boxes, weights=None, weighted=False,
                    precision=PREC_FP32_RECHECK, on_device=False):
        """DD counts (undoubled) of many periodic boxes in one launch.

        cats: N_j x 3 host arrays or (x, y, z) host column arrays, or with
        on_device (x_ptr, y_ptr, z_ptr, n) tuples of device FP64 pointers;
        boxes: BOX_SIZE per catalogue;
        weights: per-catalogue arrays (device pointers with on_device).
        Returns (counts, status, sumw) lists."""
        jobs, keep, outs = self._jobs(cats, boxes, weights, weighted, on_device)
        self._check(self.lib.fcfcg_count_batch(self.h, jobs, len(cats),
                                               int(bool(weighted)),
                                               int(precision), int(bool(on_device))))
        del keep
        return (outs, [jobs[j].status for j in range(len(cats))],
                [jobs[j].sumw for j in range(len(cats))])

    def autotune_batch(self, cats, boxes, weights=None, weighted=False,
                       on_device=False):
        jobs, keep, outs = self._jobs(cats, boxes, weights, weighted, on_device)
        k = C.c_int()
        ms = C.c_double()
        self._check(self.lib.fcfcg_autotune_batch(
            self.h, jobs, len(cats), int(bool(weighted)), int(bool(on_device)),
            C.byref(k), C.byref(ms)))
        del keep, outs
        return k.value, ms.value

    def adjoint(self, a: int, b: int | None, g):
        """Gradient of sum_k g_k C_k (C: the weighted count of slots a, b as
        count_pairs(weighted=True) returns it) with respect to the weights of
        slot a (and of slot b for a cross count): (dw_a, dw_b or None)."""
        isauto = b is None or b == a
        g = np.ascontiguousarray(g, np.float64)
        if g.shape != (self.ntot,):
            raise ValueError("g needs %d entries" % self.ntot)
        na = self._n.get(a, (0, False))[0]
        dwa = np.zeros(na)
        dwb = None
        if not isauto:
            dwb = np.zeros(self._n.get(b, (0, False))[0])
        self._check(self.lib.fcfcg_adjoint(self.h, a, a if isauto else b,
                                           int(isauto), capi.ptr(g),
                                           capi.ptr(dwa), capi.ptr(dwb)))
        return dwa, dwb

    def stats(self) -> dict:
        s = capi.Stats()
        self._check(self.lib.fcfcg_stats_get(self.h, C.byref(s)))
        return s.as_dict()

    # -- post-processing (eval_cf.c) ---------------------------------------
    def normalise(self, cnt, isauto, weighted, n1, n2=None):
        """eval_pairs: auto counts doubled; returns (cnt, norm, ncnt)."""
        cnt = np.asarray(cnt)
        if isauto:
            cnt = cnt * 2
        norm = self.lib.fcfcg_norm(int(isauto), int(weighted), float(n1),
                                   float(n2 if n2 is not None else 0.0))
        return cnt, norm, cnt / norm

    def analytic_rr(self):
        rr = np.zeros(self.ntot)
        self._check(self.lib.fcfcg_analytic_rr(self.h, capi.ptr(rr)))
        return rr

    def multipoles(self, xi, poles):
        xi = np.ascontiguousarray(xi, np.float64)
        pl = np.ascontiguousarray(poles, np.int32)
        mp = np.zeros(len(pl) * self.ns)
        self._check(self.lib.fcfcg_multipoles(self.h, capi.ptr(xi), len(pl),
                                              capi.ptr(pl), capi.ptr(mp)))
        return mp.reshape(len(pl), self.ns)

    def wp(self, xi):
        xi = np.ascontiguousarray(xi, np.float64)
        out = np.zeros(self.ns)
        self._check(self.lib.fcfcg_wp(self.h, capi.ptr(xi), capi.ptr(out)))
        return out

    # -- files (save_res.c / read_res.c) ------------------------------------
    def write_paircount(self, fname, ofmt, isauto, weighted, ntr, wtr, norm,
                        ncnt, cnt):
        nt = np.zeros(2, np.uint64)
        nt[:len(ntr)] = ntr
        wt = np.zeros(2, np.float64)
        if wtr is not None:
            wt[:len(wtr)] = wtr
        ncnt = np.ascontiguousarray(ncnt, np.float64)
        ic = None if weighted else np.ascontiguousarray(cnt, np.int64)
        wc = np.ascontiguousarray(cnt, np.float64) if weighted else None
        self._check(self.lib.fcfcg_write_paircount(
            self.h, fname.encode(), int(ofmt), int(isauto), int(weighted),
            capi.ptr(nt), capi.ptr(wt), float(norm), capi.ptr(ncnt),
            capi.ptr(ic), capi.ptr(wc)))

    def read_paircount(self, fname):
        au, wt = C.c_int(), C.c_int()
        nt = np.zeros(2, np.uint64)
        wtr = np.zeros(2)
        norm = C.c_double()
        ncnt = np.zeros(self.ntot)
        ic = np.zeros(self.ntot, np.int64)
        wc = np.zeros(self.ntot)
        self._check(self.lib.fcfcg_read_paircount(
            self.h, fname.encode(), C.byref(au), C.byref(wt), capi.ptr(nt),
            capi.ptr(wtr), C.byref(norm), capi.ptr(ncnt), capi.ptr(ic),
            capi.ptr(wc)))
        return dict(auto=bool(au.value), weighted=bool(wt.value), ntr=nt,
                    wtr=wtr, norm=norm.value, ncnt=ncnt,
                    cnt=wc if wt.value else ic)

    def write_cf(self, fname, xi):
        xi = np.ascontiguousarray(xi, np.float64)
        self._check(self.lib.fcfcg_write_cf(self.h, fname.encode(), capi.ptr(xi)))

    def write_multipoles(self, fname, poles, mp):
        pl = np.ascontiguousarray(poles, np.int32)
        mp = np.ascontiguousarray(mp, np.float64).ravel()
        self._check(self.lib.fcfcg_write_multipoles(
            self.h, fname.encode(), len(pl), capi.ptr(pl), capi.ptr(mp)))

    def write_wp(self, fname, wp):
        wp = np.ascontiguousarray(wp, np.float64)
        self._check(self.lib.fcfcg_write_wp(self.h, fname.encode(), capi.ptr(wp)))


class CountGraph:
    """Counts of one PairCounter captured as a CUDA graph; run() replays it
    (the catalogues are read when it runs) and returns one histogram per
    count: int64 counts, or FP64 weighted sums."""

    def __init__(self, pc: PairCounter, pairs, precision=PREC_FP32_RECHECK):
        self.pc = pc
        n = len(pairs)
        items = (capi.CountItem * n)()
        self.out = []
        for i, (a, b, weighted) in enumerate(pairs):
            isauto = b is None or b == a
            b = a if b is None else b
            it = items[i]
            it.slot_a, it.slot_b = int(a), int(b)
            it.isauto, it.withwt = int(isauto), int(bool(weighted))
            if weighted:
                res = np.zeros(pc.ntot, np.float64)
                it.wcnt = res.ctypes.data_as(C.POINTER(C.c_double))
            else:
                res = np.zeros(pc.ntot, np.int64)
                it.icnt = res.ctypes.data_as(C.POINTER(C.c_int64))
            self.out.append(res)
        self._items = items
        self.h = None
        h = C.c_void_p()
        pc._check(pc.lib.fcfcg_graph_create(pc.h, items, n, int(precision),
                                            C.byref(h)))
        self.h = h
        pc._graphs[id(self)] = self

    def run(self):
        self.pc._check(self.pc.lib.fcfcg_graph_run(self.h))
        return [r.copy() for r in self.out]

    def info(self):
        """(times captured, kernel launches per run)."""
        n = C.c_int()
        k = C.c_uint64()
        self.pc._check(self.pc.lib.fcfcg_graph_info(self.h, C.byref(n),
                                                    C.byref(k)))
        return n.value, k.value

    def close(self):
        if self.h and self.pc.h:
            self.pc.lib.fcfcg_graph_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
