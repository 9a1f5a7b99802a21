"""Reader for FCFC pair-count files (binary OUTPUT_FORMAT = 0 and ASCII = 1).

Binary layout (FCFC v1.0.1 save_res_bin, src/fcfc/2pt_box/save_res.c:177-310):
a text header line, then records each framed by the same uint64 byte count
before and after:
  spec      int32[7|8]  precision, mu=1, periodic, auto/cross, weighted,
                        binning scheme, ns, (nmu | np)
  box       double[3]   rescaled box sides   (periodic files only)
  sbin      double[ns+1]
  pbin      double[np+1]                      ((s_perp, pi) only)
  tracers   auto: double sum(w) | uint64 n;  cross: double[2] | uint64[2]
  norm      double
  ncnt      double[ntot]   normalised counts
  cnt       int64[ntot] | double[ntot]   raw (doubled for auto) counts
"""
from __future__ import annotations

import struct
from dataclasses import dataclass

import numpy as np


@dataclass
class PairCountFile:
    header: str
    single_prec: bool
    mu_one: bool
    periodic: bool
    auto: bool
    weighted: bool
    bintype: int
    ns: int
    n2: int
    box: np.ndarray | None
    sbin: np.ndarray
    pbin: np.ndarray | None
    tracers: np.ndarray
    norm: float
    ncnt: np.ndarray
    cnt: np.ndarray


def _records(data: bytes, pos: int):
    out = []
    while pos < len(data):
        (n,) = struct.unpack_from("<Q", data, pos)
        body = data[pos + 8: pos + 8 + n]
        (n2,) = struct.unpack_from("<Q", data, pos + 8 + n)
        if n2 != n:
            raise ValueError("corrupted record framing")
        out.append(body)
        pos += 16 + n
    return out


def read_binary(path: str) -> PairCountFile:
    data = open(path, "rb").read()
    nl = data.index(b"\n") + 1
    header = data[:nl].decode()
    recs = _records(data, nl)
    spec = np.frombuffer(recs[0], np.int32)
    bintype = int(spec[5])
    # box sizes and bin edges are `real`: float in a SINGLE_PREC build
    real = np.float32 if spec[0] == 0 else np.float64
    k = 1
    box = None
    if spec[2]:
        box = np.frombuffer(recs[k], real).astype(np.float64)
        k += 1
    sbin = np.frombuffer(recs[k], real).astype(np.float64)
    k += 1
    pbin = None
    if bintype == 2:
        pbin = np.frombuffer(recs[k], real).astype(np.float64)
        k += 1
    weighted = bool(spec[4])
    tr = np.frombuffer(recs[k], np.float64 if weighted else np.uint64).copy()
    k += 1
    (norm,) = struct.unpack("<d", recs[k])
    k += 1
    ncnt = np.frombuffer(recs[k], np.float64).copy()
    k += 1
    cnt = np.frombuffer(recs[k], np.float64 if weighted else np.int64).copy()
    return PairCountFile(header, spec[0] == 0, bool(spec[1]), bool(spec[2]),
                         spec[3] == 0, weighted, bintype, int(spec[6]),
                         int(spec[7]) if len(spec) > 7 else 1, box, sbin, pbin,
                         tr, norm, ncnt, cnt)
