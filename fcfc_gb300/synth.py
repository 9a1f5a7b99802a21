"""Seeded synthetic catalogues with the shapes of FCFC's usual workloads.

* ``uniform_box``      -- Poisson points in a periodic box.
* ``neyman_scott``     -- clustered box: uniform parent centres, Poisson(mean)
                          children per parent offset by an isotropic Gaussian,
                          wrapped periodically.
* ``mock_boxes``       -- many Neyman-Scott boxes of log-uniform size at a
                          fixed number density (the batched-mock workload).
* ``survey_radecz``    -- RA uniform in a range, sin(Dec) uniform, redshift
                          from a truncated normal.
* ``radecz_to_xyz``    -- comoving Cartesian coordinates, flat LCDM.
* ``fkp_weights``      -- 1 / (1 + n(z) P0) with n(z) from the redshift
                          histogram of the sample in comoving shells.
* ``catalogue``        -- one of the above from a JSON-able spec, with the
                          sha256 of its bytes (``catalogue_sha256``): the
                          full-size fixtures name their catalogues this way.

Everything is numpy only and deterministic for a given seed.  The same seed
gives the same bytes on x86-64 and aarch64: the generators use numpy's bit
stream, its uniform / normal / Poisson / lognormal samplers (whose streams do
not depend on the platform) and IEEE-exact arithmetic.  Where a value passes
through a vectorised transcendental function (numpy's ufuncs use different
SIMD implementations per platform, which differ in the last bit), the value
is rounded to float32 afterwards, so an ulp of difference is absorbed.
"""
from __future__ import annotations

import hashlib

import numpy as np

C_KMS = 299792.458


def uniform_box(n: int, box, seed: int = 0, dtype=np.float64) -> np.ndarray:
    rng = np.random.default_rng(seed)
    box = np.broadcast_to(np.asarray(box, np.float64), (3,))
    x = rng.random((n, 3)) * box
    x = np.minimum(x, np.nextafter(box, 0))
    return x.astype(dtype).astype(np.float64)


def neyman_scott(nparent: int, box, mean_children: float = 100.0,
                 sigma: float = 5.0, seed: int = 0,
                 float32: bool = False) -> np.ndarray:
    """Neyman-Scott process in a periodic box; ``float32`` rounds the
    coordinates to float32 (kept as float64 values)."""
    rng = np.random.default_rng(seed)
    box = np.broadcast_to(np.asarray(box, np.float64), (3,))
    centres = rng.random((nparent, 3)) * box
    nchild = rng.poisson(mean_children, nparent)
    pos = np.repeat(centres, nchild, axis=0)
    pos += rng.normal(0.0, sigma, pos.shape)
    pos = np.mod(pos, box)
    if float32:
        pos = pos.astype(np.float32).astype(np.float64)
    pos = np.where(pos >= box, 0.0, pos)
    return pos


def lognormal_weights(n: int, sigma: float = 0.3, seed: int = 1) -> np.ndarray:
    return np.random.default_rng(seed).lognormal(0.0, sigma, n)


def mock_boxes(nmock: int = 256, seed: int = 7, density: float = 2.5e-4,
               nmin: float = 1e4, nmax: float = 1e6, first: int = 0,
               sizes_only: bool = False):
    """Neyman-Scott boxes (Poisson(100) children, sigma = 5 Mpc/h), N
    log-uniform in [nmin, nmax], box side (N / density)^(1/3) rounded to
    float32.  Mocks ``first`` .. ``nmock - 1``: ([catalogues], [box sides]),
    or with ``sizes_only`` ([parents], [box sides]) without generating the
    points."""
    rng = np.random.default_rng(seed)
    u = rng.uniform(np.log(nmin), np.log(nmax), nmock)
    cats, boxes = [], []
    for j in range(first, nmock):
        n = float(np.exp(u[j]))
        L = float(np.float32((n / density) ** (1.0 / 3.0)))
        npar = max(1, int(round(n / 100)))
        cats.append(npar if sizes_only else
                    neyman_scott(npar, L, 100.0, 5.0, seed=seed * 100003 + j))
        boxes.append(L)
    return cats, boxes


def comoving_distance(z, omega_m: float = 0.31, npt: int = 4096):
    """Flat LCDM comoving distance in Mpc/h (trapezoid on a fine grid)."""
    z = np.asarray(z, np.float64)
    zmax = float(np.max(z)) if z.size else 0.0
    zz = np.linspace(0.0, max(zmax, 1e-6), npt)
    a = 1 + zz
    ez = np.sqrt(omega_m * (a * a * a) + (1 - omega_m))
    integ = np.concatenate([[0.0], np.cumsum(0.5 * (1 / ez[1:] + 1 / ez[:-1])
                                             * np.diff(zz))])
    return np.interp(z, zz, integ) * C_KMS / 100.0


def survey_radecz(n: int, ra=(100.0, 260.0), dec=(0.0, 60.0), zmu=0.55,
                  zsig=0.10, zr=(0.4, 0.7), seed: int = 0) -> np.ndarray:
    """(RA, Dec, z) rows; Dec = arcsin(u) is rounded to float32."""
    rng = np.random.default_rng(seed)
    r = rng.uniform(ra[0], ra[1], n)
    s0, s1 = np.sin(np.radians(dec[0])), np.sin(np.radians(dec[1]))
    d = np.degrees(np.arcsin(rng.uniform(s0, s1, n)))
    d = d.astype(np.float32).astype(np.float64)
    z = np.empty(0)
    while z.size < n:
        t = rng.normal(zmu, zsig, 2 * n)
        z = np.concatenate([z, t[(t >= zr[0]) & (t <= zr[1])]])
    return np.stack([r, d, z[:n]], axis=1)


def radecz_to_xyz(rdz: np.ndarray, omega_m: float = 0.31) -> np.ndarray:
    ra, dec = np.radians(rdz[:, 0]), np.radians(rdz[:, 1])
    dist = comoving_distance(rdz[:, 2], omega_m)
    return np.stack([dist * np.cos(dec) * np.cos(ra),
                     dist * np.cos(dec) * np.sin(ra),
                     dist * np.sin(dec)], axis=1)


def fkp_weights(rdz: np.ndarray, p0: float = 1e4, omega_m: float = 0.31,
                dz: float = 0.01, sky_fraction: float | None = None,
                ra=(100.0, 260.0), dec=(0.0, 60.0), at=None) -> np.ndarray:
    """FKP weights with n(z) from the redshift histogram of ``rdz``,
    evaluated at the redshifts of ``at`` (default ``rdz`` itself: randoms
    take the data's n(z)); rounded to float32."""
    z = rdz[:, 2]
    if sky_fraction is None:
        area = np.radians(ra[1] - ra[0]) * (np.sin(np.radians(dec[1])) -
                                            np.sin(np.radians(dec[0])))
        sky_fraction = area / (4 * np.pi)
    edges = np.arange(z.min(), z.max() + dz, dz)
    if edges.size < 2:
        edges = np.array([z.min(), z.max() + dz])
    cnt, _ = np.histogram(z, edges)
    rr = comoving_distance(edges, omega_m)
    r3 = rr * rr * rr
    vol = sky_fraction * 4 * np.pi / 3 * (r3[1:] - r3[:-1])
    nz = cnt / np.maximum(vol, 1e-300)
    za = z if at is None else at[:, 2]
    idx = np.clip(np.searchsorted(edges, za, side="right") - 1, 0, cnt.size - 1)
    w = 1.0 / (1.0 + nz[idx] * p0)
    return w.astype(np.float32).astype(np.float64)


# --------------------------------------------------------------------------
# Catalogues named by a spec (the full-size fixtures).

def catalogue(spec: dict) -> np.ndarray:
    """The catalogue a spec names, N x 3 (x y z, or RA Dec z) or N x 4 (with
    weights).  Spec keys: ``gen`` (uniform_box | neyman_scott | mock |
    survey) and that generator's arguments; ``weights``: a lognormal sigma
    with ``wseed`` (boxes) or "fkp" (survey; ``fkp_of``: the spec of the
    catalogue whose n(z) they use, default this one)."""
    g = spec["gen"]
    if g == "uniform_box":
        x = uniform_box(spec["n"], spec["box"], seed=spec["seed"])
    elif g == "neyman_scott":
        x = neyman_scott(spec["nparent"], spec["box"], spec.get("mean", 100.0),
                         spec.get("sigma", 5.0), seed=spec["seed"],
                         float32=spec.get("float32", False))
    elif g == "mock":
        cats, _ = mock_boxes(spec["index"] + 1, seed=spec["seed"],
                             first=spec["index"])
        x = cats[0]
    elif g == "survey":
        x = survey_radecz(spec["n"], seed=spec["seed"])
    else:
        raise ValueError("unknown generator %r" % g)
    w = spec.get("weights")
    if w is None:
        return x
    if w == "fkp":
        src = catalogue(spec["fkp_of"]) if "fkp_of" in spec else x
        return np.c_[x, fkp_weights(src, at=x)]
    return np.c_[x, lognormal_weights(len(x), float(w), seed=spec["wseed"])]


def catalogue_sha256(a: np.ndarray) -> str:
    """sha256 of a catalogue's float64 bytes (C order)."""
    return hashlib.sha256(np.ascontiguousarray(a, np.float64).tobytes()
                          ).hexdigest()
