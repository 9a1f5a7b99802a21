"""Seeded synthetic catalogues with the shapes of FCFC's usual workloads.

* ``uniform_box``      -- Poisson points in a periodic box.
* ``neyman_scott``     -- clustered box: uniform parent centres, Poisson(mean)
                          children per parent offset by an isotropic Gaussian,
                          wrapped periodically.
* ``survey``           -- RA uniform in a range, sin(Dec) uniform, redshift
                          from a truncated normal; converted to comoving
                          Cartesian coordinates in a flat LCDM cosmology.
* ``fkp_weights``      -- 1 / (1 + n(z) P0) with n(z) from the redshift
                          histogram of the sample in comoving shells.

Everything is numpy only and deterministic for a given seed.
"""
from __future__ import annotations

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


def comoving_distance(z, omega_m: float = 0.31, npt: int = 4096):
    """Flat LCDM comoving distance in Mpc/h (trapezoid on a fine grid)."""
    z = np.asarray(z, np.float64)
    zmax = float(np.max(z)) if z.size else 0.0
    zz = np.linspace(0.0, max(zmax, 1e-6), npt)
    ez = np.sqrt(omega_m * (1 + zz) ** 3 + (1 - omega_m))
    integ = np.concatenate([[0.0], np.cumsum(0.5 * (1 / ez[1:] + 1 / ez[:-1])
                                             * np.diff(zz))])
    return np.interp(z, zz, integ) * C_KMS / 100.0


def survey_radecz(n: int, ra=(100.0, 260.0), dec=(0.0, 60.0), zmu=0.55,
                  zsig=0.10, zr=(0.4, 0.7), seed: int = 0) -> np.ndarray:
    rng = np.random.default_rng(seed)
    r = rng.uniform(ra[0], ra[1], n)
    s0, s1 = np.sin(np.radians(dec[0])), np.sin(np.radians(dec[1]))
    d = np.degrees(np.arcsin(rng.uniform(s0, s1, n)))
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
                ra=(100.0, 260.0), dec=(0.0, 60.0)) -> np.ndarray:
    """FKP weights with n(z) from the sample's redshift histogram."""
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
    vol = sky_fraction * 4 * np.pi / 3 * (rr[1:] ** 3 - rr[:-1] ** 3)
    nz = cnt / np.maximum(vol, 1e-300)
    idx = np.clip(np.searchsorted(edges, z, side="right") - 1, 0, cnt.size - 1)
    return 1.0 / (1.0 + nz[idx] * p0)
