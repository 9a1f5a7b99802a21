"""Pairs placed on FCFC's bin boundaries, for the near-edge exactness tests.

For every decision boundary of a binning -- each s^2 (or s_perp^2) edge, each
mu edge (mu^2 nmu^2 = k^2, k = 1 .. nmu; k = nmu is mu = 1), each pi (box) or
pi^2 (survey) edge, and the lower edges when s_min / pi_min > 0 -- this builds
pairs whose FP64 value, computed as FCFC computes it, is the edge itself and
the 1st, 2nd and 4th representable values on either side of it.  The values
follow FCFC's per-pair formulas in its order of operations:
  box     src/fcfc/2pt_box/metric_common.c:140-235 (dx = x1 - x2; s^2 =
          dx^2 + dy^2 + dz^2; mu^2 nmu^2 = (dz^2 / s^2) nmu^2; s_perp^2 =
          dx^2 + dy^2; pi = |dz|);
  survey  src/fcfc/2pt/metric_common.c:142-260 (t = 2 x1.x2, S = s1 + s2,
          s^2 = S - t, pi^2 = (s1 - s2)^2 / (S + t), s_perp^2 = s^2 - pi^2,
          mu^2 nmu^2 = (pi^2 / s^2) nmu^2), s_i = |x_i|^2 as build_tree.c:53;
after the rescale x fac of build_tree.c:121-131 (as the oracle restates them,
oracle/fcfc_oracle.c fco_bin_box / fco_bin_survey / fco_cat_make).

A pair is built from a first point and a separation chosen analytically,
then one coordinate of the second point is moved by whole units in its last
place; the values this reaches around the edge (in a box the free coordinate
is one whose component of the separation is small, so the steps are single
ulps; in a survey, far from the observer, s^2 = S - t only takes values on a
grid of ulp(S)) are sorted, and the pairs at steps {0, 1, 2, 4} above and
{1, 2, 4} below the edge kept.  Pairs are spaced on a lattice (box) or on
spherical shells (survey) more than three outer radii apart, so no two
constructed pairs interact: each catalogue's in-range candidates are
exactly its constructed pairs.
"""
from __future__ import annotations

import numpy as np

STEPS_UP = (0, 1, 2, 4)
STEPS_DOWN = (1, 2, 4)


# ---------------------------------------------------------------- values ---

def _rescale(x, fac):
    return x * fac if fac != 1 else x


def box_values(a, b, fac, nmu):
    """FCFC's FP64 values of the box pairs (a[i], b[i]) (arrays n x 3, raw
    coordinates, no periodic image between them)."""
    A = _rescale(a, fac)
    B = _rescale(b, fac)
    dx = A[:, 0] - B[:, 0]
    dy = A[:, 1] - B[:, 1]
    dz = A[:, 2] - B[:, 2]
    dz2 = dz * dz
    s2 = dx * dx + dy * dy + dz2
    with np.errstate(divide="ignore", invalid="ignore"):
        q2 = (dz2 / s2) * float(nmu * nmu)
    return {"s2": s2, "q2": q2, "sp2": dx * dx + dy * dy, "pi": np.abs(dz)}


def survey_values(a, b, fac, nmu):
    """FCFC's FP64 values of the survey pairs (a[i], b[i])."""
    A = _rescale(a, fac)
    B = _rescale(b, fac)
    s1 = A[:, 0] * A[:, 0] + A[:, 1] * A[:, 1] + A[:, 2] * A[:, 2]
    s2_ = B[:, 0] * B[:, 0] + B[:, 1] * B[:, 1] + B[:, 2] * B[:, 2]
    t = (A[:, 0] * B[:, 0] + A[:, 1] * B[:, 1] + A[:, 2] * B[:, 2]) * 2
    S = s1 + s2_
    d = S - t
    dd = s1 - s2_
    pi2 = dd * dd / (S + t)
    with np.errstate(divide="ignore", invalid="ignore"):
        q2 = (pi2 / d) * float(nmu * nmu)
    # the iso binning takes s^2 from the differences (metric_common.c:152)
    dx = A[:, 0] - B[:, 0]
    dy = A[:, 1] - B[:, 1]
    dz = A[:, 2] - B[:, 2]
    return {"s2": d, "q2": q2, "sp2": d - pi2, "pi2": pi2,
            "s2iso": dx * dx + dy * dy + dz * dz}


# ---------------------------------------------------------- construction ---

def _around(values_of, a, b0, axis, edge, span):
    """Second points b (moving b0[axis] by n ulps, |n| <= span) whose value
    is the edge and the chosen steps around it: {step: b} (missing steps are
    left out when the reachable values do not extend that far)."""
    n = np.arange(-span, span + 1, dtype=np.float64)
    step = np.spacing(abs(b0[axis]))
    bb = np.repeat(b0[None, :], len(n), axis=0)
    bb[:, axis] = b0[axis] + n * step
    aa = np.repeat(a[None, :], len(n), axis=0)
    v = values_of(aa, bb)
    ok = np.isfinite(v)
    vals = np.unique(v[ok])
    i0 = int(np.searchsorted(vals, edge, side="left"))
    out = {}
    for s in STEPS_UP:
        if i0 + s < len(vals):
            out[s] = bb[np.nonzero(v == vals[i0 + s])[0][0]]
    for s in STEPS_DOWN:
        if i0 - s >= 0:
            out[-s] = bb[np.nonzero(v == vals[i0 - s])[0][0]]
    return out


def _crossing(values_of, a, b0, axis, edge, lim=1 << 40):
    """Move b0[axis] by whole ulps until the value crosses the edge (the
    value is monotone in the move): the b closest to the crossing."""
    step = np.spacing(abs(b0[axis]))

    def f(n):
        b = b0.copy()
        b[axis] = b0[axis] + n * step
        return values_of(a[None, :], b[None, :])[0], b
    v0, _ = f(0)
    # the direction in which the value grows: probe until it changes
    sgn = 0.0
    for p in range(4, 44, 2):
        up_v, _ = f(1 << p)
        if up_v != v0:
            sgn = 1.0 if up_v > v0 else -1.0
            break
    if sgn == 0.0:
        return None
    want_up = v0 < edge
    lo, hi = 0, 1
    # exponential search for a bracket, then bisection
    while hi < lim:
        v, _ = f(sgn * hi * (1 if want_up else -1))
        if (v >= edge) == want_up:
            break
        lo, hi = hi, hi * 2
    while hi - lo > 1:
        mid = (lo + hi) // 2
        v, _ = f(sgn * mid * (1 if want_up else -1))
        if (v >= edge) == want_up:
            hi = mid
        else:
            lo = mid
    return f(sgn * hi * (1 if want_up else -1))[1]


def _unit(rng):
    v = rng.normal(size=3)
    return v / np.linalg.norm(v)


class Builder:
    """Collects constructed pairs: a, b (raw coordinates), and for each the
    boundary it sits on and its step from it."""

    def __init__(self, geometry, fac, nmu, span=600):
        self.geometry = geometry
        self.fac = fac
        self.nmu = nmu
        self.span = span
        self.a, self.b, self.tag = [], [], []

    def values_of(self, key):
        if self.geometry == "box":
            return lambda a, b: box_values(a, b, self.fac, self.nmu)[key]
        return lambda a, b: survey_values(a, b, self.fac, self.nmu)[key]

    def add(self, key, edge, make, axis, tag, cross=True):
        """Pairs at every step around one boundary, each at its own site:
        make() returns a fresh (first point, second point near the edge).
        A pair is kept only when its value is within `want` steps of the
        edge's neighbourhood as constructed: the reachable values around it
        are no coarser than tol(edge) apart and the edge lies among them."""
        f = self.values_of(key)
        n = 0
        for want in STEPS_UP + tuple(-s for s in STEPS_DOWN):
            for _attempt in range(4):
                a, b0 = make()
                b1 = _crossing(f, a, b0, axis, edge) if cross else b0
                if b1 is None:
                    continue
                span = self.span
                while True:
                    got = _around(f, a, b1, axis, edge, span)
                    if want in got or span > 200000:
                        break
                    span *= 4
                if want not in got:
                    continue
                v = f(a[None, :], got[want][None, :])[0]
                # |v - edge| may not exceed (|want| + 1) reachable steps
                lim = (abs(want) + 1) * self.step_tol(edge)
                if abs(v - edge) <= lim:
                    self.a.append(a.copy())
                    self.b.append(got[want].copy())
                    self.tag.append((tag, want))
                    n += 1
                    break
        return n

    def step_tol(self, edge):
        """Largest spacing of reachable values near an edge: one ulp of the
        edge in a box; in a survey the grid of S - t (|x| up to 1750 raw:
        S < 2 (1750 fac)^2 + ...) and of pi^2 = dd^2 / (S + t)."""
        if self.geometry == "box":
            return np.spacing(abs(edge)) * 2
        big = 2 * (2000.0 * self.fac) ** 2 * 4
        return max(np.spacing(big) * 4, np.spacing(abs(edge)) * 2)

    def catalogue(self):
        """N x 3 raw coordinates: a0, b0, a1, b1, ... (a before b: in an
        auto count the image shift, none here, goes to the smaller index)."""
        out = np.empty((2 * len(self.a), 3))
        out[0::2] = np.array(self.a)
        out[1::2] = np.array(self.b)
        return out


def _ab(a, d):
    return a, a - d


def _mid_mu(rng, nmu):
    """A mu in the middle of a random mu bin (far from mu edges)."""
    return (rng.integers(0, nmu) + 0.5) / nmu


def _direction(mu, small, rng):
    """Unit separation with |z component| = mu and |x component| = small
    (the free axis for fine steps), y taking the rest."""
    y2 = max(1.0 - mu * mu - small * small, 0.0)
    sx = 1 if rng.random() < 0.5 else -1
    sy = 1 if rng.random() < 0.5 else -1
    sz = 1 if rng.random() < 0.5 else -1
    return np.array([sx * small, sy * np.sqrt(y2), sz * mu])


def box_pairs(bins, L, seed=0):
    """Constructed pairs for a periodic box binning.  bins: dict with
    bintype (0 iso, 1 smu, 2 spi), fac, s2 (rescaled squared edges), nmu,
    p (rescaled pi edges, spi), reach (raw outer radius)."""
    rng = np.random.default_rng(seed)
    fac, nmu, bt = bins["fac"], bins.get("nmu", 1), bins["bintype"]
    B = Builder("box", fac, nmu)
    sp = 3.2 * bins["reach"]
    nl = int(L // sp)
    sites = [(i, j, k) for i in range(nl) for j in range(nl) for k in range(nl)]
    rng.shuffle(sites)
    # the lowest layer is kept for pairs placed next to z = 0 (pi edges)
    site = iter([t for t in sites if t[2] > 0])
    low = iter([t for t in sites if t[2] == 0])

    def origin(small_z=False):
        i, j, k = next(low if small_z else site)
        c = (np.array([i, j, k]) + 0.5) * sp + rng.uniform(-0.1, 0.1, 3) * sp
        if small_z:
            c[2] = rng.uniform(0.5, 2.0)
        return c
    s2e = bins["s2"]
    ns = len(s2e) - 1
    se = np.sqrt(s2e) / fac                   # raw s edges
    # s (or s_perp) boundaries
    k0 = 0 if s2e[0] > 0 else 1
    for k in range(k0, ns + 1):
        if bt == 2:
            # s_perp^2 = dx^2 + dy^2 with dy small; pi in a middle bin
            pe = bins["p"] / fac
            j = rng.integers(0, len(pe) - 1)
            pi = 0.5 * (pe[j] + pe[j + 1])
            d = np.array([se[k] * np.sqrt(1 - 1e-10), 1e-5 * se[k], pi])
            B.add("sp2", s2e[k], lambda: _ab(origin(), d), 1, ("s", k))
        else:
            mu = _mid_mu(rng, nmu) if bt == 1 else rng.uniform(0.1, 0.9)
            d = se[k] * _direction(mu, 1e-5, rng)
            B.add("s2", s2e[k], lambda: _ab(origin(), d), 0, ("s", k))
    if bt == 1:
        # mu boundaries: mu^2 nmu^2 = k^2 at an s in the middle of an s bin
        for k in range(1, nmu + 1):
            j = rng.integers(0, ns)
            s = 0.5 * (se[j] + se[j + 1])
            mu = k / nmu
            small = 1e-5 if k < nmu else 0.0
            d = s * _direction(min(mu, 1.0), small, rng)
            if k == nmu:
                # mu = 1: along z, the free axis x from dx = 0: the values
                # reachable are nmu^2 itself and those below it
                d = np.array([0.0, 0.0, s])
                B.add("q2", float(k * k), lambda: _ab(origin(), d), 0,
                      ("mu", k), cross=False)
                continue
            B.add("q2", float(k * k), lambda: _ab(origin(), d), 0, ("mu", k))
    if bt == 2:
        pe = bins["p"]
        k0 = 0 if pe[0] > 0 else 1
        for k in range(k0, len(pe)):
            j = rng.integers(0, ns)
            sp_ = 0.5 * (se[j] + se[j + 1])
            d = np.array([sp_ * 0.6, sp_ * 0.8, -pe[k] / fac])
            B.add("pi", pe[k], lambda: _ab(origin(small_z=True), d), 2,
                  ("pi", k))
    return B


def survey_pairs(bins, radii=(1000.0, 1250.0, 1500.0, 1750.0), seed=0):
    """Constructed pairs for a survey binning, first points on spherical
    shells at the given comoving radii (raw units)."""
    rng = np.random.default_rng(seed)
    fac, nmu, bt = bins["fac"], bins.get("nmu", 1), bins["bintype"]
    B = Builder("survey", fac, nmu, span=40)
    sp = 3.2 * bins["reach"]
    centres = []
    for r in radii:
        n = int(4 * np.pi * r * r / (sp * sp))
        g = (1 + 5 ** 0.5) / 2
        for i in range(n):
            zz = 1 - (2 * i + 1) / n
            rr = np.sqrt(1 - zz * zz)
            ph = 2 * np.pi * i / g
            centres.append(r * np.array([rr * np.cos(ph), rr * np.sin(ph), zz]))
    rng.shuffle(centres)
    site = iter(centres)
    s2e = bins["s2"]
    ns = len(s2e) - 1
    se = np.sqrt(s2e) / fac

    def sep(a, s, mu):
        """Separation d = a - b of length s at mu to the midpoint line of
        sight a + b (a few fixed-point steps)."""
        w0 = _unit(rng)
        u = a / np.linalg.norm(a)
        for _ in range(6):
            w = w0 - np.dot(w0, u) * u
            w /= np.linalg.norm(w)
            d = s * (mu * u + np.sqrt(max(1 - mu * mu, 0.0)) * w)
            m = 2 * a - d
            u = m / np.linalg.norm(m)
        return d

    def survey_make(s, mu):
        def make():
            a = next(site)
            b0 = a - sep(a, s, mu)
            return a, b0
        return make

    k0 = 0 if s2e[0] > 0 else 1
    key_s = {0: "s2iso", 1: "s2", 2: "sp2"}[bt]
    for k in range(k0, ns + 1):
        mu = _mid_mu(rng, nmu) if bt == 1 else rng.uniform(0.1, 0.9)
        if bt == 2:
            pe = np.sqrt(bins["p"]) / fac
            j = rng.integers(0, len(pe) - 1)
            pi = 0.5 * (pe[j] + pe[j + 1])
            s = np.hypot(se[k], pi)
            mu = pi / s
        else:
            s = se[k]
        mk = survey_make(s, mu)
        B.add(key_s, s2e[k], mk, 2, ("s", k))
    if bt == 1:
        for k in range(1, nmu + 1):
            j = rng.integers(0, ns)
            s = 0.5 * (se[j] + se[j + 1])
            B.add("q2", float(k * k), survey_make(s, k / nmu), 2, ("mu", k))
    if bt == 2:
        p2e = bins["p"]
        k0 = 0 if p2e[0] > 0 else 1
        for k in range(k0, len(p2e)):
            j = rng.integers(0, ns)
            spp = 0.5 * (se[j] + se[j + 1])
            pi = np.sqrt(p2e[k]) / fac
            s = np.hypot(spp, pi)
            B.add("pi2", p2e[k], survey_make(s, pi / s), 2, ("pi", k))
    return B


# -------------------------------------------------------------- configs ---

def configs():
    """The binnings the near-edge tests use: (name, survey, bintype, oracle
    Bins keyword arguments, box side or None, outer radius, nmu)."""
    lg = np.geomspace(0.1, 40.0, 25)
    lg2 = np.geomspace(0.1, 40.0, 21)
    lg3 = np.geomspace(0.5, 40.0, 21)
    return [
        ("box_smu_lin", False, 1, dict(ns=20, smin=0, ds=2, nmu=25), 4000.0, 40.0, 25),
        ("box_smu_bench", False, 1, dict(ns=40, smin=0, ds=5, nmu=100), 20000.0, 200.0, 100),
        ("box_iso_smin", False, 0, dict(ns=20, smin=3, ds=1.5), 4000.0, 33.0, 1),
        ("box_smu_log", False, 1, dict(ns=24, sedges=lg, nmu=10), 4000.0, 40.0, 10),
        ("box_spi_log", False, 2, dict(ns=20, sedges=lg2, np_=20, pmin=0, dpi=2), 4000.0, 57.0, 1),
        ("box_spi_pmin", False, 2, dict(ns=15, smin=2, ds=2, np_=10, pmin=5, dpi=2.5), 4000.0, 40.0, 1),
        ("survey_smu", True, 1, dict(ns=8, smin=0, ds=5, nmu=20), None, 40.0, 20),
        ("survey_iso_smin", True, 0, dict(ns=19, smin=2, ds=2), None, 40.0, 1),
        ("survey_spi_log", True, 2, dict(ns=20, sedges=lg3, np_=20, pmin=0, dpi=2), None, 57.0, 1),
    ]


def build(cfg, seed=0):
    """(catalogue, Builder, oracle Bins) of one configuration."""
    from oracle import fcfc_oracle as fo
    name, survey, bt, kw, L, reach, nmu = cfg
    ob = fo.Bins(survey, bt, box=L, **kw)
    _, _, s2, p = ob.tables()
    bins = dict(bintype=bt, fac=ob.rescale, s2=s2, nmu=nmu, reach=reach, p=p)
    B = survey_pairs(bins, seed=seed) if survey else box_pairs(bins, L, seed=seed)
    return B.catalogue(), B, ob, bins


def expected_counts(B, bins, ntot, survey):
    """The histogram FCFC's rules give the constructed pairs, from their FP64
    values: bin k of an axis when edge_k <= v < edge_k+1 (FCFC's integer and
    hybrid tables both resolve to this), mu bin floor(sqrt(q2)) with q2 >=
    nmu^2 (mu = 1) dropped, out of range below the lowest or at/above the
    highest edge."""
    a = np.array(B.a)
    b = np.array(B.b)
    nmu = bins.get("nmu", 1)
    v = (survey_values if survey else box_values)(a, b, bins["fac"], nmu)
    s2e = bins["s2"]
    ns = len(s2e) - 1
    bt = bins["bintype"]
    key = {0: "s2iso" if survey else "s2", 1: "s2", 2: "sp2"}[bt]
    sv = v[key]
    si = np.searchsorted(s2e, sv, side="right") - 1
    ok = (si >= 0) & (si < ns)
    if s2e[0] == 0:
        ok |= (sv < 0) & (bt == 2)      # s_perp^2 slightly negative: bin 0
        si = np.where((sv < 0) & (bt == 2), 0, si)
    idx = si.copy()
    if bt == 1:
        q2 = v["q2"]
        p = np.floor(q2)
        ok &= p < nmu * nmu
        mi = np.floor(np.sqrt(np.clip(p, 0, None))).astype(np.int64)
        mi = np.where(mi * mi > p, mi - 1, mi)
        idx = si + mi * ns
    if bt == 2:
        pv = v["pi2"] if survey else v["pi"]
        pe = bins["p"]
        pj = np.searchsorted(pe, pv, side="right") - 1
        ok &= (pj >= 0) & (pj < len(pe) - 1)
        idx = si + pj * ns
    out = np.zeros(ntot, np.int64)
    np.add.at(out, idx[ok], 1)
    return out


def pair_values(B, bins, survey):
    """(value, edge) of every constructed pair, for its own boundary."""
    out = []
    bt = bins["bintype"]
    for (tag, step), a, b in zip(B.tag, B.a, B.b):
        kind, k = tag
        if kind == "s":
            key = {0: "s2iso" if survey else "s2", 1: "s2", 2: "sp2"}[bt]
            edge = bins["s2"][k]
        elif kind == "mu":
            key, edge = "q2", float(k * k)
        else:
            key, edge = ("pi2" if survey else "pi"), bins["p"][k]
        out.append((B.values_of(key)(a[None, :], b[None, :])[0], edge, step))
    return out
