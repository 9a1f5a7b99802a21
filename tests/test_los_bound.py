"""The line-of-sight prefilter of the survey (s_perp, pi) kernel, checked on
the CPU as arithmetic: with m = x_a + x_b = 2 x_b + d and |m| <= 2|x_b| + s,
pi = |d.m| / |m| < pi_max implies |d.u_b| < pi_max + (pi_max s + s^2) /
(2|x_b|).  The kernel tests |d.u_b| < los_p + (los_pr + los_h s^2) / |x_b|
in FP32 with los_p = pi_max (1 + 2^-8) + R 2^-12, los_pr = (1 + 2^-8)
pi_max R / 2, los_h = (1 + 2^-8) / 2, R the outer radius, for |x_b| > R.
Pairs placed just inside pi_max, at the largest separations and the
nearest allowed |x_b| (the worst cases of the bound), must all pass the
test evaluated in float32; pairs well outside must mostly fail it."""
import numpy as np


def _pi_exact(xa, xb):
    d = xa - xb
    m = xa + xb
    return np.abs((d * m).sum(1)) / np.linalg.norm(m, axis=1)


def _kernel_test(xa, xb, pmax, R):
    f32 = np.float32
    f = 1 + 2.0 ** -8
    los_p = f32(pmax * f + R * 2.0 ** -12 + 1e-6)
    los_pr = f32(0.5 * f * pmax * R)
    los_h = f32(0.5 * f)
    xb32 = xb.astype(f32)
    d32 = (xa - xb).astype(f32)
    r2 = (xb32 * xb32).sum(1, dtype=f32)
    ir = (f32(1) / np.sqrt(r2)).astype(f32)
    u = xb32 * ir[:, None]
    t = (d32 * u).sum(1, dtype=f32)
    v = (d32 * d32).sum(1, dtype=f32)
    thr = v * (los_h * ir) + (los_pr * ir + los_p)
    keep = np.abs(t) < thr
    return np.where(r2 > f32(R * R), keep, True)


def _pairs(rng, n, pmax, spmax, dist, pi_target):
    u = rng.normal(size=(n, 3))
    u /= np.linalg.norm(u, axis=1)[:, None]
    c = u * dist[:, None]                 # pair midpoint: line of sight u
    perp = rng.normal(size=(n, 3))
    perp -= (perp * u).sum(1)[:, None] * u
    perp /= np.linalg.norm(perp, axis=1)[:, None]
    d = pi_target[:, None] * u * rng.choice([-1.0, 1.0], n)[:, None] + \
        perp * (spmax * rng.uniform(0.9, 1.0, n))[:, None]
    return c + 0.5 * d, c - 0.5 * d       # x_a, x_b


def test_prefilter_keeps_every_pair_inside_pi_max():
    rng = np.random.default_rng(5)
    for pmax, spmax in ((40.0, 100.0), (5.0, 30.0), (80.0, 20.0)):
        R = np.sqrt(pmax ** 2 + spmax ** 2) * (1 + 1e-6)
        n = 200000
        dist = R * rng.uniform(1.0, 3.0, n) + rng.uniform(0, 3000, n) * \
            (rng.random(n) < 0.3)
        xa, xb = _pairs(rng, n, pmax, spmax, dist,
                        pmax * (1 - rng.uniform(1e-9, 1e-3, n)))
        pi = _pi_exact(xa, xb)
        s = np.linalg.norm(xa - xb, axis=1)
        inside = (pi < pmax) & (s < R)
        assert inside.mean() > 0.9
        keep = _kernel_test(xa, xb, pmax, R) & _kernel_test(xb, xa, pmax, R)
        assert keep[inside].all(), np.nonzero(inside & ~keep)[0][:5]


def test_prefilter_drops_pairs_far_beyond_pi_max():
    rng = np.random.default_rng(6)
    pmax, spmax = 40.0, 100.0
    R = np.sqrt(pmax ** 2 + spmax ** 2)
    n = 100000
    xa, xb = _pairs(rng, n, pmax, 20.0, rng.uniform(1000, 2000, n),
                    np.full(n, 60.0))
    assert (_pi_exact(xa, xb) > 55).all()
    assert (~_kernel_test(xa, xb, pmax, R)).mean() > 0.99
