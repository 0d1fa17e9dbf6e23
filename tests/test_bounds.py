"""Properties the reconnection pass relies on (CPU, numpy).

The pass may decide a pair on corrections that lack the last rewirings when
a bound on the missing segments' terms decides it: a straight segment S at
distance d (closest point) from a point adds at most kappa |S| / (4 pi d^2)
to its velocity, because |dl x r| / |r|^3 <= |dl| / d^2 along it.  The law
is the reference's closed form for a straight segment (octree.c:321-342,
tangle.c:536-559: R = start - r, Rp1 = end - r).
"""
from __future__ import annotations

import numpy as np

KAPPA = 9.97e-4


def segment_law(R, Rp1):
    lR = np.linalg.norm(R, axis=-1)
    lRp1 = np.linalg.norm(Rp1, axis=-1)
    dot = np.sum(R * Rp1, axis=-1)
    pr = lR * lRp1
    sc = KAPPA / (4 * np.pi) * (lR + lRp1) / (pr * (pr + dot))
    return np.cross(R, Rp1) * sc[..., None]


def dist_to_segment(q, a, b):
    s = b - a
    u = np.clip(np.sum((q - a) * s, axis=-1) / np.sum(s * s, axis=-1), 0.0, 1.0)
    return np.linalg.norm(q - (a + u[..., None] * s), axis=-1)


def test_segment_term_within_its_distance_bound():
    rng = np.random.default_rng(7)
    n = 200_000
    a = rng.normal(size=(n, 3))
    s = rng.normal(size=(n, 3)) * rng.uniform(1e-4, 2.0, size=(n, 1))
    q = rng.normal(size=(n, 3)) * rng.uniform(0.01, 3.0, size=(n, 1))
    d = dist_to_segment(q, a, a + s)
    keep = d > 1e-6
    w = segment_law(a[keep] - q[keep], a[keep] + s[keep] - q[keep])
    bound = KAPPA * np.linalg.norm(s[keep], axis=-1) / (4 * np.pi * d[keep] ** 2)
    ratio = np.linalg.norm(w, axis=-1) / bound
    assert ratio.max() <= 1.0 + 1e-9


def test_sphere_bound_covers_the_four_segments():
    """Far from a ball around the changed segments (radius rho about one of
    their ends), every point of them is at least |q - c| - rho away."""
    rng = np.random.default_rng(8)
    for _ in range(2000):
        ends = rng.normal(size=(8, 3)) * 1e-3
        c = ends[0]
        rho = np.linalg.norm(ends - c, axis=-1).max()
        q = c + rng.normal(size=3) * rng.uniform(4.01, 50.0) * rho
        D = np.linalg.norm(q - c)
        if D <= 4 * rho:
            continue
        a, b = ends[0::2], ends[1::2]
        d = dist_to_segment(q[None, :], a, b)
        assert np.all(d >= D - rho - 1e-15)
        w = segment_law(a - q, b - q)
        total = np.linalg.norm(w.sum(axis=0))
        slen = np.linalg.norm(b - a, axis=-1).sum()
        assert total <= KAPPA * slen / (4 * np.pi * (D - rho) ** 2) * (1 + 1e-9)
