"""Seeded synthetic tangles for the benchmark and the parity tests.

Random numbers come from a counter-based Philox4x32-10 generator (Salmon et
al., "Parallel random numbers: as easy as 1, 2, 3", SC'11) written here in
numpy, so the same seed gives the same tangle on every machine and numpy
version.

Tangles:
  * random_walk_tangle - closed random-walk loops: start uniform in the box,
    initial tangent uniform on the sphere, each step turns the tangent by a
    N(0, sigma) angle about an axis uniform in the plane normal to it, steps
    of length delta; the loop is closed by subtracting the linear end-point
    drift and wrapped into the periodic box.
  * ring_tangle - circular rings with the node placement of OpenVort's
    add_loop (src/vortex_injection.c:49-103): N = int(4 pi R/(dl_max+dl_min))
    nodes, basis from perpendicular() (vortex_injection.c:18-40).
  * ensemble - independent random-walk tangles with per-tangle parameters.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import abi

_M0, _M1 = np.uint64(0xD2511F53), np.uint64(0xCD9E8D57)
_W0, _W1 = np.uint64(0x9E3779B9), np.uint64(0xBB67AE85)
_MASK = np.uint64(0xFFFFFFFF)


def philox4x32(c0, c1, c2, c3, seed: int):
    """Philox4x32-10 on uint32 counter words (broadcast numpy arrays)."""
    c0, c1, c2, c3 = (np.asarray(x, dtype=np.uint64) & _MASK for x in (c0, c1, c2, c3))
    c0, c1, c2, c3 = np.broadcast_arrays(c0, c1, c2, c3)
    k0 = np.uint64(seed & 0xFFFFFFFF)
    k1 = np.uint64((seed >> 32) & 0xFFFFFFFF)
    for _ in range(10):
        p0 = _M0 * c0
        p1 = _M1 * c2
        hi0, lo0 = p0 >> np.uint64(32), p0 & _MASK
        hi1, lo1 = p1 >> np.uint64(32), p1 & _MASK
        c0, c1, c2, c3 = hi1 ^ c1 ^ k0, lo1, hi0 ^ c3 ^ k1, lo0
        k0 = (k0 + _W0) & _MASK
        k1 = (k1 + _W1) & _MASK
    return c0, c1, c2, c3


def uniform2(seed: int, a, b, purpose: int):
    """Two uniform doubles in [0,1) per counter (a, b, purpose)."""
    w0, w1, w2, w3 = philox4x32(a, b, purpose, 0, seed)
    s = np.float64(2.0 ** -53)
    u0 = ((w0 >> np.uint64(5)).astype(np.float64) * 67108864.0 + (w1 >> np.uint64(6)).astype(np.float64)) * s
    u1 = ((w2 >> np.uint64(5)).astype(np.float64) * 67108864.0 + (w3 >> np.uint64(6)).astype(np.float64)) * s
    return u0, u1


def normal2(seed: int, a, b, purpose: int):
    """Two standard normals per counter (Box-Muller)."""
    u0, u1 = uniform2(seed, a, b, purpose)
    r = np.sqrt(-2.0 * np.log1p(-u0))
    return r * np.cos(2 * np.pi * u1), r * np.sin(2 * np.pi * u1)


def _unit(v):
    return v / np.linalg.norm(v, axis=-1, keepdims=True)


def _wrap_into_box(pos, lo, hi):
    """enforce_periodic_boundaries (src/tangle.c:793-814) on a fresh tangle."""
    L = hi - lo
    for a in range(3):
        x = pos[:, a]
        for _ in range(8):
            low = x < lo[a]
            high = x > hi[a]
            if not (low.any() or high.any()):
                break
            x[low] += L[a]
            x[high] -= L[a]
    return pos


@dataclass
class HostTangle:
    """Host tangle in OpenVort's layout, backed by numpy arrays.

    ``state()`` returns a ``struct tangle_state`` (ctypes) whose arrays alias
    the numpy buffers; it is valid while this object lives.
    """

    pos: np.ndarray
    fwd: np.ndarray
    rev: np.ndarray
    box_lo: np.ndarray
    box_hi: np.ndarray
    n_images: int = 26
    status: np.ndarray | None = None
    walls: tuple = (1, 1, 1, 1, 1, 1)
    meta: dict = field(default_factory=dict)
    image_set: str = ""   # a named boundary configuration (sets images and walls)

    def __post_init__(self):
        n = len(self.pos)
        self.pos = np.ascontiguousarray(self.pos, dtype=np.float64)
        self.vels = np.zeros((n, 3))
        self.vs = np.zeros((n, 3))
        self.tangents = np.zeros((n, 3))
        self.normals = np.zeros((n, 3))
        self.recalc = np.zeros(n, dtype=np.int32)
        self.conn = np.ascontiguousarray(np.stack([self.fwd, self.rev], axis=1).astype(np.int32))
        st = np.full((n, 2), -1, dtype=np.int32)
        if self.status is None:
            st[:, 0] = abi.OV_FREE
        else:
            st[:, 0] = self.status
        self.stat = st
        if self.image_set:
            imgs, self.walls = abi.image_set(self.image_set)
            self.n_images = len(imgs)
            self._images = abi.image_table_of(imgs)
        else:
            self._images = abi.image_table(self.n_images)
        self._state = None

    @property
    def n(self) -> int:
        return len(self.pos)

    def state(self) -> abi.TangleState:
        s = abi.TangleState()
        dp = lambda a: a.ctypes.data_as(C.POINTER(abi.Vec3))  # noqa: E731
        s.vnodes, s.vels, s.vs = dp(self.pos), dp(self.vels), dp(self.vs)
        s.tangents, s.normals = dp(self.tangents), dp(self.normals)
        s.recalculate = self.recalc.ctypes.data_as(C.POINTER(C.c_int))
        s.connections = self.conn.ctypes.data_as(C.POINTER(abi.Neighbour))
        s.status = self.stat.ctypes.data_as(C.POINTER(abi.NodeStatus))
        s.box.bottom_left_back.p[:] = list(self.box_lo)
        s.box.top_right_front.p[:] = list(self.box_hi)
        s.box.wall[:] = list(self.walls)
        s.bimg.images = C.cast(self._images, C.POINTER(abi.ImageTangle))
        s.bimg.n = self.n_images
        s.N = self.n
        s.next_empty = -1
        s.total_empty = int((self.stat[:, 0] == abi.OV_EMPTY).sum())
        self._state = s
        return s


class SphTangle:
    """Host tangle of the spherical fork (section of a spherical shell),
    numpy-backed; ``state()`` gives its ``struct tangle_state``."""

    def __init__(self, pos, fwd, rev, status, pin, domain=(0.02, 0.1, np.radians(15), np.radians(15))):
        n = len(pos)
        self.pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(n, 3)
        self.vels = np.zeros((n, 3))
        self.vs = np.zeros((n, 3))
        self.tangents = np.zeros((n, 3))
        self.normals = np.zeros((n, 3))
        self.recalc = np.zeros(n, dtype=np.int32)
        self.conn = np.ascontiguousarray(np.stack([fwd, rev], 1), dtype=np.int32)
        self.stat = np.ascontiguousarray(np.stack([status, pin], 1), dtype=np.int32)
        self.domain = tuple(float(v) for v in domain)

    @property
    def n(self):
        return len(self.pos)

    def state(self) -> abi.SphTangleState:
        s = abi.SphTangleState()
        dp = lambda a: a.ctypes.data_as(C.POINTER(abi.Vec3))  # noqa: E731
        s.vnodes, s.vels, s.vs = dp(self.pos), dp(self.vels), dp(self.vs)
        s.tangents, s.normals = dp(self.tangents), dp(self.normals)
        s.recalculate = self.recalc.ctypes.data_as(C.POINTER(C.c_int))
        s.connections = self.conn.ctypes.data_as(C.POINTER(abi.Neighbour))
        s.status = self.stat.ctypes.data_as(C.POINTER(abi.NodeStatus))
        d = s.domain_section
        d.inner_radius, d.outer_radius, d.azimut_angle, d.polar_angle = self.domain
        s.N = self.n
        s.next_empty = -1
        s.total_empty = int((self.stat[:, 0] == abi.OV_EMPTY).sum())
        self._state = s
        return s


def spherical_tangle(n_rings: int = 12, ring_radius: float = 0.004, dl: float = 1e-3, seed: int = 7,
                     line: bool = True, empty: int = 3) -> SphTangle:
    """Seeded rings inside the spherical fork's default section (radii 0.02
    to 0.1 cm, +-15 degrees in both angles), a few of them across an angular
    edge, plus a radial line pinned on the inner surface (slipping) and the
    outer one, and some EMPTY slots."""
    rng = np.random.default_rng(seed)
    A = np.radians(15)
    pos, fwd, rev, st, pin = [], [], [], [], []
    base = 0
    npts = max(8, int(round(2 * np.pi * ring_radius / dl)))
    for r in range(n_rings):
        rad = rng.uniform(0.035, 0.085)
        az = rng.uniform(-0.8, 0.8) * A if r % 4 else 0.97 * A    # every fourth ring near the azimuth edge
        pl = rng.uniform(-0.8, 0.8) * A
        c = rad * np.array([np.cos(az) * np.cos(pl), np.cos(az) * np.sin(pl), np.sin(az)])
        axis = rng.normal(size=3)
        axis /= np.linalg.norm(axis)
        u = np.cross(axis, [1.0, 0.0, 0.0] if abs(axis[0]) < 0.9 else [0.0, 1.0, 0.0])
        u /= np.linalg.norm(u)
        v = np.cross(axis, u)
        phi = 2 * np.pi * np.arange(npts) / npts
        pos.append(c + ring_radius * (np.cos(phi)[:, None] * u + np.sin(phi)[:, None] * v))
        k = np.arange(npts)
        fwd.append(base + (k + 1) % npts)
        rev.append(base + (k - 1) % npts)
        st.append(np.full(npts, abi.OV_FREE))
        pin.append(np.full(npts, -1))
        base += npts
    if line:
        m = int(round((0.1 - 0.02) / dl))
        rr = np.linspace(0.02, 0.1, m + 1)
        ang = np.array([0.3 * A, -0.4 * A])
        d = np.array([np.cos(ang[0]) * np.cos(ang[1]), np.cos(ang[0]) * np.sin(ang[1]), np.sin(ang[0])])
        pos.append(rr[:, None] * d[None, :])
        k = np.arange(m + 1)
        f = base + k + 1
        f[-1] = -1
        b = base + k - 1
        b[0] = -1
        fwd.append(f)
        rev.append(b)
        s_ = np.full(m + 1, abi.OV_FREE)
        s_[0], s_[-1] = abi.OV_PINNED_SLIP, abi.OV_PINNED
        p_ = np.full(m + 1, -1)
        p_[0], p_[-1] = abi.OV_INNER, abi.OV_OUTER
        st.append(s_)
        pin.append(p_)
        base += m + 1
    if empty:
        pos.append(np.zeros((empty, 3)))
        fwd.append(np.full(empty, -1))
        rev.append(np.full(empty, -1))
        st.append(np.full(empty, abi.OV_EMPTY))
        pin.append(np.full(empty, -1))
    return SphTangle(np.concatenate(pos), np.concatenate(fwd), np.concatenate(rev), np.concatenate(st),
                     np.concatenate(pin))


def random_walk_tangle(n_loops: int, per_loop: int = 256, D: float = 0.1, delta: float = 1e-3,
                       sigma: float = 0.3, seed: int = 1, n_images: int = 26) -> HostTangle:
    """Closed random-walk loops in the periodic cube [0, D)^3."""
    loops = np.arange(n_loops, dtype=np.uint64)
    ux, uy = uniform2(seed, loops, 0xFFFFFFFF, 0)
    uz, _ = uniform2(seed, loops, 0xFFFFFFFF, 1)
    x0 = np.stack([ux, uy, uz], axis=1) * D
    g0, g1 = normal2(seed, loops, 0xFFFFFFFF, 2)
    g2, _ = normal2(seed, loops, 0xFFFFFFFF, 3)
    t = _unit(np.stack([g0, g1, g2], axis=1))

    pts = np.empty((n_loops, per_loop + 1, 3))
    pts[:, 0] = x0
    for j in range(1, per_loop + 1):
        th, _ = normal2(seed, loops, j, 4)
        th *= sigma
        phi, _ = uniform2(seed, loops, j, 5)
        phi *= 2 * np.pi
        # orthonormal basis of the plane normal to t
        ref = np.where(np.abs(t[:, :1]) < 0.9, np.array([[1.0, 0, 0]]), np.array([[0, 1.0, 0]]))
        e1 = _unit(np.cross(t, ref))
        e2 = np.cross(t, e1)
        w = np.cos(phi)[:, None] * e1 + np.sin(phi)[:, None] * e2  # = axis x t, uniform
        t = _unit(np.cos(th)[:, None] * t + np.sin(th)[:, None] * w)
        pts[:, j] = pts[:, j - 1] + delta * t
    drift = pts[:, per_loop] - pts[:, 0]
    frac = (np.arange(per_loop) / per_loop)[None, :, None]
    loop_pts = pts[:, :per_loop] - frac * drift[:, None, :]
    pos = np.mod(loop_pts.reshape(-1, 3), D)
    pos[pos >= D] -= D
    k = np.arange(n_loops * per_loop)
    base = (k // per_loop) * per_loop
    j = k % per_loop
    fwd = base + (j + 1) % per_loop
    rev = base + (j - 1) % per_loop
    lo = np.zeros(3)
    hi = np.full(3, float(D))
    ht = HostTangle(pos, fwd, rev, lo, hi, n_images=n_images)
    ht.meta = dict(kind="random_walk", n_loops=n_loops, per_loop=per_loop, D=D, delta=delta,
                   sigma=sigma, seed=seed)
    return ht


def _perpendicular(d):
    """perpendicular() of vortex_injection.c:18-40."""
    a = np.array([1.0, 0, 0])
    res = d * (-np.dot(a, d)) + a
    if np.sqrt(np.dot(res, res)) > 1e-8:
        return res / np.sqrt(np.dot(res, res))
    b = np.array([0, 1.0, 0])
    res = d * (-np.dot(b, d)) + b
    return res / np.sqrt(np.dot(res, res))


def ring_tangle(n_rings: int = 8, radius: float = 0.02, D: float = 0.1, dl_min: float = 1e-3,
                dl_max: float = 3e-3, seed: int = 7, n_images: int = 26) -> HostTangle:
    """Rings with add_loop's node placement, centres uniform, axes uniform on S^2."""
    npts = int(4 * np.pi * radius / (dl_max + dl_min))
    rings = np.arange(n_rings, dtype=np.uint64)
    cx, cy = uniform2(seed, rings, 0, 10)
    cz, _ = uniform2(seed, rings, 0, 11)
    centers = np.stack([cx, cy, cz], axis=1) * D
    g0, g1 = normal2(seed, rings, 0, 12)
    g2, _ = normal2(seed, rings, 0, 13)
    axes = _unit(np.stack([g0, g1, g2], axis=1))
    pos = []
    for r in range(n_rings):
        d = axes[r]
        z = _perpendicular(d)
        u = np.cross(z, d)
        v = np.cross(d, u)
        u = u / np.sqrt(np.dot(u, u))
        v = v / np.sqrt(np.dot(v, v))
        phi = 2 * np.pi / npts * np.arange(npts)
        pos.append(u[None] * (radius * np.cos(phi))[:, None] + v[None] * (radius * np.sin(phi))[:, None]
                   + centers[r][None])
    pos = np.concatenate(pos)
    lo, hi = np.zeros(3), np.full(3, float(D))
    pos = _wrap_into_box(pos, lo, hi)
    k = np.arange(n_rings * npts)
    base = (k // npts) * npts
    j = k % npts
    ht = HostTangle(pos, base + (j + 1) % npts, base + (j - 1) % npts, lo, hi, n_images=n_images)
    ht.meta = dict(kind="rings", n_rings=n_rings, radius=radius, D=D, npts=npts, seed=seed)
    return ht


def crossing_rings(n_pairs: int = 8, radius: float = 0.02, D: float = 0.1, dl_min: float = 1e-3,
                   dl_max: float = 3e-3, seed: int = 43, gap_min: float = 2e-4, gap_max: float = 2e-3,
                   n_images: int = 26) -> HostTangle:
    """Pairs of rings that pass close to one another, so that the time steps
    reconnect: ring A of each pair is placed as in ring_tangle (seeded centre
    and axis); ring B passes A's point at angle 0 at a seeded gap in
    [gap_min, gap_max], outside A, its plane tilted about A's radius there by
    a seeded angle in [20, 160] degrees.  Node placement as add_loop's."""
    npts = int(4 * np.pi * radius / (dl_max + dl_min))
    ids = np.arange(n_pairs, dtype=np.uint64)
    cx, cy = uniform2(seed, ids, 0, 30)
    cz, ug = uniform2(seed, ids, 0, 31)
    ub, _ = uniform2(seed, ids, 0, 32)
    g0, g1 = normal2(seed, ids, 0, 33)
    g2, _ = normal2(seed, ids, 0, 34)
    centers = np.stack([cx, cy, cz], axis=1) * D
    axes = _unit(np.stack([g0, g1, g2], axis=1))
    phi = 2 * np.pi / npts * np.arange(npts)
    pos = []
    for i in range(n_pairs):
        d = axes[i]
        z = _perpendicular(d)
        u = _unit(np.cross(z, d))
        v = np.cross(d, u)
        pos.append(centers[i] + radius * (np.cos(phi)[:, None] * u + np.sin(phi)[:, None] * v))
        gap = gap_min + ug[i] * (gap_max - gap_min)
        beta = np.radians(20 + 140 * ub[i])
        w = np.cos(beta) * d + np.sin(beta) * v
        cb = centers[i] + (2 * radius + gap) * u
        pos.append(cb + radius * (np.cos(phi + np.pi)[:, None] * u + np.sin(phi + np.pi)[:, None] * w))
    lo, hi = np.zeros(3), np.full(3, float(D))
    pos = _wrap_into_box(np.concatenate(pos), lo, hi)
    k = np.arange(2 * n_pairs * npts)
    base = (k // npts) * npts
    j = k % npts
    ht = HostTangle(pos, base + (j + 1) % npts, base + (j - 1) % npts, lo, hi, n_images=n_images)
    ht.meta = dict(kind="crossing_rings", n_pairs=n_pairs, radius=radius, D=D, npts=npts, seed=seed)
    return ht


@dataclass
class EnsembleMember:
    tangle: HostTangle
    alpha: float
    alpha_p: float
    vn: float


def ensemble(n_tangles: int = 48, min_nodes: int = 2048, max_nodes: int = 131072, per_loop: int = 256,
             D: float = 0.1, seed: int = 11) -> list[EnsembleMember]:
    """Independent tangles with log-uniform node counts and per-tangle parameters."""
    ids = np.arange(n_tangles, dtype=np.uint64)
    u_n, u_a = uniform2(seed, ids, 0, 20)
    u_ap, u_vn = uniform2(seed, ids, 0, 21)
    out = []
    for i in range(n_tangles):
        n = np.exp(np.log(min_nodes) + u_n[i] * (np.log(max_nodes) - np.log(min_nodes)))
        n_loops = max(1, int(round(n / per_loop)))
        t = random_walk_tangle(n_loops, per_loop, D=D, seed=seed * 1000 + i)
        out.append(EnsembleMember(t, 0.03 + u_a[i] * 0.27, u_ap[i] * 0.02, 0.2 + u_vn[i] * 1.8))
    return out


def member_params(m: EnsembleMember, **over) -> abi.Params:
    """Run parameters of one ensemble member: the random-walk set with the
    member's alpha, alpha' and v_n (along x)."""
    return config_params("rw", alpha=m.alpha, alpha_p=m.alpha_p, vn=(abi.OV_SIMPLE, m.vn, (1, 0, 0)), **over)


def config_params(name: str, **over) -> abi.Params:
    """Run parameters of the named benchmark configuration."""
    base = dict(kappa=9.97e-4, vortex_width=1.3e-8, alpha=0.098, alpha_p=0.016, use_bh=1,
                bh_resolution=0.4, vs=(abi.OV_NO_FLOW, 0.0, (0, 0, 0)),
                vb=(abi.OV_NO_FLOW, 0.0, (0, 0, 0)), vn=(abi.OV_SIMPLE, 0.5, (1, 0, 0)),
                dl_min=5e-4, dl_max=1.5e-3, rec_dist=4e-4, use_freq_filter=0)
    if name == "rings8":
        base.update(dl_min=1e-3, dl_max=3e-3, rec_dist=8e-4)
    elif name == "large":
        base.update(vn=(abi.OV_SIMPLE, 1.0, (1, 0, 0)), use_freq_filter=1, freq_to_cutoff=0.8)
    base.update(over)
    return abi.make_params(**base)
