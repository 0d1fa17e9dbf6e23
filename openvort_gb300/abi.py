"""ctypes mirror of the C ABI (include/ov_tangle.h, include/openvort_gpu.h).

The tangle layout is OpenVort's ``struct tangle_state`` (include/tangle.h:47-66
of the reference); parameters are its process globals
(include/vortex_constants.h:11-60) gathered into one struct.
"""
from __future__ import annotations

import ctypes as C
import itertools

import numpy as np

OV_EMPTY, OV_FREE, OV_PINNED, OV_PINNED_SLIP = -1, 0, 1, 2
OV_WALL_OPEN, OV_WALL_PERIODIC, OV_WALL_MIRROR = 0, 1, 2
OV_NO_FLOW, OV_SIMPLE, OV_DECREASING = 0, 1, 2
OV_PREC_FP64, OV_PREC_MIXED, OV_PREC_DD = 0, 1, 2
# OV_PREC_FP64's tree walk: FP32 tests on split positions with FP64 inside
# guard bands (default), or every test in FP64
OV_WALK_SPLIT, OV_WALK_FP64 = 0, 1
OV_F_POS, OV_F_VELS, OV_F_VS, OV_F_TANGENTS, OV_F_NORMALS, OV_F_TOPOLOGY, OV_F_ALL = 1, 2, 4, 8, 16, 32, 63

STATUS_NAMES = {
    0: "OV_OK", 1: "OV_ERR_ARG", 2: "OV_ERR_CUDA", 3: "OV_ERR_ALLOC", 4: "OV_ERR_DEPTH",
    5: "OV_ERR_STACK", 6: "OV_ERR_NAN", 7: "OV_ERR_TIMEOUT", 8: "OV_ERR_TOPOLOGY",
    9: "OV_ERR_NODEVICE", 10: "OV_ERR_STATE",
}


class Vec3(C.Structure):
    _fields_ = [("p", C.c_double * 3)]


class Neighbour(C.Structure):
    _fields_ = [("forward", C.c_int), ("reverse", C.c_int)]


class NodeStatus(C.Structure):
    _fields_ = [("status", C.c_int), ("pin_wall", C.c_int)]


class DomainBox(C.Structure):
    _fields_ = [("bottom_left_back", Vec3), ("top_right_front", Vec3), ("wall", C.c_int * 6)]


class ImageTangle(C.Structure):
    _fields_ = [("shift", C.c_int * 3), ("reflect", C.c_int * 3), ("number_of_reflects", C.c_int)]


class BoundaryImages(C.Structure):
    _fields_ = [("images", C.POINTER(ImageTangle)), ("n", C.c_int)]


class TangleState(C.Structure):
    _fields_ = [
        ("vnodes", C.POINTER(Vec3)), ("vels", C.POINTER(Vec3)), ("vs", C.POINTER(Vec3)),
        ("tangents", C.POINTER(Vec3)), ("normals", C.POINTER(Vec3)),
        ("recalculate", C.POINTER(C.c_int)), ("connections", C.POINTER(Neighbour)),
        ("status", C.POINTER(NodeStatus)), ("box", DomainBox), ("bimg", BoundaryImages),
        ("N", C.c_int), ("next_empty", C.c_int), ("total_empty", C.c_int),
    ]


class SphDomain(C.Structure):
    """ov_sph_domain: the spherical fork's section (radii, angular half widths)."""
    _fields_ = [("inner_radius", C.c_double), ("outer_radius", C.c_double), ("azimut_angle", C.c_double),
                ("polar_angle", C.c_double)]


class SphTangleState(C.Structure):
    """ov_sph_tangle_state: the spherical fork's tangle_state (status.pin_wall = pin_surface)."""
    _fields_ = [
        ("vnodes", C.POINTER(Vec3)), ("vels", C.POINTER(Vec3)), ("vs", C.POINTER(Vec3)),
        ("tangents", C.POINTER(Vec3)), ("normals", C.POINTER(Vec3)),
        ("recalculate", C.POINTER(C.c_int)), ("connections", C.POINTER(Neighbour)),
        ("status", C.POINTER(NodeStatus)), ("domain_section", SphDomain),
        ("N", C.c_int), ("next_empty", C.c_int), ("total_empty", C.c_int),
    ]


class SphParams(C.Structure):
    """ov_sph_params: the spherical fork's globals on its velocity path."""
    _fields_ = [("kappa", C.c_double), ("vortex_width", C.c_double), ("alpha", C.c_double), ("alpha_p", C.c_double),
                ("use_mutual_friction", C.c_int), ("bh_resolution", C.c_double), ("dl_min", C.c_double),
                ("dl_max", C.c_double), ("q_dot", C.c_double), ("temp_bath", C.c_double),
                ("use_temperature", C.c_int), ("outer_surface", C.c_int)]


OV_INNER, OV_OUTER = 0, 1


class ExtVel(C.Structure):
    _fields_ = [("type", C.c_int), ("strength", C.c_double), ("time_of_linear_decrease", C.c_double),
                ("starting_strength", C.c_double), ("direction", Vec3)]


class Params(C.Structure):
    _fields_ = [
        ("kappa", C.c_double), ("vortex_width", C.c_double), ("alpha", C.c_double),
        ("alpha_p", C.c_double), ("use_mutual_friction", C.c_int), ("use_bh", C.c_int),
        ("bh_resolution", C.c_double), ("vn", ExtVel), ("vs", ExtVel), ("vb", ExtVel),
        ("dl_min", C.c_double), ("dl_max", C.c_double), ("rec_dist", C.c_double),
        ("reconnection_angle_cutoff", C.c_double), ("small_loop_cutoff", C.c_int),
        ("use_freq_filter", C.c_int), ("freq_to_cutoff", C.c_double), ("num_threads", C.c_int),
        ("pin_mode", C.c_int),
    ]


class Stats(C.Structure):
    _fields_ = [(n, C.c_int64) for n in (
        "node_evals", "cells", "max_depth", "visits", "accepts", "warp_steps", "fp64_fallbacks",
        "near_field_fp64", "out_of_root", "reconnections", "remesh_added", "remesh_removed",
        "small_loops_removed", "error_word", "reconnect_candidates", "reconnect_fp64_pairs",
        "reconnect_exact_pairs", "reconnect_evaluated", "wall_clipped", "wall_removed", "injected_nodes",
        "reconnect_lazy_evals")]


class Injection(C.Structure):
    """ov_injection: the reference's injection settings (vortex_constants.h:48-56)
    and the state of the drand48 stream they draw from (rand48[0] = low 16 bits)."""
    _fields_ = [("loop_injection", C.c_int), ("loop_frequency", C.c_double), ("line_injection", C.c_int),
                ("line_n", C.c_int), ("line_frequency", C.c_double), ("line_polarized", C.c_int),
                ("rand48", C.c_ushort * 3)]


def srand48_state(seed: int) -> tuple[int, int, int]:
    """The drand48 state srand48(seed) leaves: the high 32 bits from the seed,
    the low 16 bits 0x330E (POSIX)."""
    seed &= 0xFFFFFFFF
    return (0x330E, seed & 0xFFFF, seed >> 16)


def make_injection(seed: int = 0, loop_frequency: float = 0.0, line_n: int = 0, line_frequency: float = 0.0,
                   line_polarized: bool = False) -> Injection:
    """Injection settings; a frequency of 0 leaves that kind off."""
    inj = Injection()
    inj.loop_injection = int(loop_frequency > 0)
    inj.loop_frequency = loop_frequency if loop_frequency > 0 else 1.0
    inj.line_injection = int(line_frequency > 0 and line_n > 0)
    inj.line_n = line_n
    inj.line_frequency = line_frequency if line_frequency > 0 else 1.0
    inj.line_polarized = int(line_polarized)
    inj.rand48[:] = srand48_state(seed)
    return inj


class Tuning(C.Structure):
    """ov_tuning: launch shape of the traversal."""
    _fields_ = [("warps_per_block", C.c_int), ("query_groups", C.c_int), ("blocks_per_sm", C.c_int),
                ("largest_first", C.c_int), ("high_occupancy", C.c_int)]


assert C.sizeof(TangleState) == 168 and C.sizeof(DomainBox) == 72 and C.sizeof(ExtVel) == 56
assert C.sizeof(SphTangleState) == 112 and SphTangleState.N.offset == 96


def image_shifts(n_images: int) -> list[tuple[int, int, int]]:
    """Periodic image shifts in the reference's table order.

    periodic_6/18/26 (src/boundary_images.c:13-72) list the shifts of
    {-1,0,1}^3 minus the origin with at most 1, 2 or 3 non-zero entries, in
    lexicographic order; ``0`` gives open boundaries.
    """
    maxnz = {0: 0, 6: 1, 18: 2, 26: 3}[n_images]
    out = [s for s in itertools.product((-1, 0, 1), repeat=3) if 0 < sum(map(abs, s)) <= maxnz]
    assert len(out) == n_images
    return out


# Faces (boundaries.h): LEFT, RIGHT, BACK, FRONT, DOWN, UP.
_L, _R, _B, _F, _D, _U = 0, 1, 2, 3, 4, 5
_P, _M, _O = OV_WALL_PERIODIC, OV_WALL_MIRROR, OV_WALL_OPEN


def image_set(name: str):
    """(images, walls) of one of the reference's named boundary configurations
    (src/boundary_images.c): images is a list of (shift, reflect faces), in
    the reference's table order, walls the six wall types of the box.

    The wall tables are data the drop-in must reproduce as the reference
    defines them, including two entries that look unintended: in
    wall_1_18 (boundary_images.c:193) the image (1, -1, 0) carries one
    reflection through LEFT (its count is written `01` with no face given),
    and wall_parallel_planes (:121-131) lists (-1, 1, -1) and (-1, 1, 1)
    twice while (1, -1, -1) and (1, -1, 1) are missing.
    """
    def lex(maxnz, reflect_down=False):
        out = []
        for sh in image_shifts({1: 6, 2: 18, 3: 26}[maxnz]):
            out.append((sh, (_D,) if reflect_down and sh[2] == -1 else ()))
        return out
    if name in ("periodic_6", "periodic_18", "periodic_26"):
        n = int(name.split("_")[1])
        return [(sh, ()) for sh in image_shifts(n)], (_P,) * 6
    if name == "open":
        return [], (_O,) * 6
    if name == "wall_1_open":
        return [((0, 0, -1), (_D,))], (_O, _O, _O, _O, _M, _O)
    walls_1 = (_P, _P, _P, _P, _M, _P)
    if name == "wall_1_6":
        return [(sh, r) for sh, r in lex(1, True) if sh != (0, 0, 1)], walls_1
    if name == "wall_1_18":
        out = lex(2, True)
        out = [(sh, (_L,) if sh == (1, -1, 0) else r) for sh, r in out]
        return out, walls_1
    if name == "wall_1_26":
        return lex(3, True), walls_1
    if name == "wall_2_4":
        return [((-1, 0, 0), ()), ((1, 0, 0), ()), ((0, -1, 0), ()), ((0, 1, 0), ()),
                ((0, 0, -1), (_D,)), ((0, 0, 1), (_U,))], (_P, _P, _P, _P, _M, _M)
    if name == "wall_2_2":
        return [((-1, 0, 0), ()), ((1, 0, 0), ()), ((0, -1, 0), (_B,)), ((0, 1, 0), (_F,)),
                ((0, 0, -1), (_D,)), ((0, 0, 1), (_U,))], (_P, _P, _M, _M, _M, _M)
    if name == "wall_parallel_planes":
        out = [((-1, 0, 0), ()), ((1, 0, 0), ()), ((0, -1, 0), ()), ((0, 1, 0), ()),
               ((0, 0, -1), (_D,)), ((0, 0, 1), (_U,))]
        out += [((-1, -1, 0), ()), ((1, -1, 0), ()), ((-1, 1, 0), ()), ((1, 1, 0), ())]
        for z, face in ((-1, _D), (1, _U)):
            out += [((1, 0, z), (face,)), ((-1, 0, z), (face,)), ((0, 1, z), (face,)), ((0, -1, z), (face,))]
        for z, face in ((-1, _D), (1, _U)):
            out += [((1, 1, z), (face,)), ((-1, 1, z), (face,)), ((-1, 1, z), (face,)), ((-1, -1, z), (face,))]
        return out, (_P, _P, _P, _P, _M, _M)
    if name == "wall_canal":
        def refl(sh):
            r = []
            if sh[1] == -1: r.append(_B)
            if sh[1] == 1: r.append(_F)
            if sh[2] == -1: r.append(_D)
            if sh[2] == 1: r.append(_U)
            return tuple(r)
        order = [(-1, 0, 0), (1, 0, 0), (0, -1, 0), (0, 1, 0), (0, 0, -1), (0, 0, 1),
                 (0, -1, -1), (0, -1, 1), (0, 1, -1), (0, 1, 1)]
        for x in (-1, 1):
            order += [(x, -1, 0), (x, 1, 0), (x, 0, -1), (x, 0, 1),
                      (x, -1, -1), (x, -1, 1), (x, 1, -1), (x, 1, 1)]
        return [(sh, refl(sh)) for sh in order], (_P, _P, _M, _M, _M, _M)
    raise ValueError(f"unknown boundary configuration {name!r}")


def image_table_of(images):
    """ctypes array of ImageTangle for a list of (shift, reflect faces)."""
    arr = (ImageTangle * max(len(images), 1))()
    for i, (sh, refl) in enumerate(images):
        arr[i].shift[:] = sh
        r = list(refl) + [0] * (3 - len(refl))
        arr[i].reflect[:] = r
        arr[i].number_of_reflects = len(refl)
    return arr


def image_table(n_images: int):
    """ctypes array of ImageTangle for a periodic image set (kept alive by caller)."""
    arr = (ImageTangle * max(n_images, 1))()
    for i, s in enumerate(image_shifts(n_images)):
        arr[i].shift[:] = s
        arr[i].reflect[:] = (-1, -1, -1)
        arr[i].number_of_reflects = 0
    return arr


def make_params(**kw) -> Params:
    """Reference defaults (src/initial_conditions.c:12-91) overridden by kw.

    Flow keywords: ``vn=(type, strength, (dx,dy,dz))`` and likewise vs, vb.
    """
    p = Params()
    p.kappa = 9.97e-4
    p.vortex_width = 1e-8
    p.alpha = 0.034
    p.alpha_p = 1.383e-2
    p.use_mutual_friction = 1
    p.use_bh = 1
    p.bh_resolution = 0.4
    _set_flow(p.vn, (OV_SIMPLE, 10.493799, (1.0, 0.0, 0.0)))
    _set_flow(p.vs, (OV_SIMPLE, 0.493799, (-1.0, 0.0, 0.0)))
    _set_flow(p.vb, (OV_NO_FLOW, 0.0, (0.0, 0.0, 0.0)))
    p.dl_min = 0.5e-3
    p.dl_max = 1.5e-3
    p.rec_dist = 4e-4
    p.reconnection_angle_cutoff = 5.0 * np.pi / 180.0
    p.small_loop_cutoff = 5
    p.use_freq_filter = 1
    p.freq_to_cutoff = 4.0 / 5
    p.num_threads = 1
    p.pin_mode = OV_PINNED
    for k, v in kw.items():
        if k in ("vn", "vs", "vb"):
            _set_flow(getattr(p, k), v)
        else:
            setattr(p, k, v)
    return p


def _set_flow(ev: ExtVel, spec):
    typ, strength, direction = spec[:3]
    ev.type = int(typ)
    ev.strength = float(strength)
    ev.direction.p[:] = [float(x) for x in direction]
    ev.time_of_linear_decrease = float(spec[3]) if len(spec) > 3 else 0.0
    ev.starting_strength = float(spec[4]) if len(spec) > 4 else 0.0


def vec3_view(ptr, n: int) -> np.ndarray:
    """(n,3) float64 numpy view on a C array of vec3."""
    if n == 0:
        return np.zeros((0, 3))
    return np.ctypeslib.as_array(C.cast(ptr, C.POINTER(C.c_double)), shape=(n, 3))


def int_view(ptr, n: int, width: int = 1) -> np.ndarray:
    if n == 0:
        return np.zeros((0, width) if width > 1 else (0,), dtype=np.int32)
    shape = (n, width) if width > 1 else (n,)
    return np.ctypeslib.as_array(C.cast(ptr, C.POINTER(C.c_int)), shape=shape)
