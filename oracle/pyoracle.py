"""TEST INFRASTRUCTURE ONLY: Python driver for the CPU checkers.

Loads either
  * the C restatement   (oracle/_build/libovoracle.so, kind "port"), or
  * OpenVort itself     (oracle/_ref/libovref.so, kind "reference", built from
    the reference's own sources by oracle/Makefile where they are present),
and runs the velocity / time-step functions on C-allocated tangles in the
reference layout.  Used by tests/, the smoke check and the CPU-baseline leg
of bench.py; never by the library.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

from openvort_gb300 import abi

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "_build", "libovoracle.so")
PORT_FAST_SO = os.path.join(HERE, "_build", "libovoracle_fast.so")
REF_SO = os.path.join(HERE, "_ref", "libovref.so")

_TS = C.POINTER(abi.TangleState)


def build(ref: bool = True) -> None:
    """Compile the checkers (make -C oracle port [ref])."""
    targets = ["port"] + (["ref"] if ref else [])
    subprocess.run(["make", "-s", "-C", HERE] + targets, check=True)


class CTangle:
    """A tangle whose arrays were malloc'd by a checker library (may be realloc'd)."""

    def __init__(self, lib: "Checker", host):
        self.lib = lib
        self.ts = abi.TangleState()
        n = host.n
        lib._create(C.byref(self.ts), n)
        self.images = host._images if lib.kind == "port" else None
        v = self.views()
        v["pos"][:] = host.pos
        v["conn"][:] = host.conn
        v["status"][:] = host.stat
        v["vels"][:] = 0
        v["vs"][:] = 0
        v["tangents"][:] = 0
        v["normals"][:] = 0
        v["recalc"][:] = 0
        self.ts.box.bottom_left_back.p[:] = list(host.box_lo)
        self.ts.box.top_right_front.p[:] = list(host.box_hi)
        self.ts.box.wall[:] = list(host.walls)
        if lib.kind == "port":
            self.ts.bimg.images = C.cast(host._images, C.POINTER(abi.ImageTangle))
            self.ts.bimg.n = host.n_images
        else:
            # the reference's own table: by name, or the periodic set of that size
            self.ts.bimg = lib.reference_images(getattr(host, "image_set", "") or host.n_images)
        self.ts.next_empty = -1
        self.ts.total_empty = int((host.stat[:, 0] == abi.OV_EMPTY).sum())

    @property
    def n(self):
        return self.ts.N

    def views(self):
        n = self.ts.N
        return dict(
            pos=abi.vec3_view(self.ts.vnodes, n), vels=abi.vec3_view(self.ts.vels, n),
            vs=abi.vec3_view(self.ts.vs, n), tangents=abi.vec3_view(self.ts.tangents, n),
            normals=abi.vec3_view(self.ts.normals, n), conn=abi.int_view(self.ts.connections, n, 2),
            status=abi.int_view(self.ts.status, n, 2), recalc=abi.int_view(self.ts.recalculate, n))

    def copy(self, key):
        return np.array(self.views()[key])

    def free(self):
        if self.ts.vnodes:
            self.lib._free(C.byref(self.ts))
            self.ts.vnodes = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class Checker:
    """Common interface over the C restatement and the reference build."""

    def __init__(self, kind: str = "port", fast: bool = False):
        self.kind = kind
        if kind == "port":
            path = PORT_FAST_SO if fast else PORT_SO
            if not os.path.exists(path):
                build(ref=False)
            self.lib = C.CDLL(path)
            L = self.lib
            self._create = L.orc_tangle_create
            self._create.argtypes = [_TS, C.c_int]
            self._free = L.orc_tangle_free
            self._free.argtypes = [_TS]
            P = C.POINTER(abi.Params)
            for name, args in [
                ("orc_update_tangents_normals", [_TS]),
                ("orc_update_velocities", [_TS, C.c_double, P]),
                ("orc_rk4_step", [_TS, C.c_double, C.c_double, P]),
                ("orc_reconnect", [_TS, C.c_double, P, C.POINTER(C.c_int), C.POINTER(C.c_int), C.c_int]),
                ("orc_remesh", [_TS, C.c_double, C.c_double, C.c_double, P, C.POINTER(C.c_int),
                                C.POINTER(C.c_int)]),
                ("orc_eliminate_small_loops", [_TS, P]),
                ("orc_enforce_periodic_boundaries", [_TS]),
                ("orc_smooth", [_TS, P]),
                ("orc_direct_velocities", [_TS, C.POINTER(C.c_int), C.c_int, C.c_double, P]),
                ("orc_step", [_TS, C.c_double, C.c_double, P, C.POINTER(C.c_int)]),
                ("orc_low_pass_filter", [C.POINTER(C.c_double), C.c_int, C.c_double]),
            ]:
                getattr(L, name).argtypes = args
            L.orc_reconnect.restype = C.c_int
            L.orc_eliminate_small_loops.restype = C.c_int
            self.params = abi.make_params()
        elif kind == "reference":
            if not os.path.exists(REF_SO):
                build(ref=True)
            if not os.path.exists(REF_SO):
                raise FileNotFoundError("reference build not available (oracle/_ref)")
            self.lib = C.CDLL(REF_SO)
            L = self.lib
            self._create = L.create_tangle
            self._create.argtypes = [_TS, C.c_size_t]
            self._free = L.free_tangle
            self._free.argtypes = [_TS]
            for name, args in [
                ("update_tangents_normals", [_TS]), ("update_velocities", [_TS, C.c_double]),
                ("rk4_step", [_TS, C.c_double, C.c_double]), ("reconnect", [_TS, C.c_double]),
                ("remesh", [_TS, C.c_double, C.c_double, C.c_double]),
                ("eliminate_small_loops", [_TS]), ("enforce_periodic_boundaries", [_TS]),
                ("update_velocity", [_TS, C.c_int, C.c_double, C.c_void_p]),
                ("update_tangent_normal", [_TS, C.c_size_t]),
            ]:
                getattr(L, name).argtypes = args
            L.reconnect.restype = C.c_int
        else:
            raise ValueError(kind)

    # ---------------------------------------------------------------- setup
    def reference_images(self, n_images_or_name):
        key = n_images_or_name
        name = {6: "periodic_6", 18: "periodic_18", 26: "periodic_26", 0: "open_boundaries",
                "open": "open_boundaries"}.get(key, key)
        return abi.BoundaryImages.in_dll(self.lib, name)

    def set_params(self, p: abi.Params):
        self.params = p
        if self.kind != "reference":
            return
        L = self.lib
        dbl = lambda n, v: setattr(C.c_double.in_dll(L, n), "value", float(v))  # noqa: E731
        i32 = lambda n, v: setattr(C.c_int.in_dll(L, n), "value", int(v))  # noqa: E731
        dbl("KAPPA", p.kappa)
        dbl("VORTEX_WIDTH", p.vortex_width)
        dbl("alpha", p.alpha)
        dbl("alpha_p", p.alpha_p)
        i32("use_mutual_friction", p.use_mutual_friction)
        i32("use_BH", p.use_bh)
        dbl("BH_resolution", p.bh_resolution)
        dbl("global_dl_min", p.dl_min)
        dbl("global_dl_max", p.dl_max)
        dbl("rec_dist", p.rec_dist)
        dbl("reconnection_angle_cutoff", p.reconnection_angle_cutoff)
        i32("small_loop_cutoff", p.small_loop_cutoff)
        i32("use_freq_filter", p.use_freq_filter)
        dbl("freq_to_cutoff", p.freq_to_cutoff)
        i32("global_num_threads", max(1, p.num_threads))
        i32("pin_mode", p.pin_mode)
        for name, src in (("vn_conf", p.vn), ("vs_conf", p.vs), ("vb_conf", p.vb)):
            dst = abi.ExtVel.in_dll(L, name)
            C.memmove(C.addressof(dst), C.addressof(src), C.sizeof(abi.ExtVel))

    def tangle(self, host) -> CTangle:
        return CTangle(self, host)

    # ------------------------------------------------------------- compute
    def _p(self):
        return C.byref(self.params)

    def update_tangents_normals(self, t: CTangle):
        fn = self.lib.orc_update_tangents_normals if self.kind == "port" else self.lib.update_tangents_normals
        fn(C.byref(t.ts))

    def update_velocities(self, t: CTangle, time=0.0):
        if self.kind == "port":
            self.lib.orc_update_velocities(C.byref(t.ts), time, self._p())
        else:
            self.lib.update_velocities(C.byref(t.ts), time)

    def update_tangle(self, t: CTangle, time=0.0):
        self.update_tangents_normals(t)
        self.update_velocities(t, time)

    def rk4_step(self, t: CTangle, time, dt):
        if self.kind == "port":
            self.lib.orc_rk4_step(C.byref(t.ts), time, dt, self._p())
        else:
            self.lib.rk4_step(C.byref(t.ts), time, dt)

    def reconnect(self, t: CTangle, time=0.0, log=False):
        if self.kind == "port":
            cap = max(16, t.n)
            lk = (C.c_int * cap)()
            ll = (C.c_int * cap)()
            n = self.lib.orc_reconnect(C.byref(t.ts), time, self._p(), lk, ll, cap)
            return (n, list(zip(lk[:min(n, cap)], ll[:min(n, cap)]))) if log else n
        n = self.lib.reconnect(C.byref(t.ts), time)
        return (n, None) if log else n

    def remesh(self, t: CTangle, mn, mx, time=0.0):
        if self.kind == "port":
            a, r = C.c_int(0), C.c_int(0)
            self.lib.orc_remesh(C.byref(t.ts), mn, mx, time, self._p(), C.byref(a), C.byref(r))
            return a.value, r.value
        self.lib.remesh(C.byref(t.ts), mn, mx, time)
        return None

    def eliminate_small_loops(self, t: CTangle):
        if self.kind == "port":
            return self.lib.orc_eliminate_small_loops(C.byref(t.ts), self._p())
        self.lib.eliminate_small_loops(C.byref(t.ts))
        return None

    def enforce_periodic(self, t: CTangle):
        fn = self.lib.orc_enforce_periodic_boundaries if self.kind == "port" else \
            self.lib.enforce_periodic_boundaries
        fn(C.byref(t.ts))

    def smooth(self, t: CTangle):
        assert self.kind == "port", "the reference's smoothing needs FFTW"
        self.lib.orc_smooth(C.byref(t.ts), self._p())

    def direct_velocities(self, t: CTangle, nodes, time=0.0):
        """update_velocity(k, tree=NULL) for the listed nodes; returns (vels, vs)."""
        nodes = np.ascontiguousarray(nodes, dtype=np.int32)
        if self.kind == "port":
            self.lib.orc_direct_velocities(C.byref(t.ts), nodes.ctypes.data_as(C.POINTER(C.c_int)),
                                           len(nodes), time, self._p())
        else:
            for k in nodes:
                self.lib.update_velocity(C.byref(t.ts), int(k), time, None)
        v = t.views()
        return np.array(v["vels"][nodes]), np.array(v["vs"][nodes])

    def node_interactions(self, t: CTangle, resolution: float, threads: int = 1):
        """Per-target (visits, accepts) of the reference tree at `resolution`
        over each node's 1 + n_img query points (int64 arrays of t.n)."""
        assert self.kind == "port"
        f = self.lib.orc_node_interactions
        f.argtypes = [_TS, C.c_double, C.c_int, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)]
        vis = np.zeros(t.n, dtype=np.int64)
        acc = np.zeros(t.n, dtype=np.int64)
        f(C.byref(t.ts), resolution, int(threads), vis.ctypes.data_as(C.POINTER(C.c_longlong)),
          acc.ctypes.data_as(C.POINTER(C.c_longlong)))
        return vis, acc

    def low_pass_filter(self, x, freq_to_cutoff):
        assert self.kind == "port"
        a = np.ascontiguousarray(x, dtype=np.float64).copy()
        self.lib.orc_low_pass_filter(a.ctypes.data_as(C.POINTER(C.c_double)), len(a), freq_to_cutoff)
        return a

    def step(self, t: CTangle, time, dt):
        assert self.kind == "port"
        nr = C.c_int(0)
        self.lib.orc_step(C.byref(t.ts), time, dt, self._p(), C.byref(nr))
        return nr.value


def reference_available() -> bool:
    return os.path.exists(REF_SO)


def sph_update_tangle(sph, params, threads: int = 1, tangents: bool = True, fast: bool = False) -> None:
    """The spherical fork's update_tangents_normals + update_velocities in the
    C restatement (oracle/ov_oracle_sph.c), in place on a workloads.SphTangle."""
    path = PORT_FAST_SO if fast else PORT_SO
    if not os.path.exists(path):
        build(ref=False)
    L = C.CDLL(path)
    f = L.orc_sph_update_tangle
    f.argtypes = [C.POINTER(abi.SphTangleState), C.POINTER(abi.SphParams), C.c_double, C.c_int, C.c_int]
    f.restype = C.c_int
    st = sph.state()
    rc = f(C.byref(st), C.byref(params), 0.0, int(threads), int(tangents))
    if rc:
        raise RuntimeError(f"oracle spherical update failed ({rc})")
