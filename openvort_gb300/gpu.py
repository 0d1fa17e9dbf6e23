"""Python host binding of libovgpu (ctypes over include/openvort_gpu.h).

This mirrors the reference's own operations on a tangle:

    ctx = Context()                      # one GPU context (stream, buffers)
    ctx.set_params(params)               # the reference's globals, explicit
    ctx.upload(host_tangle)              # struct tangle_state -> HBM
    ctx.update_tangle(t)                 # update_tangle (tangle.h:114)
    ctx.rk4_step(t, dt)                  # rk4_step (vortex_dynamics.c:50)
    ctx.download(host_tangle)            # HBM -> struct tangle_state

There is no CPU fallback: every call runs the CUDA library and raises
OVError when it reports a failure, or RuntimeError when the library or a GPU
is missing.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import abi

_LIB = None
LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "lib", "libovgpu.so")


class OVError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{abi.STATUS_NAMES.get(code, code)}: {msg}")
        self.code = code


def load(path: str | None = None):
    """Load libovgpu.so (built by openvort_gb300.build); raise if absent."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise RuntimeError(f"libovgpu.so not built ({path}); run `python -m openvort_gb300.build`")
    L = C.CDLL(path)
    P = C.c_void_p
    TS = C.POINTER(abi.TangleState)
    sig = {
        "ov_ctx_create": (C.c_int, [C.POINTER(P), C.c_int]),
        "ov_ctx_destroy": (C.c_int, [P]),
        "ov_last_error": (C.c_char_p, [P]),
        "ov_set_params": (C.c_int, [P, C.POINTER(abi.Params)]),
        "ov_set_precision": (C.c_int, [P, C.c_int]),
        "ov_set_walk": (C.c_int, [P, C.c_int]),
        "ov_get_walk": (C.c_int, [P]),
        "ov_ctx_stream": (P, [P]),
        "ov_upload_tangle": (C.c_int, [P, TS]),
        "ov_download_tangle": (C.c_int, [P, TS, C.c_uint]),
        "ov_capacity": (C.c_int, [P]),
        "ov_update_tangents_normals": (C.c_int, [P]),
        "ov_update_velocities": (C.c_int, [P, C.c_double]),
        "ov_update_tangle": (C.c_int, [P, C.c_double]),
        "ov_rk4_step": (C.c_int, [P, C.c_double, C.c_double]),
        "ov_direct_velocities": (C.c_int, [P, C.POINTER(C.c_int), C.c_int, C.c_double,
                                           C.POINTER(C.c_double), C.POINTER(C.c_double)]),
        "ov_enforce_periodic_boundaries": (C.c_int, [P]),
        "ov_eliminate_small_loops": (C.c_int, [P]),
        "ov_reconnect": (C.c_int, [P, C.c_double, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                   C.POINTER(C.c_int), C.c_int]),
        "ov_remesh": (C.c_int, [P, C.c_double, C.c_double, C.c_double]),
        "ov_smooth": (C.c_int, [P]),
        "ov_step": (C.c_int, [P, C.c_double, C.c_double]),
        "ov_get_stats": (C.c_int, [P, C.POINTER(abi.Stats)]),
        "ov_timer_start": (C.c_int, [P]),
        "ov_timer_stop": (C.c_int, [P, C.POINTER(C.c_float)]),
        "ov_flush_l2": (C.c_int, [P, C.c_size_t]),
        "ov_synchronize": (C.c_int, [P]),
        "ov_kernel_launches": (C.c_int64, [P]),
        "ov_params_default": (None, [C.POINTER(abi.Params)]),
        "ov_upload_tangle_fields": (C.c_int, [P, TS, C.c_uint]),
        "ov_set_phase_timing": (C.c_int, [P, C.c_int]),
        "ov_phase_times": (C.c_int, [P, C.POINTER(C.c_float)]),
        "ov_set_node_counting": (C.c_int, [P, C.c_int]),
        "ov_inject_alloc_failure": (C.c_int, [P, C.c_int]),
        "ov_set_depth_policy": (C.c_int, [P, C.c_int]),
        "ov_get_node_counts": (C.c_int, [P, C.c_int, C.POINTER(C.c_uint), C.POINTER(C.c_uint), C.c_int]),
        "ov_measure_fma_peak": (C.c_int, [P, C.c_int, C.POINTER(C.c_double)]),
        "ov_set_rk4_graph": (C.c_int, [P, C.c_int]),
        "ov_set_host_access": (C.c_int, [P, C.c_int]),
        "ov_get_host_access": (C.c_int, [P]),
        "ov_tangle_info": (C.c_int, [P, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]),
        "ov_upload_ensemble": (C.c_int, [P, C.POINTER(TS), C.POINTER(abi.Params), C.c_int, C.c_double]),
        "ov_ensemble_size": (C.c_int, [P]),
        "ov_member_info": (C.c_int, [P, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]),
        "ov_download_member": (C.c_int, [P, C.c_int, TS, C.c_uint]),
        "ov_set_member_params": (C.c_int, [P, C.c_int, C.POINTER(abi.Params)]),
        "ov_get_tuning": (C.c_int, [P, C.POINTER(abi.Tuning)]),
        "ov_set_tuning": (C.c_int, [P, C.POINTER(abi.Tuning)]),
        "ov_autotune": (C.c_int, [P, C.c_double, C.POINTER(abi.Tuning), C.POINTER(C.c_float)]),
        "ov_step_times": (C.c_int, [P, C.POINTER(C.c_double), C.c_int]),
        "ov_enforce_wall_boundaries": (C.c_int, [P, C.c_double]),
        "ov_write_frame": (C.c_int, [TS, C.c_char_p, C.c_int]),
        "ov_frame_slots": (C.c_int, [C.c_char_p, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                     C.POINTER(C.c_int)]),
        "ov_read_frame": (C.c_int, [C.c_char_p, C.c_int, TS]),
        "ov_save_frame": (C.c_int, [P, C.c_int, C.c_char_p, C.c_int]),
        "ov_direct_sums_bounded": (C.c_int, [P, C.POINTER(C.c_int), C.c_int, C.c_int, C.POINTER(C.c_double)]),
        "ov_add_loop": (C.c_int, [P, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_double]),
        "ov_add_line_in_zdir": (C.c_int, [P, C.c_int, C.c_double, C.c_double, C.c_int]),
        "ov_set_injection": (C.c_int, [P, C.c_int, C.POINTER(abi.Injection)]),
        "ov_get_injection": (C.c_int, [P, C.c_int, C.POINTER(abi.Injection)]),
        "ov_inject_vortices": (C.c_int, [P, C.c_double]),
        "ov_erand48": (C.c_double, [C.POINTER(C.c_ushort)]),
        "ov_sph_params_default": (None, [C.POINTER(abi.SphParams)]),
        "ov_sph_update_tangents_normals": (C.c_int, [P, C.POINTER(abi.SphTangleState), C.POINTER(abi.SphParams)]),
        "ov_sph_update_velocities": (C.c_int, [P, C.POINTER(abi.SphTangleState), C.POINTER(abi.SphParams),
                                               C.c_double]),
        "ov_sph_update_tangle": (C.c_int, [P, C.POINTER(abi.SphTangleState), C.POINTER(abi.SphParams), C.c_double]),
        "ov_sph_helium": (C.c_int, [C.c_double, C.POINTER(C.c_double)]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = L
    return L


def declared_symbols() -> list[str]:
    """Every function declared in include/*.h (for the export check)."""
    import re
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")
    names = []
    for f in sorted(os.listdir(inc)):
        if not f.endswith(".h"):
            continue
        txt = open(os.path.join(inc, f)).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        for m in re.finditer(r"^\s*(?:[A-Za-z_][\w\s\*]*?)\b((?:ov|ovd)_\w+)\s*\(", txt, flags=re.M):
            names.append(m.group(1))
    return sorted(set(names))


def sph_params_default() -> abi.SphParams:
    p = abi.SphParams()
    load().ov_sph_params_default(C.byref(p))
    return p


def sph_helium(T: float) -> np.ndarray:
    """The spherical fork's He II model at T (host): superfluid, total and
    normal density, entropy, alpha(T), alpha'(T)."""
    out = (C.c_double * 6)()
    rc = load().ov_sph_helium(float(T), out)
    if rc:
        raise OVError(rc, f"temperature {T} outside the model's range")
    return np.array(out[:])


def erand48(state) -> float:
    """One draw of the injection stream from `state` (a ctypes c_ushort * 3,
    advanced in place); host only."""
    return load().ov_erand48(state)


def write_frame(host, path: str, digits: int = 15):
    """save_tangle of a host tangle (no GPU needed)."""
    st = host.state()
    rc = load().ov_write_frame(C.byref(st), path.encode(), digits)
    if rc:
        raise OVError(rc, f"writing {path}")


def read_frame(path: str, n0: int = 1):
    """load_tangle into a fresh host tangle made as create_tangle(n0) would
    be, grown as the file needs (no GPU needed); returns the HostTangle and
    its (next_empty, total_empty)."""
    from .workloads import HostTangle
    L = load()
    n, ne, te = C.c_int(0), C.c_int(0), C.c_int(0)
    rc = L.ov_frame_slots(path.encode(), n0, C.byref(n), C.byref(ne), C.byref(te))
    if rc:
        raise OVError(rc, f"reading {path}")
    ht = HostTangle(np.zeros((n.value, 3)), np.full(n.value, -1), np.full(n.value, -1), np.zeros(3), np.ones(3),
                    n_images=0, status=np.full(n.value, abi.OV_EMPTY))
    st = ht.state()
    st.next_empty, st.total_empty = 0, n0   # as create_tangle(n0) leaves them
    rc = L.ov_read_frame(path.encode(), n0, C.byref(st))
    if rc:
        raise OVError(rc, f"reading {path}")
    return ht, (st.next_empty, st.total_empty)   # the call filled ht's arrays in place


def _grown(host, n: int):
    """`host`, or a copy of it grown to n slots (new slots EMPTY)."""
    from .workloads import HostTangle
    if n <= host.n:
        return host
    pos = np.zeros((n, 3))
    pos[:host.n] = host.pos
    fwd = np.full(n, -1)
    rev = np.full(n, -1)
    st = np.full(n, abi.OV_EMPTY)
    fwd[:host.n], rev[:host.n], st[:host.n] = host.conn[:, 0], host.conn[:, 1], host.stat[:, 0]
    return HostTangle(pos, fwd, rev, host.box_lo, host.box_hi, n_images=host.n_images, status=st)


class Context:
    """One libovgpu context on one GPU."""

    def __init__(self, device: int = 0, params: abi.Params | None = None, precision: int = abi.OV_PREC_FP64):
        self.lib = load()
        self._h = C.c_void_p()
        rc = self.lib.ov_ctx_create(C.byref(self._h), device)
        if rc != 0:
            raise OVError(rc, "ov_ctx_create failed (no usable CUDA device?)")
        if params is not None:
            self.set_params(params)
        self.set_precision(precision)
        self._host = None

    # -------------------------------------------------------------- plumbing
    def _check(self, rc: int):
        if rc != 0:
            raise OVError(rc, self.lib.ov_last_error(self._h).decode())

    def close(self):
        if self._h:
            self.lib.ov_ctx_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def set_params(self, p: abi.Params):
        self.params = p
        self._check(self.lib.ov_set_params(self._h, C.byref(p)))

    def set_rk4_graph(self, on: bool):
        self._check(self.lib.ov_set_rk4_graph(self._h, int(on)))

    def set_host_access(self, direct: bool):
        """In-place uploads/downloads of the caller's arrays where the device
        reads pageable host memory (True, the default), or staged copies."""
        self._check(self.lib.ov_set_host_access(self._h, int(direct)))

    @property
    def host_access_direct(self) -> bool:
        return bool(self.lib.ov_get_host_access(self._h))

    def set_precision(self, prec: int):
        self._check(self.lib.ov_set_precision(self._h, prec))

    def set_walk(self, walk: int):
        """OV_PREC_FP64's tree walk: abi.OV_WALK_SPLIT (default) or abi.OV_WALK_FP64."""
        self._check(self.lib.ov_set_walk(self._h, walk))

    @property
    def walk(self) -> int:
        return self.lib.ov_get_walk(self._h)

    # ----------------------------------------------------------------- data
    def upload(self, host):
        """host: workloads.HostTangle (or anything with .state())."""
        self._host = host
        self._state = host.state()
        self._check(self.lib.ov_upload_tangle(self._h, C.byref(self._state)))

    def upload_fields(self, host, fields: int):
        self._host = host
        self._state = host.state()
        self._check(self.lib.ov_upload_tangle_fields(self._h, C.byref(self._state), fields))

    def upload_ensemble(self, hosts, params, headroom: float = 2.0):
        """hosts: HostTangles; params: one abi.Params per member."""
        self._members = list(hosts)
        self._mstates = [h.state() for h in self._members]
        arr = (C.POINTER(abi.TangleState) * len(hosts))(*[C.pointer(st) for st in self._mstates])
        parr = (abi.Params * len(params))(*params)
        self._check(self.lib.ov_upload_ensemble(self._h, arr, parr, len(hosts), headroom))
        self._host = None

    @property
    def ensemble_size(self) -> int:
        return self.lib.ov_ensemble_size(self._h)

    def member_info(self, i: int) -> tuple[int, int, int]:
        n, ne, te = C.c_int(0), C.c_int(0), C.c_int(0)
        self._check(self.lib.ov_member_info(self._h, i, C.byref(n), C.byref(ne), C.byref(te)))
        return n.value, ne.value, te.value

    def download_member(self, i: int, host=None, fields: int = abi.OV_F_ALL):
        """Download member i into `host` (default: the uploaded one), grown
        to the member's slot count when remesh has expanded it."""
        host = host if host is not None else self._members[i]
        n, _, _ = self.member_info(i)
        host = _grown(host, n)
        st = host.state()
        self._check(self.lib.ov_download_member(self._h, i, C.byref(st), fields))
        return host

    def set_member_params(self, i: int, p: abi.Params):
        self._check(self.lib.ov_set_member_params(self._h, i, C.byref(p)))

    def get_tuning(self) -> abi.Tuning:
        tu = abi.Tuning()
        self._check(self.lib.ov_get_tuning(self._h, C.byref(tu)))
        return tu

    def set_tuning(self, warps_per_block: int = 4, query_groups: int = 0, blocks_per_sm: int = 0,
                   largest_first: int = 1, high_occupancy: int = 0):
        tu = abi.Tuning(warps_per_block, query_groups, blocks_per_sm, largest_first, high_occupancy)
        self._check(self.lib.ov_set_tuning(self._h, C.byref(tu)))

    def autotune(self, t: float = 0.0) -> tuple[dict, float]:
        tu, ms = abi.Tuning(), C.c_float(0)
        self._check(self.lib.ov_autotune(self._h, t, C.byref(tu), C.byref(ms)))
        return {f: getattr(tu, f) for f, _ in tu._fields_}, ms.value

    def tangle_info(self) -> tuple[int, int, int]:
        n, ne, te = C.c_int(0), C.c_int(0), C.c_int(0)
        self._check(self.lib.ov_tangle_info(self._h, C.byref(n), C.byref(ne), C.byref(te)))
        return n.value, ne.value, te.value

    def download_resized(self, host):
        """Download into a copy of `host` grown to the context's slot count."""
        n, _, _ = self.tangle_info()
        return self.download(_grown(host, n))

    def download(self, host=None, fields: int = abi.OV_F_ALL):
        host = host or self._host
        st = host.state()
        self._check(self.lib.ov_download_tangle(self._h, C.byref(st), fields))
        return host

    # -------------------------------------------------------------- compute
    def update_tangents_normals(self):
        self._check(self.lib.ov_update_tangents_normals(self._h))

    def update_velocities(self, t: float = 0.0):
        self._check(self.lib.ov_update_velocities(self._h, t))

    def update_tangle(self, t: float = 0.0):
        self._check(self.lib.ov_update_tangle(self._h, t))

    def rk4_step(self, t: float, dt: float):
        self._check(self.lib.ov_rk4_step(self._h, t, dt))

    def direct_velocities(self, nodes, t: float = 0.0):
        nodes = np.ascontiguousarray(nodes, dtype=np.int32)
        v = np.zeros((len(nodes), 3))
        s = np.zeros((len(nodes), 3))
        dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))  # noqa: E731
        self._check(self.lib.ov_direct_velocities(self._h, nodes.ctypes.data_as(C.POINTER(C.c_int)),
                                                  len(nodes), t, dp(v), dp(s)))
        return v, s

    def direct_sums_bounded(self, nodes, precision: int = abi.OV_PREC_MIXED):
        """Nonlocal direct sums of `nodes`: (sums[n,3], bound[n], magnitude[n])."""
        nodes = np.ascontiguousarray(nodes, dtype=np.int32)
        out = np.zeros((len(nodes), 5))
        self._check(self.lib.ov_direct_sums_bounded(self._h, nodes.ctypes.data_as(C.POINTER(C.c_int)), len(nodes),
                                                    precision, out.ctypes.data_as(C.POINTER(C.c_double))))
        return out[:, :3].copy(), out[:, 3].copy(), out[:, 4].copy()

    def enforce_periodic(self):
        self._check(self.lib.ov_enforce_periodic_boundaries(self._h))

    def save_frame(self, path: str, member: int = 0, digits: int = 15):
        self._check(self.lib.ov_save_frame(self._h, member, path.encode(), digits))

    def add_loop(self, center, direction, radius: float, member: int = 0):
        """add_loop (vortex_injection.c:49): a ring of FREE nodes."""
        c3 = (C.c_double * 3)(*map(float, center))
        d3 = (C.c_double * 3)(*map(float, direction))
        self._check(self.lib.ov_add_loop(self._h, member, c3, d3, float(radius)))

    def add_line_in_zdir(self, x: float, y: float, direction: int, member: int = 0):
        """add_line_in_zdir (vortex_injection.c:267): a pinned line along z."""
        self._check(self.lib.ov_add_line_in_zdir(self._h, member, float(x), float(y), int(direction)))

    def set_injection(self, inj: abi.Injection, member: int = -1):
        self._check(self.lib.ov_set_injection(self._h, member, C.byref(inj)))

    def get_injection(self, member: int = 0) -> abi.Injection:
        out = abi.Injection()
        self._check(self.lib.ov_get_injection(self._h, member, C.byref(out)))
        return out

    def inject_vortices(self, t: float):
        self._check(self.lib.ov_inject_vortices(self._h, float(t)))

    def sph_update(self, sph, params: abi.SphParams, t: float = 0.0, tangents: bool = True, velocities: bool = True):
        """The spherical fork's update_tangents_normals / update_velocities /
        update_tangle on a workloads.SphTangle (arrays updated in place)."""
        st = sph.state()
        if tangents and velocities:
            rc = self.lib.ov_sph_update_tangle(self._h, C.byref(st), C.byref(params), t)
        elif tangents:
            rc = self.lib.ov_sph_update_tangents_normals(self._h, C.byref(st), C.byref(params))
        else:
            rc = self.lib.ov_sph_update_velocities(self._h, C.byref(st), C.byref(params), t)
        self._check(rc)
        return sph

    def enforce_walls(self, t: float = 0.0):
        self._check(self.lib.ov_enforce_wall_boundaries(self._h, t))

    def eliminate_small_loops(self):
        self._check(self.lib.ov_eliminate_small_loops(self._h))

    def reconnect(self, t: float = 0.0, log: bool = False):
        n = C.c_int(0)
        cap = max(16, self.capacity)
        lk, ll = (C.c_int * cap)(), (C.c_int * cap)()
        self._check(self.lib.ov_reconnect(self._h, t, C.byref(n), lk, ll, cap))
        if log:
            return n.value, list(zip(lk[:min(n.value, cap)], ll[:min(n.value, cap)]))
        return n.value

    def remesh(self, mn: float, mx: float, t: float = 0.0):
        self._check(self.lib.ov_remesh(self._h, mn, mx, t))

    def smooth(self):
        self._check(self.lib.ov_smooth(self._h))

    def step(self, t: float, dt: float):
        self._check(self.lib.ov_step(self._h, t, dt))

    STEP_PASSES = ("small_loops", "reconnect", "smooth", "periodic", "remesh", "update_tangle", "rk4_step",
                   "total", "reconnect_pairs", "reconnect_direct_sums", "reconnect_decisions", "reconnect_push",
                   "reconnect_fetch", "reconnect_correct", "reconnect_fp64", "reconnect_exact")

    def step_times(self) -> dict:
        """Host wall ms of the last step(), per pass."""
        ms = (C.c_double * 16)()
        self._check(self.lib.ov_step_times(self._h, ms, 16))
        return dict(zip(self.STEP_PASSES, list(ms)))

    @property
    def capacity(self) -> int:
        return self.lib.ov_capacity(self._h)

    def stats(self) -> dict:
        s = abi.Stats()
        self._check(self.lib.ov_get_stats(self._h, C.byref(s)))
        return {f: getattr(s, f) for f, _ in s._fields_}

    # --------------------------------------------------------------- timing
    def timer_start(self):
        self._check(self.lib.ov_timer_start(self._h))

    def timer_stop(self) -> float:
        ms = C.c_float(0)
        self._check(self.lib.ov_timer_stop(self._h, C.byref(ms)))
        return ms.value

    def flush_l2(self, nbytes: int = 256 << 20):
        self._check(self.lib.ov_flush_l2(self._h, nbytes))

    def synchronize(self):
        self._check(self.lib.ov_synchronize(self._h))

    def set_phase_timing(self, on: bool = True):
        self._check(self.lib.ov_set_phase_timing(self._h, int(on)))

    def phase_times(self) -> list[float]:
        ms = (C.c_float * 3)()
        self._check(self.lib.ov_phase_times(self._h, ms))
        return list(ms)

    def set_depth_policy(self, strict: bool):
        """strict: nodes sharing the deepest tree cell raise OV_ERR_DEPTH;
        otherwise (default) that cell is one leaf and the call succeeds."""
        self._check(self.lib.ov_set_depth_policy(self._h, int(strict)))

    def inject_alloc_failure(self, after: int = 0):
        """The allocation after `after` more successful ones fails (-1: off)."""
        self._check(self.lib.ov_inject_alloc_failure(self._h, int(after)))

    def set_node_counting(self, on: bool = True):
        self._check(self.lib.ov_set_node_counting(self._h, int(on)))

    def node_counts(self, member: int = 0, n: int | None = None):
        """(visits, accepts) per slot of a member (or the tangle) in the last
        evaluation (node counting on)."""
        n = self.member_info(member)[0] if n is None else n
        vis = np.zeros(n, dtype=np.uint32)
        acc = np.zeros(n, dtype=np.uint32)
        self._check(self.lib.ov_get_node_counts(self._h, member, vis.ctypes.data_as(C.POINTER(C.c_uint)),
                                                acc.ctypes.data_as(C.POINTER(C.c_uint)), n))
        return vis.astype(np.int64), acc.astype(np.int64)

    def fma_peak_tflops(self, precision: int) -> float:
        v = C.c_double(0)
        self._check(self.lib.ov_measure_fma_peak(self._h, precision, C.byref(v)))
        return v.value

    @property
    def kernel_launches(self) -> int:
        return self.lib.ov_kernel_launches(self._h)
