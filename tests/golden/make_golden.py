"""Generate the golden vectors in tests/golden/ from OpenVort itself.

Runs the reference compiled from its own sources (oracle/Makefile, target
``ref``: needs the OpenVort checkout, so this script runs where that exists)
and stores inputs and outputs as small .npz files.  The GPU machine has no
reference checkout; there the tests compare against these files and against
the C restatement (oracle/ov_oracle.c), which these files also pin.

Usage:  python tests/golden/make_golden.py [walls | injection | spherical | events]
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from openvort_gb300 import workloads as W  # noqa: E402
from oracle.pyoracle import Checker, build  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def params_dict(p):
    return {f: getattr(p, f) for f, _ in p._fields_ if f not in ("vn", "vs", "vb")} | {
        f"{k}_{g}": (list(getattr(getattr(p, k), g).p) if g == "direction" else getattr(getattr(p, k), g))
        for k in ("vn", "vs", "vb") for g in ("type", "strength", "direction")}


def save(name, **arrays):
    path = os.path.join(OUT, name)
    np.savez_compressed(path, **arrays)
    print("wrote", path, f"{os.path.getsize(path) / 1024:.1f} KiB")


def tangle_arrays(ht):
    return dict(pos=ht.pos, conn=ht.conn, status=ht.stat, box_lo=ht.box_lo, box_hi=ht.box_hi,
                n_images=ht.n_images)


def ref_step(c, t, time, dt):
    """main.c:125-141 for a periodic box without injection or smoothing."""
    c.eliminate_small_loops(t)
    n = c.reconnect(t, 0.0)
    c.eliminate_small_loops(t)
    c.enforce_periodic(t)
    c.remesh(t, c.params.dl_min, c.params.dl_max, 0.0)
    c.eliminate_small_loops(t)
    c.update_tangle(t, time)
    c.rk4_step(t, time, dt)
    c.enforce_periodic(t)
    return n


def port_step(c, t, time, dt):
    """ref_step in the C restatement, returning the reconnection log too."""
    c.eliminate_small_loops(t)
    n, log = c.reconnect(t, 0.0, log=True)
    c.eliminate_small_loops(t)
    c.enforce_periodic(t)
    c.remesh(t, c.params.dl_min, c.params.dl_max, 0.0)
    c.eliminate_small_loops(t)
    c.update_tangle(t, time)
    c.rk4_step(t, time, dt)
    c.enforce_periodic(t)
    return n, log


def event_trajectory(ref, ht, p, n_steps, dt, name):
    """n_steps main-loop steps (main.c:125-141, periodic box, no smoothing)
    of the reference, with the event log: reconnections per step, the
    (k, l) pairs in order (from the C restatement run beside it, which must
    leave the reference's connections, status and positions bit for bit at
    every step), the slot arrays after every step whose topology changed,
    and positions at a few steps."""
    port = Checker("port")
    p.num_threads = 8
    ref.set_params(p)
    port.set_params(p)
    t, u = ref.tangle(ht), port.tangle(ht)
    recs, pairs, n_slots, ev_steps, ev_conn, ev_status, traj, traj_steps = [], [], [], [], [], [], [], []
    keep = {0, 4, 9, 19, 49, 99, 149, n_steps - 1}
    prev = (t.copy("conn"), t.copy("status"))
    v0 = None
    for s in range(n_steps):
        n = ref_step(ref, t, s * dt, dt)
        n_port, log = port_step(port, u, s * dt, dt)
        conn, status, pos = t.copy("conn"), t.copy("status"), t.copy("pos")
        assert n_port == n, (s, n, n_port)
        assert np.array_equal(u.copy("conn"), conn) and np.array_equal(u.copy("status"), status), s
        assert np.array_equal(u.copy("pos"), pos), s
        recs.append(n)
        pairs += [(s, k, l) for k, l in log]
        n_slots.append(t.n)
        if s == 0:
            v0 = t.copy("vels")
        if conn.shape != prev[0].shape or not (np.array_equal(conn, prev[0]) and np.array_equal(status, prev[1])):
            ev_steps.append(s)
            ev_conn.append(conn)
            ev_status.append(status)
        prev = (conn, status)
        if s in keep or (ev_steps and ev_steps[-1] == s):
            live = status[:, 0] != -1
            traj.append(np.where(live[:, None], pos, 0.0))
            traj_steps.append(s)
    cap = max(n_slots)

    def pad(a, fill):
        out = np.full((cap,) + a.shape[1:], fill, dtype=a.dtype)
        out[:len(a)] = a
        return out

    out = dict(tangle_arrays(ht), dt=dt, recs=np.array(recs), n_slots=np.array(n_slots),
               rec_pairs=np.array(pairs, dtype=np.int32).reshape(-1, 3),
               event_steps=np.array(ev_steps, dtype=np.int32), traj=np.stack([pad(a, 0.0) for a in traj]),
               traj_steps=np.array(traj_steps), vels_step0=v0, conn_final=t.copy("conn"),
               status_final=t.copy("status"))
    if ev_steps:
        out["event_conn"] = np.stack([pad(a, -1) for a in ev_conn])
        out["event_status"] = np.stack([pad(a, -1) for a in ev_status])
    print(name, "reconnections", sum(recs), "pairs", len(pairs), "event steps", ev_steps)
    save(name, **out)
    t.free()
    u.free()


WALL_SETS = ("wall_1_open", "wall_1_18", "wall_1_26", "wall_2_4", "wall_2_2", "wall_parallel_planes",
             "wall_canal", "open", "periodic_6")


def walls(ref):
    """Velocities under the reference's wall (mirror-image) and open boundary
    configurations: one random-walk tangle, BH at theta 0.4 and direct sums."""
    base = W.random_walk_tangle(8, 48, D=0.1, seed=17)
    p = W.config_params("rw")
    p.num_threads = 8
    ref.set_params(p)
    out = dict(pos=base.pos, conn=base.conn, status=base.stat, box_lo=base.box_lo, box_hi=base.box_hi,
               sets=np.array(WALL_SETS))
    nodes = np.arange(0, base.n, 13, dtype=np.int32)
    out["direct_nodes"] = nodes
    for name in WALL_SETS:
        ht = W.HostTangle(base.pos.copy(), base.conn[:, 0].copy(), base.conn[:, 1].copy(), base.box_lo,
                          base.box_hi, image_set=name)
        t = ref.tangle(ht)
        ref.update_tangle(t, 0.0)
        out[f"{name}_vels"], out[f"{name}_vs"] = t.copy("vels"), t.copy("vs")
        dv, dvs = ref.direct_velocities(t, nodes, 0.0)
        out[f"{name}_direct_vels"], out[f"{name}_direct_vs"] = dv, dvs
        t.free()
    save("walls.npz", **out)


def wall_rings(n_rings=6, radius=0.012, npts=40, seed=23):
    """Rings in a box with mirror walls in z (wall_2_4), placed so that some
    dip through the bottom or top wall and some pass within rec_dist of it."""
    rng = np.random.default_rng(seed)
    pos, fwd, rev = [], [], []
    for r in range(n_rings):
        cx, cy = rng.uniform(0.02, 0.08, 2)
        top = r % 2 == 1
        gap = [-0.004, 0.0002, 0.0, -0.001, 0.00035, 0.003][r % 6]
        cz = (0.1 - radius - gap) if top else (radius + gap)
        phi = 2 * np.pi * np.arange(npts) / npts
        tilt = rng.uniform(-0.3, 0.3)
        x = cx + radius * np.cos(phi) * np.cos(tilt)
        y = cy + radius * np.cos(phi) * np.sin(tilt)
        z = cz + radius * np.sin(phi)
        base = r * npts
        k = np.arange(npts)
        pos.append(np.stack([x, y, z], 1))
        fwd.append(base + (k + 1) % npts)
        rev.append(base + (k - 1) % npts)
    return W.HostTangle(np.concatenate(pos), np.concatenate(fwd), np.concatenate(rev), np.zeros(3),
                        np.full(3, 0.1), image_set="wall_2_4")


def wall_steps(ref):
    """enforce_wall_boundaries on its own, then three main-loop steps
    (main.c:125-141 without injection and smoothing) under mirror walls."""
    import ctypes as C
    ht = wall_rings()
    p = W.config_params("rings8", rec_dist=8e-4)
    p.num_threads = 8
    ref.set_params(p)
    t = ref.tangle(ht)
    ref.lib.enforce_wall_boundaries.argtypes = [C.c_void_p, C.c_double]
    ref.lib.enforce_wall_boundaries(C.addressof(t.ts), 0.0)
    out = dict(pos=ht.pos, conn=ht.conn, status=ht.stat, box_lo=ht.box_lo, box_hi=ht.box_hi)
    out["enf_N"], out["enf_pos"], out["enf_conn"], out["enf_status"] = t.n, t.copy("pos"), t.copy("conn"), \
        t.copy("status")
    # the reference's frame file of this state
    out["enf_vels"], out["enf_tangents"], out["enf_normals"] = t.copy("vels"), t.copy("tangents"), \
        t.copy("normals")
    ref.lib.save_tangle.argtypes = [C.c_char_p, C.c_void_p]
    ref.lib.save_tangle(os.path.join(OUT, "frame_walls.txt").encode(), C.addressof(t.ts))
    dt = 5e-5
    recs, conns, stats, poss, ns = [], [], [], [], []
    for s_ in range(3):
        ref.lib.enforce_wall_boundaries(C.addressof(t.ts), 0.0)
        recs.append(ref_step(ref, t, s_ * dt, dt))
        conns.append(t.copy("conn"))
        stats.append(t.copy("status"))
        poss.append(t.copy("pos"))
        ns.append(t.n)
    nmax = max(ns)
    pad = lambda a, fill: np.concatenate([a, np.full((nmax - len(a),) + a.shape[1:], fill, a.dtype)])  # noqa: E731
    out["recs"], out["dt"], out["steps_N"] = np.array(recs), dt, np.array(ns)
    out["steps_conn"] = np.stack([pad(a, -1) for a in conns])
    out["steps_status"] = np.stack([pad(a, -1) for a in stats])
    out["steps_pos"] = np.stack([pad(a, 0.0) for a in poss])
    # EMPTY slots hold whatever realloc left there: store zeros
    out["enf_pos"][out["enf_status"][:, 0] == -1] = 0.0
    for s_ in range(3):
        out["steps_pos"][s_][out["steps_status"][s_][:, 0] == -1] = 0.0
    t.free()
    save("wall_steps.npz", **out)


def _libc():
    import ctypes as C
    libc = C.CDLL("libc.so.6")
    libc.drand48.restype = C.c_double
    libc.srand48.argtypes = [C.c_long]
    return libc


def _set_injection(ref, inj):
    import ctypes as C
    L = ref.lib
    C.c_int.in_dll(L, "loop_injection").value = inj["loop_injection"]
    C.c_double.in_dll(L, "loop_injection_frequency").value = inj["loop_frequency"]
    C.c_int.in_dll(L, "line_injection").value = inj["line_injection"]
    C.c_int.in_dll(L, "line_injection_n").value = inj["line_n"]
    C.c_double.in_dll(L, "line_injection_frequency").value = inj["line_frequency"]
    C.c_int.in_dll(L, "line_injection_polarized").value = inj["line_polarized"]


def _state(t):
    return dict(N=t.n, pos=t.copy("pos"), conn=t.copy("conn"), status=t.copy("status"),
                next_empty=t.ts.next_empty, total_empty=t.ts.total_empty)


def injection(ref):
    """add_loop / add_line_in_zdir on a wall tangle with a freed ring (slot
    reuse, pool doubling, both branches of perpendicular), and the drand48
    stream the injection draws from."""
    import ctypes as C
    ht = wall_rings()
    ring = slice(2 * 40, 3 * 40)   # free the third ring's slots
    ht.stat[ring, 0] = -1
    ht.conn[ring] = -1
    p = W.config_params("rings8", rec_dist=8e-4)
    out = dict(pos=ht.pos, conn=ht.conn, status=ht.stat, box_lo=ht.box_lo, box_hi=ht.box_hi)
    V = C.c_double * 3
    calls = [("loop", (0.05, 0.05, 0.05), (1.0, 0.0, 0.0), 0.004), ("loop", (0.03, 0.06, 0.02), (0.3, -0.5, 0.8), 0.02),
             ("line", 0.031, 0.077, +1), ("line", 0.062, 0.018, -1), ("loop", (0.07, 0.02, 0.09), (0, 0, -1), 0.009)]
    ref.lib.add_loop.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_double]
    ref.lib.add_line_in_zdir.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_int]
    for k, call in enumerate(calls):
        p.pin_mode = 1 if k < 3 else 2   # PINNED, then PINNED_SLIP for the second line
        ref.set_params(p)
        if k == 0:
            t = ref.tangle(ht)
        if call[0] == "loop":
            ref.lib.add_loop(C.addressof(t.ts), C.byref(V(*call[1])), C.byref(V(*call[2])), call[3])
        else:
            ref.lib.add_line_in_zdir(C.addressof(t.ts), call[1], call[2], call[3])
        for key, v in _state(t).items():
            out[f"c{k}_{key}"] = v
        # EMPTY slots hold whatever realloc left there
        out[f"c{k}_pos"][out[f"c{k}_status"][:, 0] == -1] = 0.0
    t.free()
    libc = _libc()
    libc.srand48(20240607)
    out["rand_seed"] = 20240607
    out["rand_draws"] = np.array([libc.drand48() for _ in range(64)])
    save("inject.npz", **out)


INJECT_CONF = dict(loop_injection=1, loop_frequency=2e4, line_injection=1, line_n=1, line_frequency=1e4,
                   line_polarized=1, seed=777)


def inject_steps(ref):
    """inject_vortices then the main-loop body (main.c:123-141 without
    smoothing) for three steps under mirror walls in z."""
    import ctypes as C
    ht = wall_rings()
    p = W.config_params("rings8", rec_dist=8e-4)
    p.num_threads = 8
    ref.set_params(p)
    _set_injection(ref, INJECT_CONF)
    libc = _libc()
    libc.srand48(INJECT_CONF["seed"])
    t = ref.tangle(ht)
    ref.lib.enforce_wall_boundaries.argtypes = [C.c_void_p, C.c_double]
    ref.lib.inject_vortices.argtypes = [C.c_void_p, C.c_double]
    dt = 5e-5
    out = dict(pos=ht.pos, conn=ht.conn, status=ht.stat, box_lo=ht.box_lo, box_hi=ht.box_hi, dt=dt,
               **{f"inj_{k}": v for k, v in INJECT_CONF.items()})
    recs, states = [], []
    for s_ in range(3):
        ref.lib.inject_vortices(C.addressof(t.ts), s_ * dt)
        ref.lib.enforce_wall_boundaries(C.addressof(t.ts), 0.0)
        recs.append(ref_step(ref, t, s_ * dt, dt))
        states.append(_state(t))
    out["next_draw"] = libc.drand48()
    nmax = max(st["N"] for st in states)
    pad = lambda a, fill: np.concatenate([a, np.full((nmax - len(a),) + a.shape[1:], fill, a.dtype)])  # noqa: E731
    out["recs"], out["steps_N"] = np.array(recs), np.array([st["N"] for st in states])
    out["steps_conn"] = np.stack([pad(st["conn"], -1) for st in states])
    out["steps_status"] = np.stack([pad(st["status"], -1) for st in states])
    out["steps_pos"] = np.stack([pad(st["pos"], 0.0) for st in states])
    for s_ in range(3):
        out["steps_pos"][s_][out["steps_status"][s_][:, 0] == -1] = 0.0
    t.free()
    save("inject_steps.npz", **out)


class _quiet_stdout:
    """The spherical fork prints from its inner loops: silence fd 1 around calls."""

    def __enter__(self):
        import sys as _s
        _s.stdout.flush()
        self.saved = os.dup(1)
        self.null = os.open(os.devnull, os.O_WRONLY)
        os.dup2(self.null, 1)

    def __exit__(self, *exc):
        import ctypes as C
        C.CDLL(None).fflush(None)   # C stdio's buffer goes to the silenced descriptor
        os.dup2(self.saved, 1)
        os.close(self.null)
        os.close(self.saved)


SPH_CASES = {"plain": dict(use_temperature=0), "temperature": dict(use_temperature=1)}


def spherical():
    """The spherical fork's update_tangents_normals and update_velocities
    (outer surface open) on seeded rings in its default section, a radial
    line pinned on both surfaces, and EMPTY slots; with and without the He II
    temperature model.  Also the model's values on a grid of temperatures."""
    import ctypes as C
    from openvort_gb300 import abi
    L = C.CDLL(os.path.join(ROOT, "oracle", "_ref", "libovref_sph.so"))
    TS = C.POINTER(abi.SphTangleState)
    L.create_tangle.argtypes = [TS, C.c_size_t]
    L.free_tangle.argtypes = [TS]
    L.update_tangents_normals.argtypes = [TS]
    L.update_velocities.argtypes = [TS, C.c_double]
    sph = W.spherical_tangle()
    out = dict(pos=sph.pos, conn=sph.conn, status=sph.stat, domain=np.array(sph.domain))
    dbl = lambda n, v: setattr(C.c_double.in_dll(L, n), "value", float(v))  # noqa: E731
    i32 = lambda n, v: setattr(C.c_int.in_dll(L, n), "value", int(v))  # noqa: E731
    for tag, case in SPH_CASES.items():
        dbl("KAPPA", 9.97e-4); dbl("VORTEX_WIDTH", 1e-8); dbl("alpha", 0.034); dbl("alpha_p", 1.383e-2)
        i32("use_mutual_friction", 1); dbl("BH_resolution", 0.4); dbl("global_dl_min", 0.5e-3)
        dbl("global_dl_max", 1.5e-3); dbl("q_dot", 0.03); dbl("temp_bath", 1.65); i32("outer_surface", 0)
        i32("global_num_threads", 8); i32("use_temperature", case["use_temperature"])
        ts = abi.SphTangleState()
        L.create_tangle(C.byref(ts), sph.n)
        n = sph.n
        for name, arr in (("vnodes", sph.pos), ("vels", sph.vels), ("vs", sph.vs), ("tangents", sph.tangents),
                          ("normals", sph.normals)):
            abi.vec3_view(getattr(ts, name), n)[:] = arr
        abi.int_view(ts.connections, n, 2)[:] = sph.conn
        abi.int_view(ts.status, n, 2)[:] = sph.stat
        d = ts.domain_section
        d.inner_radius, d.outer_radius, d.azimut_angle, d.polar_angle = sph.domain
        with _quiet_stdout():
            L.update_tangents_normals(C.byref(ts))
            L.update_velocities(C.byref(ts), 0.0)
        for name in ("tangents", "normals", "vels", "vs"):
            out[f"{tag}_{name}"] = np.array(abi.vec3_view(getattr(ts, name), n))
        L.free_tangle(C.byref(ts))
    names = ["superfluid_density", "total_density", "normal_density", "entropy", "mutual_firction_alpha",
             "mutual_firction_alpha_p"]
    Ts = np.linspace(1.31, 2.17, 44)
    vals = []
    with _quiet_stdout():
        for T in Ts:
            row = []
            for nm in names:
                f = getattr(L, nm)
                f.restype, f.argtypes = C.c_double, [C.c_double]
                row.append(f(T))
            vals.append(row)
    out["helium_T"], out["helium"] = Ts, np.array(vals)
    save("spherical.npz", **out)


def main():
    build(ref=True)
    ref = Checker("reference")
    if len(sys.argv) > 1 and sys.argv[1] == "walls":
        walls(ref)
        wall_steps(ref)
        return
    if len(sys.argv) > 1 and sys.argv[1] == "events":
        event_trajectory(ref, W.ring_tangle(), W.config_params("rings8"), 200, 5e-5, "rings8_steps.npz")
        event_trajectory(ref, W.crossing_rings(), W.config_params("rings8"), 200, 5e-5, "crossing_steps.npz")
        return
    if len(sys.argv) > 1 and sys.argv[1] == "spherical":
        spherical()
        return
    if len(sys.argv) > 1 and sys.argv[1] == "injection":
        injection(ref)
        inject_steps(ref)
        return

    # 1. BH velocities (theta 0.4, 0.3 and 0.5) and direct sums on a small random-walk tangle
    ht = W.random_walk_tangle(16, 64, D=0.1, seed=3)
    p = W.config_params("rw")
    p.num_threads = 8
    out = tangle_arrays(ht)
    for theta in (0.3, 0.4, 0.5):
        p.bh_resolution = theta
        ref.set_params(p)
        t = ref.tangle(ht)
        ref.update_tangle(t, 0.0)
        tag = f"{int(theta * 10)}"
        out[f"vels_{tag}"] = t.copy("vels")
        out[f"vs_{tag}"] = t.copy("vs")
        if theta == 0.4:
            out["tangents"] = t.copy("tangents")
            out["normals"] = t.copy("normals")
            nodes = np.arange(0, ht.n, 7, dtype=np.int32)
            dv, dvs = ref.direct_velocities(t, nodes, 0.0)
            out["direct_nodes"], out["direct_vels"], out["direct_vs"] = nodes, dv, dvs
        t.free()
    p.bh_resolution = 0.4
    save("rw16x64.npz", **out)

    # 2. Ring configuration (8 rings, 496 nodes): 200 full steps with the event log;
    #    and crossing ring pairs (16 rings, 992 nodes), whose 200 steps reconnect
    dt = 5e-5
    event_trajectory(ref, W.ring_tangle(), W.config_params("rings8"), 200, dt, "rings8_steps.npz")
    event_trajectory(ref, W.crossing_rings(), W.config_params("rings8"), 200, dt, "crossing_steps.npz")

    # 3. Dense random walk: reconnections and remeshing in the first steps
    ht = W.random_walk_tangle(24, 64, D=0.03, seed=5)
    p = W.config_params("rw")
    p.num_threads = 8
    ref.set_params(p)
    t = ref.tangle(ht)
    recs, conns, stats, poss = [], [], [], []
    for s in range(4):
        recs.append(ref_step(ref, t, s * dt, dt))
        conns.append(t.copy("conn"))
        stats.append(t.copy("status"))
        poss.append(t.copy("pos"))
    save("dense_steps.npz", **tangle_arrays(ht), recs=np.array(recs), conn_steps=np.stack(conns),
         status_steps=np.stack(stats), traj=np.stack(poss), dt=dt)
    t.free()

    # 4. Remesh in both directions (coarse walk -> inserts, fine walk -> removals)
    out = {}
    for tag, delta in (("coarse", 2.2e-3), ("fine", 3e-4)):
        ht = W.random_walk_tangle(8, 48, D=0.1, delta=delta, seed=9)
        ref.set_params(W.config_params("rw"))
        t = ref.tangle(ht)
        ref.remesh(t, 5e-4, 1.5e-3, 0.0)
        for k, v in tangle_arrays(ht).items():
            out[f"{tag}_in_{k}"] = v
        out[f"{tag}_pos"], out[f"{tag}_conn"], out[f"{tag}_status"] = t.copy("pos"), t.copy("conn"), t.copy("status")
        out[f"{tag}_N"] = t.n
        t.free()
    save("remesh.npz", **out)

    # 5. Config-B-sized tangle: velocities of a fixed node subsample from the full BH evaluation
    ht = W.random_walk_tangle(256, 256, D=0.1, seed=1)
    p = W.config_params("rw")
    p.num_threads = 8
    ref.set_params(p)
    t = ref.tangle(ht)
    ref.update_tangle(t, 0.0)
    sub = np.arange(0, ht.n, 97, dtype=np.int32)
    save("rw256x256_sub.npz", nodes=sub, pos_sub=ht.pos[sub], vels=t.copy("vels")[sub], vs=t.copy("vs")[sub],
         pos_checksum=np.array([ht.pos.sum(), (ht.pos ** 2).sum()]))
    t.free()

    # 6. Wall (mirror-image) and open boundary configurations
    walls(ref)
    wall_steps(ref)

    # 7. Injection (add_loop, add_line_in_zdir, inject_vortices in the main loop)
    injection(ref)
    inject_steps(ref)

    # 8. The spherical fork's velocity path
    spherical()


if __name__ == "__main__":
    main()
