"""The drop-in layer (include/ov_dropin.h): OpenVort's own function
signatures, parameters read from the reference's globals, acting in place
on a malloc'd tangle_state - checked against the C oracle (needs a GB300).

The layer is compiled here with tests/dropin_globals.c standing in for the
reference's global definitions.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from openvort_gb300 import abi, gpu, workloads as W
from oracle.pyoracle import Checker
from tests._util import node_rel_err, rel_err, used

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
TS = C.POINTER(abi.TangleState)


@pytest.fixture(scope="module")
def dropin(tmp_path_factory):
    gpu.load()
    out = tmp_path_factory.mktemp("dropin") / "libovdropin_test.so"
    libdir = os.path.join(ROOT, "openvort_gb300", "lib")
    subprocess.run(["gcc", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-o", str(out),
                    os.path.join(ROOT, "openvort_gb300", "csrc", "ov_dropin.c"),
                    os.path.join(ROOT, "tests", "dropin_globals.c"),
                    "-L" + libdir, "-lovgpu", "-Wl,-rpath," + libdir, "-lm"], check=True)
    L = C.CDLL(str(out))
    for name, args, res in [
        ("ovd_update_tangents_normals", [TS], None), ("ovd_update_velocities", [TS, C.c_double], None),
        ("ovd_update_velocity", [TS, C.c_int, C.c_double, C.c_void_p], None),
        ("ovd_rk4_step", [TS, C.c_double, C.c_double], None), ("ovd_reconnect", [TS, C.c_double], C.c_int),
        ("ovd_remesh", [TS, C.c_double, C.c_double, C.c_double], None),
        ("ovd_eliminate_small_loops", [TS], None), ("ovd_enforce_periodic_boundaries", [TS], None),
        ("ovd_smooth", [TS], None), ("ovd_octree_build", [TS], C.c_void_p),
        ("ovd_octree_get_vs", [TS, C.c_void_p, C.POINTER(abi.Vec3), C.c_double, C.POINTER(abi.Vec3)], None),
        ("ovd_octree_destroy", [C.c_void_p], None), ("ovd_last_status", [], C.c_int),
        ("ovd_enforce_wall_boundaries", [TS, C.c_double], None),
        ("ovd_save_tangle", [C.c_char_p, TS], None), ("ovd_load_tangle", [C.c_char_p, TS], C.c_int),
        ("ovd_add_loop", [TS, C.POINTER(abi.Vec3), C.POINTER(abi.Vec3), C.c_double], None),
        ("ovd_add_line_in_zdir", [TS, C.c_double, C.c_double, C.c_int], None),
        ("ovd_inject_vortices", [TS, C.c_double], None)]:
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = res
    return L


def set_globals(L, p):
    dbl = lambda n, v: setattr(C.c_double.in_dll(L, n), "value", float(v))  # noqa: E731
    i32 = lambda n, v: setattr(C.c_int.in_dll(L, n), "value", int(v))  # noqa: E731
    dbl("KAPPA", p.kappa); dbl("VORTEX_WIDTH", p.vortex_width); dbl("alpha", p.alpha); dbl("alpha_p", p.alpha_p)
    i32("use_mutual_friction", p.use_mutual_friction); i32("use_BH", p.use_bh); dbl("BH_resolution", p.bh_resolution)
    dbl("global_dl_min", p.dl_min); dbl("global_dl_max", p.dl_max); dbl("rec_dist", p.rec_dist)
    dbl("reconnection_angle_cutoff", p.reconnection_angle_cutoff); i32("small_loop_cutoff", p.small_loop_cutoff)
    i32("use_freq_filter", p.use_freq_filter); dbl("freq_to_cutoff", p.freq_to_cutoff)
    i32("pin_mode", p.pin_mode)
    for name, src in (("vn_conf", p.vn), ("vs_conf", p.vs), ("vb_conf", p.vb)):
        dst = abi.ExtVel.in_dll(L, name)
        C.memmove(C.addressof(dst), C.addressof(src), C.sizeof(abi.ExtVel))


def test_velocities_and_rk4_in_place(dropin):
    port = Checker("port")
    ht = W.random_walk_tangle(16, 64, D=0.1, seed=71)
    p = W.config_params("rw")
    set_globals(dropin, p)
    port.set_params(p)
    a, b = port.tangle(ht), port.tangle(ht)     # a: drop-in, b: oracle (same malloc'd layout)
    dropin.ovd_update_tangents_normals(C.byref(a.ts))
    dropin.ovd_update_velocities(C.byref(a.ts), 0.0)
    assert dropin.ovd_last_status() == 0
    port.update_tangle(b, 0.0)
    assert node_rel_err(a.copy("vels"), b.copy("vels")) < 1e-10
    dropin.ovd_rk4_step(C.byref(a.ts), 0.0, 5e-5)
    port.rk4_step(b, 0.0, 5e-5)
    assert rel_err(a.copy("pos") - ht.pos, b.copy("pos") - ht.pos) < 1e-9
    # update_velocity, direct branch, for one node
    dropin.ovd_update_velocity(C.byref(a.ts), 5, 0.0, None)
    vd, _ = port.direct_velocities(b, [5], 0.0)
    assert node_rel_err(a.copy("vels")[5:6], vd) < 1e-10


def test_topology_passes_in_place(dropin, golden):
    from tests._util import host_from_arrays
    g = golden("remesh.npz")
    ht = host_from_arrays(g, prefix="coarse_in_")
    p = W.config_params("rw")
    set_globals(dropin, p)
    port = Checker("port")
    t = port.tangle(ht)                 # malloc'd arrays: the drop-in may realloc them
    dropin.ovd_remesh(C.byref(t.ts), 5e-4, 1.5e-3, 0.0)
    assert dropin.ovd_last_status() == 0
    assert t.n == int(g["coarse_N"])
    np.testing.assert_array_equal(t.copy("conn"), g["coarse_conn"])
    ht2 = W.random_walk_tangle(40, 48, D=0.03, seed=61)
    a, b = port.tangle(ht2), port.tangle(ht2)
    n_gpu = dropin.ovd_reconnect(C.byref(a.ts), 0.0)
    port.set_params(p)
    n_ref = port.reconnect(b, 0.0)
    assert n_gpu == n_ref > 0
    np.testing.assert_array_equal(a.copy("conn"), b.copy("conn"))
    dropin.ovd_eliminate_small_loops(C.byref(a.ts))
    port.eliminate_small_loops(b)
    np.testing.assert_array_equal(a.copy("status"), b.copy("status"))


def test_octree_api(dropin):
    ht = W.random_walk_tangle(8, 48, D=0.1, seed=72)
    p = W.config_params("rw")
    set_globals(dropin, p)
    port = Checker("port")
    t = port.tangle(ht)
    tree = dropin.ovd_octree_build(C.byref(t.ts))
    assert tree
    port.lib.orc_octree_build.argtypes = [TS]
    port.lib.orc_octree_build.restype = C.c_void_p
    port.lib.orc_octree_get_vs.argtypes = [TS, C.c_void_p, C.POINTER(abi.Vec3), C.c_double,
                                          C.POINTER(abi.Params), C.POINTER(abi.Vec3)]
    port.lib.orc_octree_destroy.argtypes = [C.c_void_p]
    otree = port.lib.orc_octree_build(C.byref(t.ts))
    for r in ([0.05, 0.05, 0.05], [0.0, 0.1, 0.02], [0.13, -0.04, 0.07]):
        q = abi.Vec3()
        q.p[:] = r
        got, ref = abi.Vec3(), abi.Vec3()
        dropin.ovd_octree_get_vs(C.byref(t.ts), tree, C.byref(q), 0.4, C.byref(got))
        port.lib.orc_octree_get_vs(C.byref(t.ts), otree, C.byref(q), 0.4, C.byref(p), C.byref(ref))
        np.testing.assert_allclose(list(got.p), list(ref.p), rtol=1e-10, atol=1e-14)
    dropin.ovd_octree_destroy(tree)
    port.lib.orc_octree_destroy(otree)


def vec3(v):
    out = abi.Vec3()
    out.p[:] = list(map(float, v))
    return out


def test_injection_walls_and_frames_in_place(dropin, golden, tmp_path):
    """add_loop / add_line_in_zdir, then inject_vortices + enforce_wall_boundaries
    + the rest of the main loop through the drop-in, against the reference's
    run; save_tangle / load_tangle round trip of the result."""
    from tests.test_gpu_inject import CALLS, wall_tangle
    port = Checker("port")
    g = golden("inject.npz")
    p = W.config_params("rings8", rec_dist=8e-4)
    t = port.tangle(wall_tangle(g))
    for k, call in enumerate(CALLS):
        p.pin_mode = abi.OV_PINNED if k < 3 else abi.OV_PINNED_SLIP
        set_globals(dropin, p)
        if call[0] == "loop":
            dropin.ovd_add_loop(C.byref(t.ts), C.byref(vec3(call[1])), C.byref(vec3(call[2])), call[3])
        else:
            dropin.ovd_add_line_in_zdir(C.byref(t.ts), call[1], call[2], call[3])
        assert dropin.ovd_last_status() == 0
        assert t.n == int(g[f"c{k}_N"])
        assert (t.ts.next_empty, t.ts.total_empty) == (int(g[f"c{k}_next_empty"]), int(g[f"c{k}_total_empty"]))
        np.testing.assert_array_equal(t.copy("conn"), g[f"c{k}_conn"])
        np.testing.assert_array_equal(t.copy("status"), g[f"c{k}_status"])

    g = golden("inject_steps.npz")
    p = W.config_params("rings8", rec_dist=8e-4)
    set_globals(dropin, p)
    i32 = lambda n, v: setattr(C.c_int.in_dll(dropin, n), "value", int(v))  # noqa: E731
    dbl = lambda n, v: setattr(C.c_double.in_dll(dropin, n), "value", float(v))  # noqa: E731
    i32("loop_injection", g["inj_loop_injection"]); dbl("loop_injection_frequency", g["inj_loop_frequency"])
    i32("line_injection", g["inj_line_injection"]); i32("line_injection_n", g["inj_line_n"])
    dbl("line_injection_frequency", g["inj_line_frequency"]); i32("line_injection_polarized", g["inj_line_polarized"])
    libc = C.CDLL("libc.so.6")
    libc.srand48.argtypes = [C.c_long]
    libc.drand48.restype = C.c_double
    libc.srand48(int(g["inj_seed"]))
    t = port.tangle(wall_tangle(g))
    ts = C.byref(t.ts)
    dt = float(g["dt"])
    for s_ in range(3):
        dropin.ovd_inject_vortices(ts, s_ * dt)
        dropin.ovd_enforce_wall_boundaries(ts, 0.0)
        dropin.ovd_eliminate_small_loops(ts)
        assert dropin.ovd_reconnect(ts, 0.0) == int(g["recs"][s_])
        dropin.ovd_eliminate_small_loops(ts)
        dropin.ovd_enforce_periodic_boundaries(ts)
        dropin.ovd_remesh(ts, p.dl_min, p.dl_max, 0.0)
        dropin.ovd_eliminate_small_loops(ts)
        dropin.ovd_update_tangents_normals(ts)
        dropin.ovd_update_velocities(ts, s_ * dt)
        dropin.ovd_rk4_step(ts, s_ * dt, dt)
        dropin.ovd_enforce_periodic_boundaries(ts)
        assert dropin.ovd_last_status() == 0
        n = t.n
        assert n == int(g["steps_N"][s_])
        np.testing.assert_array_equal(t.copy("conn"), g["steps_conn"][s_][:n])
        np.testing.assert_array_equal(t.copy("status"), g["steps_status"][s_][:n])
        live = g["steps_status"][s_][:n, 0] != abi.OV_EMPTY
        ref = g["steps_pos"][s_][:n][live]
        assert np.abs(t.copy("pos")[live] - ref).max() / np.abs(ref).max() < 1e-10
    assert libc.drand48() == float(g["next_draw"])
    i32("loop_injection", 0); i32("line_injection", 0)

    path = str(tmp_path / "frame.txt").encode()
    dropin.ovd_save_tangle(path, ts)
    back = port.tangle(W.HostTangle(np.zeros((1, 3)), np.full(1, -1), np.full(1, -1), np.zeros(3), np.full(3, 0.1),
                                    status=np.full(1, abi.OV_EMPTY)))
    back.ts.next_empty, back.ts.total_empty = 0, 1
    assert dropin.ovd_load_tangle(path, C.byref(back.ts)) == 0
    assert back.n >= t.n
    live = t.copy("status")[:, 0] != abi.OV_EMPTY
    np.testing.assert_array_equal(back.copy("conn")[:t.n][live], t.copy("conn")[live])
    np.testing.assert_array_equal(back.copy("status")[:t.n][live], t.copy("status")[live])
    assert np.abs(back.copy("pos")[:t.n][live] - t.copy("pos")[live]).max() < 1e-15
