"""Pin the CPU oracle (C restatement) against OpenVort itself.

Two sources of truth:
  * golden vectors in tests/golden/, produced by OpenVort compiled from its
    own sources (tests/golden/make_golden.py) - checked everywhere;
  * the live reference build (oracle/_ref) - checked bit-for-bit where it
    exists (not on machines without the OpenVort checkout).
"""
from __future__ import annotations

import numpy as np
import pytest

from oracle.pyoracle import Checker, reference_available
from openvort_gb300 import workloads as W
from tests._util import check_event_trajectory, host_from_arrays, node_rel_err, rel_err, used

# Same build flags on the same machine give identical bits; across machines
# libm's log() may differ in the last place, so cross-machine checks allow a
# few ulps.
CROSS_MACHINE_TOL = 1e-12


@pytest.fixture(scope="module")
def port():
    return Checker("port")


def _ref_step(c, t, time, dt, log=False):
    c.eliminate_small_loops(t)
    n = c.reconnect(t, 0.0, log=log)
    c.eliminate_small_loops(t)
    c.enforce_periodic(t)
    c.remesh(t, c.params.dl_min, c.params.dl_max, 0.0)
    c.eliminate_small_loops(t)
    c.update_tangle(t, time)
    c.rk4_step(t, time, dt)
    c.enforce_periodic(t)
    return n


@pytest.mark.parametrize("theta", [0.3, 0.4, 0.5])
def test_bh_velocities_match_golden(port, golden, theta):
    g = golden("rw16x64.npz")
    ht = host_from_arrays(g)
    p = W.config_params("rw", bh_resolution=theta)
    p.num_threads = 4
    port.set_params(p)
    t = port.tangle(ht)
    port.update_tangle(t, 0.0)
    tag = f"{int(theta * 10)}"
    assert node_rel_err(t.copy("vels"), g[f"vels_{tag}"]) < CROSS_MACHINE_TOL
    assert node_rel_err(t.copy("vs"), g[f"vs_{tag}"]) < CROSS_MACHINE_TOL
    if theta == 0.4:
        assert rel_err(t.copy("tangents"), g["tangents"]) < CROSS_MACHINE_TOL
        assert rel_err(t.copy("normals"), g["normals"]) < CROSS_MACHINE_TOL


def test_direct_sum_matches_golden(port, golden):
    g = golden("rw16x64.npz")
    ht = host_from_arrays(g)
    p = W.config_params("rw")
    p.num_threads = 4
    port.set_params(p)
    t = port.tangle(ht)
    port.update_tangents_normals(t)
    vels, vs = port.direct_velocities(t, g["direct_nodes"], 0.0)
    assert node_rel_err(vels, g["direct_vels"]) < CROSS_MACHINE_TOL
    assert node_rel_err(vs, g["direct_vs"]) < CROSS_MACHINE_TOL


@pytest.mark.parametrize("name", ["rings8_steps.npz", "crossing_steps.npz"])
def test_200_steps_event_log_matches_golden(port, golden, name):
    """The 8-ring configuration (no reconnection in 200 steps) and the
    crossing ring pairs (12 reconnections in 200 steps): per-step
    reconnection counts and (k, l) pairs, topology after every event step,
    positions at the stored steps."""
    g = golden(name)
    ht = host_from_arrays(g)
    p = W.config_params("rings8")
    p.num_threads = 4
    port.set_params(p)
    t = port.tangle(ht)
    dt = float(g["dt"])

    def step(s):
        return _ref_step(port, t, s * dt, dt, log=True)

    def snapshot():
        return t.copy("conn"), t.copy("status"), t.copy("pos")

    recs = check_event_trajectory(g, step, snapshot, CROSS_MACHINE_TOL, pass_log=True)
    assert sum(recs) == (0 if name.startswith("rings8") else 12)
    t.free()


@pytest.mark.parametrize("name,cfg", [("dense_steps.npz", "rw")])
def test_steps_match_golden(port, golden, name, cfg):
    g = golden(name)
    ht = host_from_arrays(g)
    p = W.config_params(cfg)
    p.num_threads = 4
    port.set_params(p)
    t = port.tangle(ht)
    dt = float(g["dt"])
    nsteps = len(g["recs"])
    recs, traj = [], []
    for s in range(nsteps):
        recs.append(port.step(t, s * dt, dt))
        traj.append(t.copy("pos"))
        if name.startswith("dense"):
            np.testing.assert_array_equal(t.copy("conn"), g["conn_steps"][s])
            np.testing.assert_array_equal(t.copy("status"), g["status_steps"][s])
    assert recs == list(g["recs"])
    steps = g["traj_steps"] if "traj_steps" in g else np.arange(nsteps)
    for i, s in enumerate(steps):
        m = used(g["status_final"] if "status_final" in g else g["status_steps"][s])
        assert rel_err(traj[s][m], g["traj"][i][m]) < CROSS_MACHINE_TOL
    if "conn_final" in g:
        np.testing.assert_array_equal(t.copy("conn"), g["conn_final"])


@pytest.mark.parametrize("tag", ["coarse", "fine"])
def test_remesh_matches_golden(port, golden, tag):
    g = golden("remesh.npz")
    ht = host_from_arrays(g, prefix=f"{tag}_in_")
    port.set_params(W.config_params("rw"))
    t = port.tangle(ht)
    added, removed = port.remesh(t, 5e-4, 1.5e-3, 0.0)
    assert added + removed > 0
    assert t.n == int(g[f"{tag}_N"])
    np.testing.assert_array_equal(t.copy("conn"), g[f"{tag}_conn"])
    np.testing.assert_array_equal(t.copy("status"), g[f"{tag}_status"])
    m = used(g[f"{tag}_status"])
    assert rel_err(t.copy("pos")[m], g[f"{tag}_pos"][m]) < CROSS_MACHINE_TOL


def test_config_b_subsample_matches_golden(port, golden):
    g = golden("rw256x256_sub.npz")
    ht = W.random_walk_tangle(256, 256, D=0.1, seed=1)
    np.testing.assert_allclose(ht.pos[g["nodes"]], g["pos_sub"], rtol=0, atol=1e-15)
    p = W.config_params("rw")
    p.num_threads = 8
    port.set_params(p)
    t = port.tangle(ht)
    port.update_tangle(t, 0.0)
    assert node_rel_err(t.copy("vels")[g["nodes"]], g["vels"]) < 1e-10


@pytest.mark.skipif(not reference_available(), reason="OpenVort checkout not built here")
@pytest.mark.parametrize("case", ["rw_theta3", "dense_steps", "remesh_coarse", "out_of_box"])
def test_bit_identical_to_live_reference(case):
    ref, port = Checker("reference"), Checker("port")
    p = W.config_params("rw")
    p.num_threads = 4
    if case == "rw_theta3":
        ht = W.random_walk_tangle(12, 48, D=0.1, seed=21)
        p.bh_resolution = 0.3
    elif case == "dense_steps":
        ht = W.random_walk_tangle(16, 48, D=0.025, seed=22)
    elif case == "remesh_coarse":
        ht = W.random_walk_tangle(6, 40, D=0.1, delta=3e-3, seed=23)
    else:
        # nodes pushed outside the root box (RK4 stage positions are unwrapped)
        ht = W.random_walk_tangle(8, 40, D=0.1, seed=24)
        ht.pos[::5] += 0.004
    outs = []
    for c in (ref, port):
        c.set_params(p)
        t = c.tangle(ht)
        if case == "dense_steps":
            for s in range(3):
                _ref_step(c, t, s * 5e-5, 5e-5) if c is ref else c.step(t, s * 5e-5, 5e-5)
        elif case == "remesh_coarse":
            c.remesh(t, p.dl_min, p.dl_max, 0.0)
            c.update_tangle(t, 0.0)
        else:
            c.update_tangle(t, 0.0)
            c.rk4_step(t, 0.0, 5e-5)
        outs.append({k: t.copy(k) for k in ("pos", "vels", "conn", "status")})
    for k in ("conn", "status"):
        np.testing.assert_array_equal(outs[0][k], outs[1][k], err_msg=k)
    m = used(outs[0]["status"])   # EMPTY slots hold whatever realloc left there
    for k in ("pos", "vels"):
        np.testing.assert_array_equal(outs[0][k][m], outs[1][k][m], err_msg=k)


def test_ring_velocity_known_answer(port):
    """Thesis p.15 eq. 2.1: v = kappa/(4 pi R) (ln(8R/a0) - 1/2), within 5%."""
    R, D = 0.02, 1.0
    ht = W.ring_tangle(n_rings=1, radius=R, D=D, dl_min=5e-4, dl_max=1.5e-3, seed=3, n_images=0)
    ht.walls = (0, 0, 0, 0, 0, 0)
    p = W.config_params("rw", use_mutual_friction=0, vortex_width=1.3e-8)
    port.set_params(p)
    t = port.tangle(ht)
    port.update_tangle(t, 0.0)
    v = np.linalg.norm(t.copy("vels"), axis=1).mean()
    v_exact = 9.97e-4 / (4 * np.pi * R) * (np.log(8 * R / 1.3e-8) - 0.5)
    assert abs(v / v_exact - 1) < 0.05


@pytest.mark.skipif(not reference_available(), reason="OpenVort checkout not built here")
@pytest.mark.parametrize("name", ["periodic_6", "periodic_18", "periodic_26", "wall_1_open", "wall_1_18",
                                  "wall_1_26", "wall_2_4", "wall_2_2", "wall_parallel_planes", "wall_canal"])
def test_boundary_tables_match_reference(name):
    """The named boundary configurations equal the reference's own tables
    (read from the compiled reference), entry by entry."""
    import ctypes as C
    import os
    from openvort_gb300 import abi
    lib = C.CDLL(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle", "_ref",
                              "libovref.so"))
    bimg = abi.BoundaryImages.in_dll(lib, name)
    ours, _ = abi.image_set(name)
    assert bimg.n == len(ours)
    for j, (sh, refl) in enumerate(ours):
        e = bimg.images[j]
        assert tuple(e.shift) == tuple(sh), j
        assert e.number_of_reflects == len(refl), j
        assert tuple(e.reflect[:len(refl)]) == tuple(refl), j


@pytest.mark.parametrize("name", ["wall_1_open", "wall_1_18", "wall_1_26", "wall_2_4", "wall_2_2",
                                  "wall_parallel_planes", "wall_canal", "open", "periodic_6"])
def test_wall_configurations_match_golden(port, golden, name):
    """Mirror-image and open boundaries: the restatement's BH and direct-sum
    velocities equal the reference's (golden vectors from the reference)."""
    g = golden("walls.npz")
    ht = W.HostTangle(g["pos"].copy(), g["conn"][:, 0].copy(), g["conn"][:, 1].copy(), g["box_lo"], g["box_hi"],
                      image_set=name)
    port.set_params(W.config_params("rw"))
    t = port.tangle(ht)
    port.update_tangle(t, 0.0)
    assert node_rel_err(t.copy("vels"), g[f"{name}_vels"]) < 1e-12
    dv, _ = port.direct_velocities(t, g["direct_nodes"], 0.0)
    assert node_rel_err(dv, g[f"{name}_direct_vels"]) < 1e-12
    t.free()


def _decreasing_params():
    """v_n and v_s both DECREASING (external_velocity.c:39-56): linear ramps
    from a starting strength to the final one over 1e-4 s."""
    from openvort_gb300 import abi
    p = W.config_params("rw")
    for flow, (s0, s1, d) in ((p.vn, (1.0, 0.2, (1.0, 0.5, 0.0))), (p.vs, (-0.3, 0.1, (0.0, 1.0, 2.0)))):
        flow.type = abi.OV_DECREASING
        flow.starting_strength = s0
        flow.strength = s1
        flow.time_of_linear_decrease = 1e-4
        flow.direction.p[:] = d
    return p


@pytest.mark.skipif(not reference_available(), reason="OpenVort checkout not built here")
@pytest.mark.parametrize("time", [0.0, 3e-5, 1e-4, 2.5e-4])
def test_decreasing_flow_bit_identical_to_live_reference(time):
    ht = W.random_walk_tangle(8, 48, D=0.1, seed=19)
    p = _decreasing_params()
    p.num_threads = 4
    out = {}
    for kind in ("port", "reference"):
        c = Checker(kind)
        c.set_params(p)
        t = c.tangle(ht)
        c.update_tangle(t, time)
        c.rk4_step(t, time, 5e-5)
        out[kind] = (t.copy("vels"), t.copy("vs"), t.copy("pos"))
        t.free()
    for a, b in zip(out["port"], out["reference"]):
        np.testing.assert_array_equal(a, b)
