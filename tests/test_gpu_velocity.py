"""GPU parity of the velocity path through the C ABI (needs a GB300).

Gates: FP64 velocities within 1e-10 relative per node of the reference's
CPU Barnes-Hut (golden vectors from OpenVort itself, and the C oracle at
sizes the golden files do not hold); tangents/normals within 1e-12.
"""
from __future__ import annotations

import numpy as np
import pytest

from openvort_gb300 import abi, gpu, workloads as W
from oracle.pyoracle import Checker
from tests._util import host_from_arrays, node_rel_err, rel_err

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10


@pytest.fixture(scope="module")
def port():
    return Checker("port")


WALKS = [abi.OV_WALK_SPLIT, abi.OV_WALK_FP64]


def _gpu_eval(ht, p, t=0.0, walk=abi.OV_WALK_SPLIT):
    ctx = gpu.Context(0, params=p)
    ctx.set_walk(walk)
    ctx.upload(ht)
    ctx.update_tangle(t)
    ctx.download(ht)
    st = ctx.stats()
    ctx.close()
    return st


@pytest.mark.parametrize("walk", WALKS)
@pytest.mark.parametrize("theta", [0.3, 0.4, 0.5])
def test_bh_matches_reference_golden(golden, theta, walk):
    g = golden("rw16x64.npz")
    ht = host_from_arrays(g)
    p = W.config_params("rw", bh_resolution=theta)
    st = _gpu_eval(ht, p, walk=walk)
    tag = f"{int(theta * 10)}"
    assert st["error_word"] == 0
    assert node_rel_err(ht.vels, g[f"vels_{tag}"]) < FP64_TOL
    assert node_rel_err(ht.vs, g[f"vs_{tag}"]) < FP64_TOL
    if theta == 0.4:
        assert rel_err(ht.tangents, g["tangents"]) < 1e-12
        assert rel_err(ht.normals, g["normals"]) < 1e-12


@pytest.mark.parametrize("walk", WALKS)
def test_interaction_counts_match_oracle_tree(port, golden, walk):
    """Same tree, same decisions: per-target visits/accepts equal the pointer octree's."""
    import ctypes as C

    g = golden("rw16x64.npz")
    ht = host_from_arrays(g)
    p = W.config_params("rw")
    st = _gpu_eval(ht, p, walk=walk)
    t = port.tangle(ht)
    from oracle.pyoracle import Checker as _C  # noqa: F401

    class Counts(C.Structure):
        _fields_ = [("visits", C.c_longlong), ("accepts", C.c_longlong), ("max_depth", C.c_int),
                    ("cells", C.c_longlong)]

    cnt = Counts()
    port.lib.orc_count_interactions.argtypes = [C.POINTER(abi.TangleState), C.c_double, C.POINTER(Counts)]
    port.lib.orc_count_interactions(C.byref(t.ts), 0.4, C.byref(cnt))
    assert st["cells"] == cnt.cells
    assert st["max_depth"] == cnt.max_depth
    assert st["accepts"] == cnt.accepts
    assert st["visits"] == cnt.visits


def test_direct_sum_matches_reference_golden(golden):
    g = golden("rw16x64.npz")
    ht = host_from_arrays(g)
    ctx = gpu.Context(0, params=W.config_params("rw"))
    ctx.upload(ht)
    ctx.update_tangents_normals()
    vels, vs = ctx.direct_velocities(g["direct_nodes"], 0.0)
    ctx.close()
    assert node_rel_err(vels, g["direct_vels"]) < FP64_TOL
    assert node_rel_err(vs, g["direct_vs"]) < FP64_TOL


def test_config_b_full_size_vs_oracle(port, golden):
    """65,536 nodes (256 loops x 256), theta 0.4: every node against the oracle."""
    ht = W.random_walk_tangle(256, 256, D=0.1, seed=1)
    p = W.config_params("rw")
    p.num_threads = 16
    st = _gpu_eval(ht, p)
    assert st["error_word"] == 0
    port.set_params(p)
    t = port.tangle(ht)
    port.update_tangle(t, 0.0)
    assert node_rel_err(ht.vels, t.copy("vels")) < FP64_TOL
    g = golden("rw256x256_sub.npz")
    assert node_rel_err(ht.vels[g["nodes"]], g["vels"]) < FP64_TOL


@pytest.mark.parametrize("images", [None, "wall_2_4"])
def test_split_walk_equals_fp64_walk(images):
    """OV_PREC_FP64's two walks: the same decisions (visits, accepts) and FP64
    velocities a few ulps apart (the law's square roots and divisions)."""
    base = W.random_walk_tangle(256, 256, D=0.1, seed=1)
    ht = base if images is None else W.HostTangle(base.pos.copy(), base.conn[:, 0].copy(), base.conn[:, 1].copy(),
                                                   base.box_lo, base.box_hi, image_set=images)
    p = W.config_params("rw")
    out = []
    for walk in WALKS:
        st = _gpu_eval(ht, p, walk=walk)
        assert st["error_word"] == 0
        out.append((np.array(ht.vels), st))
    (v_split, st_split), (v_64, st_64) = out
    assert st_split["visits"] == st_64["visits"] and st_split["accepts"] == st_64["accepts"]
    assert node_rel_err(v_split, v_64) < 1e-12


def test_theta_zero_equals_direct_sum():
    """theta = 0 accepts only leaves, so the tree sum is the direct sum."""
    ht = W.random_walk_tangle(6, 40, D=0.1, seed=31)
    p = W.config_params("rw", bh_resolution=0.0)
    ctx = gpu.Context(0, params=p)
    ctx.upload(ht)
    ctx.update_tangle(0.0)
    ctx.download(ht)
    nodes = np.arange(ht.n, dtype=np.int32)
    dv, _ = ctx.direct_velocities(nodes, 0.0)
    ctx.close()
    assert node_rel_err(ht.vels, dv) < 1e-12


@pytest.mark.parametrize("walk", WALKS)
@pytest.mark.parametrize("case", ["out_of_box", "empty_slots", "single_loop", "mixed_loop_sizes"])
def test_edge_cases_vs_oracle(port, case, walk):
    rng = np.random.default_rng(5)
    if case == "out_of_box":
        ht = W.random_walk_tangle(10, 48, D=0.1, seed=24)
        ht.pos[::5] += 0.004          # RK4 stage positions leave the box
    elif case == "empty_slots":
        base = W.random_walk_tangle(10, 48, D=0.1, seed=25)
        m = base.n + base.n // 2
        where = rng.choice(m, base.n, replace=False)      # node i lives in slot where[i]
        pos = np.zeros((m, 3))
        fwd = np.full(m, -1)
        rev = np.full(m, -1)
        status = np.full(m, abi.OV_EMPTY)
        pos[where] = base.pos
        fwd[where] = where[base.fwd]
        rev[where] = where[base.rev]
        status[where] = abi.OV_FREE
        ht = W.HostTangle(pos, fwd, rev, base.box_lo, base.box_hi, status=status)
    elif case == "single_loop":
        ht = W.random_walk_tangle(1, 64, D=0.1, seed=26)
    else:
        a = W.random_walk_tangle(3, 100, D=0.1, seed=27)
        b = W.random_walk_tangle(5, 7, D=0.1, seed=28)
        n = a.n
        ht = W.HostTangle(np.concatenate([a.pos, b.pos]), np.concatenate([a.fwd, b.fwd + n]),
                          np.concatenate([a.rev, b.rev + n]), a.box_lo, a.box_hi)
    p = W.config_params("rw")
    st = _gpu_eval(ht, p, walk=walk)
    assert st["error_word"] == 0
    port.set_params(p)
    t = port.tangle(ht)
    port.update_tangle(t, 0.0)
    used = ht.stat[:, 0] != abi.OV_EMPTY
    assert node_rel_err(ht.vels[used], t.copy("vels")[used]) < FP64_TOL
    if case == "out_of_box":
        assert st["out_of_root"] == int(((ht.pos < 0) | (ht.pos > 0.1)).any(axis=1).sum())


def test_rk4_step_vs_oracle(port):
    ht = W.random_walk_tangle(12, 64, D=0.1, seed=33)
    p = W.config_params("rw")
    dt = 5e-5
    ctx = gpu.Context(0, params=p)
    ctx.upload(ht)
    port.set_params(p)
    t = port.tangle(ht)
    for s in range(3):
        ctx.update_tangle(s * dt)
        ctx.rk4_step(s * dt, dt)
        port.update_tangle(t, s * dt)
        port.rk4_step(t, s * dt, dt)
    ctx.download(ht)
    ctx.close()
    ref = t.copy("pos")
    disp = np.abs(ref - W.random_walk_tangle(12, 64, D=0.1, seed=33).pos).max()
    assert np.abs(ht.pos - ref).max() < 1e-10 * disp


def test_all_empty_and_tiny_tangles():
    for n_loops, per in ((1, 5), (1, 6)):
        ht = W.random_walk_tangle(n_loops, per, D=0.1, seed=40)
        st = _gpu_eval(ht, W.config_params("rw"))
        assert st["error_word"] == 0 and np.all(np.isfinite(ht.vels))
    ht = W.random_walk_tangle(1, 8, D=0.1, seed=41)
    ht.stat[:, 0] = abi.OV_EMPTY
    st = _gpu_eval(ht, W.config_params("rw"))
    assert st["node_evals"] == 0 and st["cells"] == 0


@pytest.mark.parametrize("prec", [abi.OV_PREC_FP64, abi.OV_PREC_MIXED])
def test_rk4_graph_equals_stream_launches(prec):
    """The captured RK4 graph gives bit-identical positions to launching the
    same kernels one by one, over several steps (graph reused, times updated)."""
    outs = []
    for graph in (True, False):
        ht = W.random_walk_tangle(12, 64, D=0.1, seed=34)
        ctx = gpu.Context(0, params=W.config_params("rw"), precision=prec)
        ctx.set_rk4_graph(graph)
        ctx.upload(ht)
        for s in range(3):
            ctx.update_tangle(s * 5e-5)
            ctx.rk4_step(s * 5e-5, 5e-5)
        ctx.download(ht, abi.OV_F_POS)
        ctx.close()
        outs.append(np.array(ht.pos))
    np.testing.assert_array_equal(outs[0], outs[1])


@pytest.mark.parametrize("time", [0.0, 3e-5, 1e-4, 2.5e-4])
def test_decreasing_flow_vs_oracle(port, time):
    """v_n and v_s DECREASING (external_velocity.c:39-56; ramps over 1e-4 s):
    update_tangle and an RK4 step whose stage times straddle the ramp's end,
    against the oracle (itself bit-identical to OpenVort on these cases)."""
    from tests.test_oracle_pin import _decreasing_params
    ht = W.random_walk_tangle(8, 48, D=0.1, seed=19)
    p = _decreasing_params()
    p.num_threads = 4
    ctx = gpu.Context(0, params=p)
    ctx.upload(ht)
    ctx.update_tangle(time)
    v1 = np.array(ctx.download(ht, abi.OV_F_VELS | abi.OV_F_VS).vels)
    s1 = np.array(ht.vs)
    ctx.rk4_step(time, 5e-5)
    pos = np.array(ctx.download(ht, abi.OV_F_POS).pos)
    ctx.close()
    port.set_params(p)
    t = port.tangle(W.random_walk_tangle(8, 48, D=0.1, seed=19))
    port.update_tangle(t, time)
    assert node_rel_err(v1, t.copy("vels")) < FP64_TOL
    assert node_rel_err(s1, t.copy("vs")) < FP64_TOL
    port.rk4_step(t, time, 5e-5)
    assert rel_err(pos, t.copy("pos")) < FP64_TOL
    t.free()
