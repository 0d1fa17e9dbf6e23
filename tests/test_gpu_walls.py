"""Wall (mirror-image) and open boundary configurations on the GPU.

The reference's named boundary sets (src/boundary_images.c): images that
are translations, mirror reflections through a wall, or both.  Golden
vectors come from the reference itself (tests/golden/make_golden.py):
Barnes-Hut velocities at theta 0.4 and direct sums.  In the direct-sum
branch the reference adds mirror images without reflecting their velocity
(tangle.c:665-684 accumulates into vs[k] and reflects a zero vector); the
GPU direct sums reproduce that, the Barnes-Hut branch reflects as
tangle.c:640-645 does.
"""
from __future__ import annotations

import numpy as np
import pytest

from openvort_gb300 import abi, gpu, workloads as W
from tests._util import node_rel_err, rel_l2

pytestmark = pytest.mark.gpu

SETS = ["wall_1_open", "wall_1_18", "wall_1_26", "wall_2_4", "wall_2_2", "wall_parallel_planes", "wall_canal",
        "open", "periodic_6"]


def host(g, name):
    return W.HostTangle(g["pos"].copy(), g["conn"][:, 0].copy(), g["conn"][:, 1].copy(), g["box_lo"], g["box_hi"],
                        image_set=name)


@pytest.mark.parametrize("name", SETS)
def test_fp64_velocities_match_reference(golden, name):
    g = golden("walls.npz")
    ht = host(g, name)
    ctx = gpu.Context(0, params=W.config_params("rw"))
    ctx.upload(ht)
    ctx.update_tangle(0.0)
    out = ctx.download(ht)
    assert node_rel_err(out.vels, g[f"{name}_vels"]) < 1e-10
    assert node_rel_err(out.vs, g[f"{name}_vs"]) < 1e-10
    dv, dvs = ctx.direct_velocities(g["direct_nodes"], 0.0)
    ctx.close()
    assert node_rel_err(dv, g[f"{name}_direct_vels"]) < 1e-10
    assert node_rel_err(dvs, g[f"{name}_direct_vs"]) < 1e-10


@pytest.mark.parametrize("name", ["wall_2_4", "wall_canal", "wall_1_26"])
def test_mixed_matches_fp64_tree(golden, name):
    g = golden("walls.npz")
    ht = host(g, name)
    ctx = gpu.Context(0, params=W.config_params("rw"), precision=abi.OV_PREC_FP64)
    ctx.upload(ht)
    ctx.update_tangle(0.0)
    v64 = ctx.download(ht).vels.copy()
    s64 = ctx.stats()
    ctx.set_precision(abi.OV_PREC_MIXED)
    ctx.update_tangle(0.0)
    v32 = ctx.download(ht).vels.copy()
    s32 = ctx.stats()
    ctx.close()
    assert rel_l2(v32, v64) < 1e-6
    assert s32["accepts"] == s64["accepts"] and s32["visits"] == s64["visits"]


def test_bounded_sums_with_mirror_images(golden):
    g = golden("walls.npz")
    ht = host(g, "wall_canal")
    ctx = gpu.Context(0, params=W.config_params("rw"))
    ctx.upload(ht)
    nodes = np.arange(0, ht.n, 5)
    s32, b32, _ = ctx.direct_sums_bounded(nodes, abi.OV_PREC_MIXED)
    s64, b64, _ = ctx.direct_sums_bounded(nodes, abi.OV_PREC_FP64)
    ctx.close()
    assert np.all(np.abs(s32 - s64).max(axis=1) <= b32 + b64)


def test_wall_clipping_and_steps_match_reference(golden):
    """enforce_wall_boundaries (connect_to_wall, removal behind walls) and three
    full steps under mirror walls in z, against the reference's own run."""
    g = golden("wall_steps.npz")
    ht = W.HostTangle(g["pos"].copy(), g["conn"][:, 0].copy(), g["conn"][:, 1].copy(), g["box_lo"], g["box_hi"],
                      image_set="wall_2_4")
    p = W.config_params("rings8", rec_dist=8e-4)
    ctx = gpu.Context(0, params=p)
    ctx.upload(ht)
    ctx.enforce_walls(0.0)
    st = ctx.stats()
    n, _, _ = ctx.tangle_info()
    assert n == int(g["enf_N"])
    out = ctx.download_resized(ht)
    np.testing.assert_array_equal(out.conn, g["enf_conn"])
    np.testing.assert_array_equal(out.stat, g["enf_status"])
    used = g["enf_status"][:, 0] != abi.OV_EMPTY
    assert np.abs(out.pos[used] - g["enf_pos"][used]).max() < 1e-14
    assert st["wall_clipped"] > 0 and st["wall_removed"] > 0
    dt = float(g["dt"])
    for s in range(3):
        ctx.step(s * dt, dt)
        assert ctx.stats()["reconnections"] == int(g["recs"][s])
        n, _, _ = ctx.tangle_info()
        assert n == int(g["steps_N"][s])
        out = ctx.download_resized(ht)
        np.testing.assert_array_equal(out.conn, g["steps_conn"][s][:n])
        np.testing.assert_array_equal(out.stat, g["steps_status"][s][:n])
        used = g["steps_status"][s][:n, 0] != abi.OV_EMPTY
        ref = g["steps_pos"][s][:n]
        assert np.abs(out.pos[used] - ref[used]).max() / np.abs(ref[used]).max() < 1e-10
    ctx.close()
