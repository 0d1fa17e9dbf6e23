"""Mixed-precision traversal against the FP64 tree (needs a GB300).

The mixed path takes the same accept/open decisions as the FP64 path (FP32
outside a guard band, FP64 inside it), so visit and accept counts must be
equal, and velocities must agree within 1e-6 relative L2 (the stated gate).
"""
from __future__ import annotations

import numpy as np
import pytest

from openvort_gb300 import abi, gpu, workloads as W
from tests._util import rel_l2

pytestmark = pytest.mark.gpu

MIXED_TOL = 1e-6


def _eval(ht, p, prec):
    ctx = gpu.Context(0, params=p, precision=prec)
    ctx.upload(ht)
    ctx.update_tangle(0.0)
    ctx.download(ht, abi.OV_F_VELS | abi.OV_F_VS)
    st = ctx.stats()
    ctx.close()
    return np.array(ht.vels), np.array(ht.vs), st


@pytest.mark.parametrize("n_loops,theta", [(256, 0.4), (1024, 0.3), (1024, 0.5)])
def test_mixed_vs_fp64_tree(n_loops, theta):
    ht = W.random_walk_tangle(n_loops, 256, D=0.1, seed=1)
    p = W.config_params("rw", bh_resolution=theta)
    v64, s64, st64 = _eval(ht, p, abi.OV_PREC_FP64)
    v32, s32, st32 = _eval(ht, p, abi.OV_PREC_MIXED)
    assert st32["error_word"] == 0
    assert st32["accepts"] == st64["accepts"] and st32["visits"] == st64["visits"]
    assert rel_l2(v32, v64) < MIXED_TOL
    assert rel_l2(s32, s64) < MIXED_TOL


def test_mixed_rk4_and_edge_cases():
    ht = W.random_walk_tangle(10, 48, D=0.1, seed=24)
    ht.pos[::5] += 0.004
    p = W.config_params("rw")
    v64, _, _ = _eval(ht, p, abi.OV_PREC_FP64)
    v32, _, st = _eval(ht, p, abi.OV_PREC_MIXED)
    assert st["error_word"] == 0
    assert rel_l2(v32, v64) < MIXED_TOL
    # an RK4 step in mixed precision stays within the gate of the FP64 step
    out = []
    for prec in (abi.OV_PREC_FP64, abi.OV_PREC_MIXED):
        h = W.random_walk_tangle(16, 64, D=0.1, seed=50)
        ctx = gpu.Context(0, params=p, precision=prec)
        ctx.upload(h)
        ctx.update_tangle(0.0)
        ctx.rk4_step(0.0, 5e-5)
        ctx.download(h, abi.OV_F_POS)
        ctx.close()
        out.append(np.array(h.pos))
    start = W.random_walk_tangle(16, 64, D=0.1, seed=50).pos
    assert rel_l2(out[1] - start, out[0] - start) < MIXED_TOL


@pytest.mark.parametrize("n_loops,theta,images", [(256, 0.4, None), (1024, 0.3, None), (64, 0.4, "wall_2_4")])
def test_double_single_vs_fp64_tree(n_loops, theta, images):
    """OV_PREC_DD: the mixed walk's decisions with every accepted interaction
    and the sums in double-single: within 1e-10 of the FP64 tree per node and
    1e-12 in relative L2."""
    base = W.random_walk_tangle(n_loops, 256, D=0.1, seed=1)
    ht = base if images is None else W.HostTangle(base.pos.copy(), base.conn[:, 0].copy(), base.conn[:, 1].copy(),
                                                   base.box_lo, base.box_hi, image_set=images)
    p = W.config_params("rw", bh_resolution=theta)
    v64, s64, st64 = _eval(ht, p, abi.OV_PREC_FP64)
    vdd, sdd, stdd = _eval(ht, p, abi.OV_PREC_DD)
    assert stdd["error_word"] == 0
    assert stdd["accepts"] == st64["accepts"] and stdd["visits"] == st64["visits"]
    per_node = np.linalg.norm(vdd - v64, axis=1) / np.linalg.norm(v64, axis=1)
    assert per_node.max() < 1e-10
    assert rel_l2(vdd, v64) < 1e-12
    assert rel_l2(sdd, s64) < 1e-12


def test_mixed_kernel_variants_agree():
    """The periodic-image mixed kernel (variants 2-4, three register budgets)
    takes the decisions and sums of the general one (variants 0, 1) bit for
    bit: same arithmetic, same summation order."""
    ht = W.random_walk_tangle(64, 256, D=0.1, seed=4)
    p = W.config_params("rw")
    ctx = gpu.Context(0, params=p, precision=abi.OV_PREC_MIXED)
    ctx.upload(ht)
    out = []
    for ho in range(5):
        for warps in (4, 8):
            ctx.set_tuning(warps_per_block=warps, high_occupancy=ho)
            ctx.update_tangle(0.0)
            st = ctx.stats()
            assert st["error_word"] == 0
            out.append((ho, warps, st["accepts"], st["visits"], np.array(ctx.download(ht, abi.OV_F_VELS).vels)))
    ctx.close()
    _, _, acc0, vis0, v0 = out[0]
    for ho, warps, acc, vis, v in out[1:]:
        assert acc == acc0 and vis == vis0, (ho, warps)
        np.testing.assert_array_equal(v, v0, err_msg=f"variant {ho}, {warps} warps")
