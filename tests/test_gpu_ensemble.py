"""Batched ensembles (one context, many independent tangles) on the GPU.

Every member of an ensemble must evolve exactly as the same tangle does
alone in its own context: the forest build gives each member the tree it
would have alone, the work-queue traversal only changes which warp computes
which targets, and the topology passes run member by member in the
reference's order.  With the same launch shape (query groups) the FP64 and
the mixed-precision results are therefore identical to the single-tangle
runs; the gate allows 1e-13 relative for safety against a different
summation grouping.
"""
from __future__ import annotations

import numpy as np
import pytest

from openvort_gb300 import abi, gpu, workloads as W
from tests._util import node_rel_err, rel_err, used

pytestmark = pytest.mark.gpu

TUNE = dict(warps_per_block=4, query_groups=3, blocks_per_sm=0, largest_first=1)


def members(D=0.1, sizes=(8, 3, 16, 1, 5), per_loop=64, seed=300):
    """Random-walk members of uneven size with their own alpha, alpha', v_n."""
    out = []
    for i, n_loops in enumerate(sizes):
        ht = W.random_walk_tangle(n_loops, per_loop, D=D, seed=seed + i)
        p = W.config_params("rw", alpha=0.03 + 0.05 * i, alpha_p=0.004 * i,
                            vn=(abi.OV_SIMPLE, 0.2 + 0.4 * i, (1, 0, 0)))
        out.append((ht, p))
    return out


def clone(ht):
    """A fresh host tangle with ht's data (downloads must not alias inputs)."""
    out = W.HostTangle(ht.pos.copy(), ht.conn[:, 0].copy(), ht.conn[:, 1].copy(), ht.box_lo, ht.box_hi,
                       n_images=ht.n_images, status=ht.stat[:, 0].copy())
    out.stat[:, 1] = ht.stat[:, 1]
    return out


def single(ht, p, precision):
    ctx = gpu.Context(0, params=p, precision=precision)
    ctx.set_tuning(**TUNE)
    ctx.upload(ht)
    return ctx


def ensemble(ms, precision, headroom=2.0, tune=TUNE):
    ctx = gpu.Context(0, params=ms[0][1], precision=precision)
    ctx.set_tuning(**tune)
    ctx.upload_ensemble([m[0] for m in ms], [m[1] for m in ms], headroom=headroom)
    return ctx


@pytest.mark.parametrize("precision", [abi.OV_PREC_FP64, abi.OV_PREC_MIXED])
def test_member_velocities_equal_single_runs(precision):
    ms = members()
    ens = ensemble(ms, precision)
    assert ens.ensemble_size == len(ms)
    ens.update_tangle(0.0)
    st = ens.stats()
    total = 0
    for i, (ht, p) in enumerate(ms):
        got = ens.download_member(i, clone(ht))
        ctx = single(ht, p, precision)
        ctx.update_tangle(0.0)
        ref = ctx.download(clone(ht))
        n1 = ctx.stats()["node_evals"]
        ctx.close()
        m = used(ref)
        total += n1
        assert got.n >= ref.n
        np.testing.assert_array_equal(got.conn[:ref.n], ref.conn)
        assert node_rel_err(got.vels[:ref.n][m], ref.vels[m]) <= 1e-13, i
        assert node_rel_err(got.vs[:ref.n][m], ref.vs[m]) <= 1e-13, i
    assert st["node_evals"] == total
    assert st["error_word"] == 0
    ens.close()


def test_queue_order_and_block_shape_do_not_change_results():
    ms = members(sizes=(6, 2, 9))
    outs = []
    for tune in (TUNE, dict(TUNE, largest_first=0, warps_per_block=2),
                 dict(TUNE, warps_per_block=8, blocks_per_sm=1), dict(TUNE, high_occupancy=1)):
        ens = ensemble(ms, abi.OV_PREC_FP64, tune=tune)
        ens.update_tangle(0.0)
        outs.append([ens.download_member(i, clone(ms[i][0])).vels for i in range(len(ms))])
        ens.close()
    for o in outs[1:]:
        for a, b in zip(outs[0], o):
            np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("precision", [abi.OV_PREC_FP64, abi.OV_PREC_MIXED])
def test_rk4_graph_matches_single_runs(precision):
    ms = members(sizes=(4, 7, 2))
    dt = 5e-5
    ens = ensemble(ms, precision)
    ens.update_tangle(0.0)
    for s in range(2):
        ens.rk4_step(s * dt, dt)
        ens.update_tangle((s + 1) * dt)
    for i, (ht, p) in enumerate(ms):
        got = ens.download_member(i, clone(ht))
        ctx = single(ht, p, precision)
        ctx.update_tangle(0.0)
        for s in range(2):
            ctx.rk4_step(s * dt, dt)
            ctx.update_tangle((s + 1) * dt)
        ref = ctx.download(clone(ht))
        ctx.close()
        m = used(ref)
        assert rel_err(got.pos[m], ref.pos[m]) <= 1e-14, i
    ens.close()


def dense_members():
    # dense small boxes (D = 0.03) reconnect and remesh within a few steps
    out = []
    for i, n_loops in enumerate((40, 12, 25)):
        ht = W.random_walk_tangle(n_loops, 48, D=0.03, seed=61 + i)
        p = W.config_params("rw", alpha=0.05 + 0.05 * i, vn=(abi.OV_SIMPLE, 0.3 + 0.5 * i, (1, 0, 0)),
                            dl_max=1.2e-3 - 1e-4 * i)
        out.append((ht, p))
    return out


@pytest.mark.parametrize("headroom", [2.0, 1.0])
def test_full_steps_match_single_runs(headroom):
    """Reconnect, remesh (with member growth past the reserved slots when
    headroom is 1), small loops and RK4, member by member."""
    ms = dense_members()
    dt = 5e-5
    ens = ensemble(ms, abi.OV_PREC_FP64, headroom=headroom)
    recs = []
    for s in range(3):
        ens.step(s * dt, dt)
        recs.append(ens.stats()["reconnections"])
    single_recs = np.zeros(3, dtype=int)
    for i, (ht, p) in enumerate(ms):
        ctx = single(ht, p, abi.OV_PREC_FP64)
        for s in range(3):
            ctx.step(s * dt, dt)
            single_recs[s] += ctx.stats()["reconnections"]
        assert ens.member_info(i) == ctx.tangle_info(), i
        ref = ctx.download_resized(clone(ht))
        got = ens.download_member(i, clone(ht))
        ctx.close()
        np.testing.assert_array_equal(got.conn, ref.conn)
        np.testing.assert_array_equal(got.stat, ref.stat)
        m = used(ref)
        assert rel_err(got.pos[m], ref.pos[m]) <= 1e-12, i
    assert recs == list(single_recs)
    ens.close()


def test_direct_velocities_stay_within_member():
    ms = members(sizes=(3, 5))
    ens = ensemble(ms, abi.OV_PREC_FP64)
    ens.update_tangents_normals()
    n0, _, _ = ens.member_info(0)
    lo1 = int(np.ceil(n0 * 2.0))   # member 1's first slot (headroom 2)
    v_e, _ = ens.direct_velocities(np.array([5, lo1 + 7]))
    for i, k in ((0, 5), (1, 7)):
        ctx = single(*ms[i], abi.OV_PREC_FP64)
        ctx.update_tangents_normals()
        v_s, _ = ctx.direct_velocities(np.array([k]))
        ctx.close()
        assert node_rel_err(v_e[i:i + 1], v_s) <= 1e-13
    ens.close()


def test_autotune_keeps_results():
    ms = members(sizes=(10, 4, 12))
    ens = ensemble(ms, abi.OV_PREC_MIXED)
    ens.update_tangle(0.0)
    before = [ens.download_member(i, clone(ms[i][0])).vels for i in range(len(ms))]
    best, ms_best = ens.autotune(0.0)
    assert best["warps_per_block"] in (2, 4, 8) and 1 <= best["query_groups"] <= 27
    assert ms_best > 0
    ens.update_tangle(0.0)
    for i, b in enumerate(before):
        out = ens.download_member(i, clone(ms[i][0]))
        m = used(out)
        assert node_rel_err(out.vels[m], b[m]) <= 1e-6
    ens.close()


def test_upload_rejects_mismatched_members():
    a = W.random_walk_tangle(2, 32, D=0.1, seed=1)
    b = W.random_walk_tangle(2, 32, D=0.05, seed=2)
    p = W.config_params("rw")
    ctx = gpu.Context(0, params=p)
    with pytest.raises(gpu.OVError):
        ctx.upload_ensemble([a, b], [p, p])
    c = W.random_walk_tangle(2, 32, D=0.1, seed=3)
    with pytest.raises(gpu.OVError):
        ctx.upload_ensemble([a, c], [p, W.config_params("rw", bh_resolution=0.5)])
    ctx.upload_ensemble([a, c], [p, W.config_params("rw", alpha=0.2)])
    with pytest.raises(gpu.OVError):
        ctx.download(clone(a))   # an ensemble downloads member by member
    ctx.close()
