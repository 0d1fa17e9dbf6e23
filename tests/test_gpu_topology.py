"""Topology passes and full time steps on the GPU against OpenVort's own
outputs (golden vectors) and the C oracle (needs a GB300).

Gates: reconnection counts, connections and status identical; positions
within 1e-10 of the reference (FP64 path; only summation order differs).
"""
from __future__ import annotations

import numpy as np
import pytest

from openvort_gb300 import abi, gpu, workloads as W
from oracle.pyoracle import Checker
from tests._util import check_event_trajectory, host_from_arrays, rel_err, used

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["rings8_steps.npz", "crossing_steps.npz"])
@pytest.mark.parametrize("mode", ["step", "passes"])
def test_200_steps_event_log_matches_reference(golden, name, mode):
    """The 8-ring configuration (496 nodes; no reconnection in 200 steps) and
    crossing ring pairs (992 nodes; 12 reconnections at steps 0-158): 200
    main-loop steps on the GPU leave the reference's reconnection counts, the
    topology after every step that changed it, and positions within 1e-10.
    mode "step" runs ov_step; "passes" runs the passes one by one and also
    checks the (k, l) pairs of every reconnection, in order."""
    g = golden(name)
    ht = host_from_arrays(g)
    p = W.config_params("rings8")
    ctx = gpu.Context(0, params=p)
    ctx.upload(ht)
    dt = float(g["dt"])

    def step(s):
        if mode == "step":
            ctx.step(s * dt, dt)
            return ctx.stats()["reconnections"]
        ctx.eliminate_small_loops()
        r = ctx.reconnect(0.0, log=True)
        ctx.eliminate_small_loops()
        ctx.enforce_periodic()
        ctx.remesh(p.dl_min, p.dl_max, 0.0)
        ctx.eliminate_small_loops()
        ctx.update_tangle(s * dt)
        ctx.rk4_step(s * dt, dt)
        ctx.enforce_periodic()
        return r

    def snapshot():
        out = ctx.download_resized(ht)
        return out.conn.copy(), out.stat.copy(), out.pos.copy()

    recs = check_event_trajectory(g, step, snapshot, 1e-10, pass_log=(mode == "passes"))
    ctx.close()
    assert sum(recs) == (0 if name.startswith("rings8") else 12)


@pytest.mark.parametrize("name,cfg", [("dense_steps.npz", "rw")])
def test_full_steps_match_reference(golden, name, cfg):
    g = golden(name)
    ht = host_from_arrays(g)
    p = W.config_params(cfg)
    ctx = gpu.Context(0, params=p)
    ctx.upload(ht)
    dt = float(g["dt"])
    recs = []
    steps = g["traj_steps"] if "traj_steps" in g else np.arange(len(g["recs"]))
    for s in range(len(g["recs"])):
        ctx.step(s * dt, dt)
        recs.append(ctx.stats()["reconnections"])
        if name.startswith("dense"):
            out = ctx.download_resized(ht)
            np.testing.assert_array_equal(out.conn, g["conn_steps"][s])
            np.testing.assert_array_equal(out.stat, g["status_steps"][s])
            m = used(g["status_steps"][s])
            assert rel_err(out.pos[m], g["traj"][s][m]) < 1e-10
        elif s in steps:
            out = ctx.download_resized(ht)
            i = list(steps).index(s)
            m = used(out.stat)
            assert rel_err(out.pos[m], g["traj"][i][m]) < 1e-10
    assert recs == list(g["recs"])
    if "conn_final" in g:
        out = ctx.download_resized(ht)
        np.testing.assert_array_equal(out.conn, g["conn_final"])
    ctx.close()


@pytest.mark.parametrize("tag", ["coarse", "fine"])
def test_remesh_matches_reference(golden, tag):
    g = golden("remesh.npz")
    ht = host_from_arrays(g, prefix=f"{tag}_in_")
    ctx = gpu.Context(0, params=W.config_params("rw"))
    ctx.upload(ht)
    ctx.remesh(5e-4, 1.5e-3, 0.0)
    n, _, _ = ctx.tangle_info()
    assert n == int(g[f"{tag}_N"])
    out = ctx.download_resized(ht)
    ctx.close()
    np.testing.assert_array_equal(out.conn, g[f"{tag}_conn"])
    np.testing.assert_array_equal(out.stat, g[f"{tag}_status"])
    m = used(g[f"{tag}_status"])
    assert rel_err(out.pos[m], g[f"{tag}_pos"][m]) < 1e-12


@pytest.mark.parametrize("n_loops,per_loop,D", [(40, 48, 0.03), (96, 64, 0.04)])
def test_reconnect_log_and_small_loops_vs_oracle(n_loops, per_loop, D):
    """The reconnection log (pairs in order), small-loop removal, connections
    and status equal the oracle's.  The denser case rewires often enough that
    most decisions use copies of the corrections lacking the last rewirings,
    covered by their bound."""
    port = Checker("port")
    ht = W.random_walk_tangle(n_loops, per_loop, D=D, seed=61)
    p = W.config_params("rw")
    port.set_params(p)
    t = port.tangle(ht)
    n_ref, log_ref = port.reconnect(t, 0.0, log=True)
    removed_ref = port.eliminate_small_loops(t)
    ctx = gpu.Context(0, params=p)
    ctx.upload(ht)
    n_gpu, log_gpu = ctx.reconnect(0.0, log=True)
    ctx.eliminate_small_loops()
    st = ctx.stats()
    out = ctx.download_resized(ht)
    ctx.close()
    assert n_ref > 0 and n_gpu == n_ref and log_gpu == log_ref
    assert st["small_loops_removed"] == removed_ref
    print("reconnections", n_gpu, "lazy evaluations", st["reconnect_lazy_evals"], "of", st["reconnect_evaluated"])
    np.testing.assert_array_equal(out.conn, t.copy("conn"))
    np.testing.assert_array_equal(out.stat, t.copy("status"))


def test_smoothing_vs_oracle():
    port = Checker("port")
    ht = W.random_walk_tangle(12, 64, D=0.1, seed=62)
    # one loop spans more than half the box so the detrended branch runs too
    k = np.arange(64)
    ht.pos[:64] = np.stack([np.mod(0.01 + k * 0.1 / 64 * 1.0, 0.1), 0.05 + 0.002 * np.sin(k), 0.05 + 0 * k], 1)
    p = W.config_params("rw", use_freq_filter=1, freq_to_cutoff=0.8)
    port.set_params(p)
    t = port.tangle(ht)
    port.smooth(t)
    ctx = gpu.Context(0, params=p)
    ctx.upload(ht)
    ctx.smooth()
    out = ctx.download(ht, abi.OV_F_POS)
    ctx.close()
    ref = t.copy("pos")
    assert np.abs(out.pos - ref).max() < 1e-12
    assert np.abs(ref - W.random_walk_tangle(12, 64, D=0.1, seed=62).pos[:]).max() > 0  # it smoothed


def test_remesh_grows_pool_like_expand_tangle():
    # every segment longer than dl_max: the pool must double, as expand_tangle does
    ht = W.random_walk_tangle(2, 20, D=0.1, delta=4e-3, seed=63)
    port = Checker("port")
    p = W.config_params("rw")
    port.set_params(p)
    t = port.tangle(ht)
    port.remesh(t, p.dl_min, p.dl_max, 0.0)
    ctx = gpu.Context(0, params=p)
    ctx.upload(ht)
    ctx.remesh(p.dl_min, p.dl_max, 0.0)
    out = ctx.download_resized(ht)
    n, ne, te = ctx.tangle_info()
    ctx.close()
    assert n == t.n and n > ht.n
    np.testing.assert_array_equal(out.conn, t.copy("conn"))
    m = used(out.stat)
    assert rel_err(out.pos[m], t.copy("pos")[m]) < 1e-12


@pytest.mark.parametrize("n_loops,D", [(64, 0.1), (40, 0.03)])
def test_reconnect_sums_within_their_bound(n_loops, D):
    """The mixed-precision direct sums reconnect decides with stay within
    their own error bound of the FP64 sums, and the FP64 sums match the
    oracle's direct sums (nonlocal part) to 1e-12 relative."""
    ht = W.random_walk_tangle(n_loops, 64 if D == 0.1 else 48, D=D, seed=77)
    ctx = gpu.Context(0, params=W.config_params("rw"))
    ctx.upload(ht)
    nodes = np.arange(0, ht.n, max(1, ht.n // 300))
    s32, b32, mag = ctx.direct_sums_bounded(nodes, abi.OV_PREC_MIXED)
    s64, b64, _ = ctx.direct_sums_bounded(nodes, abi.OV_PREC_FP64)
    # double-single far terms: the refinement reconnect uses for undecided pairs
    sdd, bdd, _ = ctx.direct_sums_bounded(nodes, abi.OV_PREC_DD)
    ctx.close()
    err = np.abs(s32 - s64).max(axis=1)
    assert np.all(err <= b32 + b64), (err / b32).max()
    assert np.all(b32 > 0) and np.all(b32 < 1e-4 * mag + 1e-300)
    err_dd = np.abs(sdd - s64).max(axis=1)
    assert np.all(err_dd <= bdd + b64), (err_dd / bdd).max()
    assert np.all(bdd < 2e-10 * mag + 1e-300)
    assert np.all(err_dd <= 1e-3 * bdd + b64)   # the bound is loose by orders of magnitude
    # with zero tangents/normals (as uploaded) and no v_s, the oracle's
    # update_velocity(k, NULL) is the nonlocal sum alone
    assert not ht.tangents.any() and not ht.normals.any()
    port = Checker("port")
    port.set_params(W.config_params("rw"))
    t = port.tangle(ht)
    _, vs_ref = port.direct_velocities(t, nodes)
    assert rel_err(s64, vs_ref) < 1e-12


@pytest.mark.parametrize("detrend", [False, True])
def test_long_loop_smoothing_vs_oracle(detrend):
    """Loops longer than one block's shared memory go through the Bluestein
    FFT path; the result equals the restatement's direct DFT low-pass."""
    n = 3000
    k = np.arange(n)
    rng = np.random.default_rng(5)
    if detrend:
        # a loop that winds once around the periodic box in x (gap > L/2 after unwrapping)
        pos = np.stack([np.mod(k * 0.1 / n, 0.1), 0.05 + 0.003 * np.sin(2 * np.pi * 7 * k / n),
                        0.05 + 0.002 * rng.standard_normal(n) * 0.1], 1)
    else:
        th = 2 * np.pi * k / n
        pos = np.stack([0.05 + 0.03 * np.cos(th), 0.05 + 0.03 * np.sin(th),
                        0.05 + 0.0005 * rng.standard_normal(n)], 1)
    pos0 = pos.copy()   # the host tangle holds `pos` itself, which the download overwrites
    ht = W.HostTangle(pos, (k + 1) % n, (k - 1) % n, np.zeros(3), np.full(3, 0.1), n_images=26)
    p = W.config_params("rw", use_freq_filter=1, freq_to_cutoff=0.8)
    port = Checker("port")
    port.set_params(p)
    t = port.tangle(ht)
    port.smooth(t)
    ctx = gpu.Context(0, params=p)
    ctx.upload(ht)
    ctx.smooth()
    out = ctx.download(ht, abi.OV_F_POS)
    ctx.close()
    ref = t.copy("pos")
    assert np.abs(out.pos - ref).max() < 1e-12
    assert np.abs(ref - pos0).max() > 1e-6   # it smoothed
