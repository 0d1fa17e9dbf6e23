"""Injection: add_loop, add_line_in_zdir and inject_vortices
(src/vortex_injection.c:18-100, 267-319, 702-800) against the reference.

Golden vectors come from the reference itself (tests/golden/make_golden.py,
``injection``): the slots, connections, statuses and bookkeeping after each
call on a wall tangle with a freed ring (slot reuse, pool doubling, both
branches of ``perpendicular``), and three main-loop steps that start with
inject_vortices under mirror walls in z (a loop injected through the top
wall every step after the first, a pinned line pair at the third).  The
draws come from drand48's recurrence, restated host-side and checked here
against the reference process's own draws.

Positions are compared to a few ulps: the ring points go through the host
libm's cos / sin, whose last bit may differ between builds of it.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from openvort_gb300 import abi, gpu, workloads as W

CALLS = [("loop", (0.05, 0.05, 0.05), (1.0, 0.0, 0.0), 0.004), ("loop", (0.03, 0.06, 0.02), (0.3, -0.5, 0.8), 0.02),
         ("line", 0.031, 0.077, +1), ("line", 0.062, 0.018, -1), ("loop", (0.07, 0.02, 0.09), (0, 0, -1), 0.009)]


def test_rand48_matches_reference_stream(golden):
    """The host restatement of drand48 reproduces the reference process's
    draws after srand48(seed) (no GPU)."""
    g = golden("inject.npz")
    st = (C.c_ushort * 3)(*abi.srand48_state(int(g["rand_seed"])))
    ours = np.array([gpu.erand48(st) for _ in range(len(g["rand_draws"]))])
    np.testing.assert_array_equal(ours, g["rand_draws"])


def test_rand48_matches_libc_erand48():
    try:
        libc = C.CDLL("libc.so.6")
    except OSError:
        pytest.skip("no glibc")
    libc.erand48.restype = C.c_double
    libc.erand48.argtypes = [C.POINTER(C.c_ushort)]
    a = (C.c_ushort * 3)(0x1234, 0xBEEF, 0x0042)
    b = (C.c_ushort * 3)(*a)
    for _ in range(200):
        assert gpu.erand48(a) == libc.erand48(b)
    assert list(a) == list(b)


def wall_tangle(g, image_set="wall_2_4"):
    return W.HostTangle(g["pos"].copy(), g["conn"][:, 0].copy(), g["conn"][:, 1].copy(), g["box_lo"], g["box_hi"],
                        image_set=image_set, status=g["status"][:, 0].copy())


def assert_state(ctx, host, g, prefix, rtol=8e-16):
    n, ne, te = ctx.tangle_info()
    assert n == int(g[f"{prefix}N"])
    assert (ne, te) == (int(g[f"{prefix}next_empty"]), int(g[f"{prefix}total_empty"]))
    out = ctx.download_resized(host)
    np.testing.assert_array_equal(out.conn, g[f"{prefix}conn"])
    np.testing.assert_array_equal(out.stat, g[f"{prefix}status"])
    used = g[f"{prefix}status"][:, 0] != abi.OV_EMPTY
    ref = g[f"{prefix}pos"][used]
    assert np.abs(out.pos[used] - ref).max() <= rtol * np.abs(ref).max()


@pytest.mark.gpu
def test_add_loop_and_lines_match_reference(golden):
    g = golden("inject.npz")
    ht = wall_tangle(g)
    p = W.config_params("rings8", rec_dist=8e-4)
    ctx = gpu.Context(0, params=p)
    ctx.upload(ht)
    for k, call in enumerate(CALLS):
        p.pin_mode = abi.OV_PINNED if k < 3 else abi.OV_PINNED_SLIP
        ctx.set_params(p)
        if call[0] == "loop":
            ctx.add_loop(call[1], call[2], call[3])
        else:
            ctx.add_line_in_zdir(call[1], call[2], call[3])
        added = ctx.stats()["injected_nodes"]
        assert added == int((g[f"c{k}_status"][:, 0] != abi.OV_EMPTY).sum()) - \
            int((g[f"c{k - 1}_status" if k else "status"][:, 0] != abi.OV_EMPTY).sum())
        assert_state(ctx, ht, g, f"c{k}_")
    ctx.close()


def injection_conf(g, seed=None):
    return abi.make_injection(seed=int(g["inj_seed"]) if seed is None else seed,
                              loop_frequency=float(g["inj_loop_frequency"]), line_n=int(g["inj_line_n"]),
                              line_frequency=float(g["inj_line_frequency"]),
                              line_polarized=bool(g["inj_line_polarized"]))


def check_steps(ctx, ht, g, member=None):
    dt = float(g["dt"])
    for s in range(3):
        ctx.step(s * dt, dt)
        if member is None:
            assert ctx.stats()["reconnections"] == int(g["recs"][s])
            n, _, _ = ctx.tangle_info()
            out = ctx.download_resized(ht)
        else:
            n = ctx.member_info(member)[0]
            out = ctx.download_member(member)
        assert n == int(g["steps_N"][s])
        np.testing.assert_array_equal(out.conn, g["steps_conn"][s][:n])
        np.testing.assert_array_equal(out.stat, g["steps_status"][s][:n])
        used = g["steps_status"][s][:n, 0] != abi.OV_EMPTY
        ref = g["steps_pos"][s][:n]
        assert np.abs(out.pos[used] - ref[used]).max() / np.abs(ref[used]).max() < 1e-10


@pytest.mark.gpu
def test_inject_steps_match_reference(golden):
    """inject_vortices at the top of each main-loop step (main.c:123-141)."""
    g = golden("inject_steps.npz")
    ht = wall_tangle(g)
    ctx = gpu.Context(0, params=W.config_params("rings8", rec_dist=8e-4))
    ctx.upload(ht)
    ctx.set_injection(injection_conf(g))
    check_steps(ctx, ht, g)
    st = ctx.get_injection().rand48
    assert gpu.erand48(st) == float(g["next_draw"])
    ctx.close()


@pytest.mark.gpu
def test_injection_off_changes_nothing(golden):
    """Injection settings with both kinds off: no draws, no nodes."""
    g = golden("inject_steps.npz")
    ht = wall_tangle(g)
    ctx = gpu.Context(0, params=W.config_params("rings8", rec_dist=8e-4))
    ctx.upload(ht)
    inj = abi.make_injection(seed=5)
    ctx.set_injection(inj)
    ctx.inject_vortices(10.0)
    assert ctx.stats()["injected_nodes"] == 0
    assert list(ctx.get_injection().rand48) == list(inj.rand48)
    assert ctx.tangle_info()[0] == ht.n
    ctx.close()


@pytest.mark.gpu
def test_ensemble_members_inject_from_their_own_streams(golden):
    """Two members with different seeds: the member seeded as the reference
    run follows it step for step; the other draws a different stream."""
    g = golden("inject_steps.npz")
    ht = wall_tangle(g)
    p = W.config_params("rings8", rec_dist=8e-4)
    ctx = gpu.Context(0, params=p)
    ctx.upload_ensemble([wall_tangle(g), ht], [p, p])
    ctx.set_injection(injection_conf(g, seed=1), member=0)
    ctx.set_injection(injection_conf(g), member=1)
    check_steps(ctx, ht, g, member=1)
    assert list(ctx.get_injection(0).rand48) != list(ctx.get_injection(1).rand48)
    ctx.close()
