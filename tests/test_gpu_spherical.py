"""The spherical fork's velocity path (src_spherical/ of OpenVort) on the GPU.

The domain is a section of a spherical shell repeated by rotations, with
the inner surface a wall represented by the spherical inversion of the
tangle.  Golden vectors come from the fork itself, compiled here
(oracle/Makefile, tests/golden/make_golden.py ``spherical``): tangents,
normals, velocities and superfluid velocities after update_tangents_normals
and update_velocities, with and without the He II temperature model, on
seeded rings (some across the azimuth edge, outside the section), a radial
line pinned on both surfaces (slipping on the inner one) and EMPTY slots.

The fork's angles go through atan2 / sin / cos; the GPU's differ from the
host libm's in the last bit, so positions rebuilt from angles agree to
rounding and the comparison is to 1e-10 per node (tangents 1e-12).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np
import pytest

from openvort_gb300 import abi, gpu, workloads as W
from tests._util import node_rel_err

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CASES = ["plain", "temperature"]
WALKS = [abi.OV_WALK_SPLIT, abi.OV_WALK_FP64]


def sph_from_golden(g):
    return W.SphTangle(g["pos"].copy(), g["conn"][:, 0].copy(), g["conn"][:, 1].copy(), g["status"][:, 0].copy(),
                       g["status"][:, 1].copy(), tuple(g["domain"]))


def params(case):
    p = gpu.sph_params_default()
    p.use_temperature = 1 if case == "temperature" else 0
    return p


def test_helium_model_matches_the_fork(golden):
    """The He II model (densities, entropy, alpha, alpha') on the host equals
    the fork's values bit for bit (no GPU)."""
    g = golden("spherical.npz")
    for T, ref in zip(g["helium_T"], g["helium"]):
        np.testing.assert_array_equal(gpu.sph_helium(T), ref)
    with pytest.raises(gpu.OVError):
        gpu.sph_helium(2.5)   # above the lambda point: the fork exits


def test_oracle_restatement_is_bit_identical_to_fork(golden):
    """The C restatement of the fork's velocity path (oracle/ov_oracle_sph.c)
    reproduces the fork's tangents, normals and velocities bit for bit."""
    from oracle.pyoracle import sph_update_tangle
    g = golden("spherical.npz")
    for case in CASES:
        sph = sph_from_golden(g)
        sph_update_tangle(sph, params(case), threads=4)
        live = g["status"][:, 0] != abi.OV_EMPTY
        for name in ("tangents", "normals", "vels", "vs"):
            np.testing.assert_array_equal(getattr(sph, name)[live], g[f"{case}_{name}"][live])


def test_workload_matches_golden(golden):
    g = golden("spherical.npz")
    s = W.spherical_tangle()
    np.testing.assert_array_equal(s.pos, g["pos"])
    np.testing.assert_array_equal(s.conn, g["conn"])


@pytest.mark.gpu
@pytest.mark.parametrize("walk", WALKS)
@pytest.mark.parametrize("case", CASES)
def test_update_tangle_matches_fork(golden, case, walk):
    g = golden("spherical.npz")
    sph = sph_from_golden(g)
    ctx = gpu.Context(0)
    ctx.set_walk(walk)
    ctx.sph_update(sph, params(case), 0.0)
    st = ctx.stats()
    ctx.close()
    live = g["status"][:, 0] != abi.OV_EMPTY
    assert node_rel_err(sph.tangents[live], g[f"{case}_tangents"][live]) < 1e-12
    # normals of the straight radial line are rounding noise: scale by the largest
    ref_n = g[f"{case}_normals"][live]
    assert np.abs(sph.normals[live] - ref_n).max() < 1e-10 * np.abs(ref_n).max()
    free = live & (g["status"][:, 0] != abi.OV_PINNED)
    assert node_rel_err(sph.vels[free], g[f"{case}_vels"][free]) < 1e-10
    assert node_rel_err(sph.vs[live], g[f"{case}_vs"][live]) < 1e-10
    assert st["visits"] > 0 and st["accepts"] > 0


@pytest.mark.gpu
def test_velocities_use_the_given_tangents(golden):
    """update_velocities alone reads the tangents and normals the caller
    holds; tangents alone leave velocities untouched."""
    g = golden("spherical.npz")
    sph = sph_from_golden(g)
    sph.tangents[:], sph.normals[:] = g["plain_tangents"], g["plain_normals"]
    ctx = gpu.Context(0)
    ctx.sph_update(sph, params("plain"), 0.0, tangents=False)
    free = (g["status"][:, 0] != abi.OV_EMPTY) & (g["status"][:, 0] != abi.OV_PINNED)
    assert node_rel_err(sph.vels[free], g["plain_vels"][free]) < 1e-10
    sph2 = sph_from_golden(g)
    sph2.vels[:] = 7.0
    ctx.sph_update(sph2, params("plain"), 0.0, velocities=False)
    ctx.close()
    assert np.all(sph2.vels == 7.0)
    live = g["status"][:, 0] != abi.OV_EMPTY
    assert node_rel_err(sph2.tangents[live], g["plain_tangents"][live]) < 1e-12


@pytest.mark.gpu
def test_outer_surface_wall_is_refused(golden):
    g = golden("spherical.npz")
    p = params("plain")
    p.outer_surface = 1
    ctx = gpu.Context(0)
    with pytest.raises(gpu.OVError):
        ctx.sph_update(sph_from_golden(g), p, 0.0)
    ctx.close()


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES)
def test_mixed_precision_matches_fp64_tree(golden, case):
    """The mixed path on the fork's geometry: FP32 walks with the FP64
    decisions (same visits and accepts), within 1e-6 relative L2 of FP64."""
    g = golden("spherical.npz")
    a, b = sph_from_golden(g), sph_from_golden(g)
    ctx = gpu.Context(0)
    ctx.sph_update(a, params(case), 0.0)
    s64 = ctx.stats()
    ctx.set_precision(abi.OV_PREC_MIXED)
    ctx.sph_update(b, params(case), 0.0)
    s32 = ctx.stats()
    ctx.close()
    free = (g["status"][:, 0] != abi.OV_EMPTY) & (g["status"][:, 0] != abi.OV_PINNED)
    err = np.linalg.norm(b.vels[free] - a.vels[free]) / np.linalg.norm(a.vels[free])
    assert err < 1e-6
    assert s32["visits"] == s64["visits"] and s32["accepts"] == s64["accepts"]


@pytest.mark.gpu
@pytest.mark.parametrize("walk", WALKS)
@pytest.mark.parametrize("case", CASES)
def test_larger_tangle_vs_oracle(case, walk):
    """A larger seeded tangle (96 rings, other seed) against the C restatement."""
    from oracle.pyoracle import sph_update_tangle
    a = W.spherical_tangle(n_rings=96, seed=11)
    b = W.spherical_tangle(n_rings=96, seed=11)
    ctx = gpu.Context(0)
    ctx.set_walk(walk)
    ctx.sph_update(a, params(case), 0.0)
    ctx.close()
    sph_update_tangle(b, params(case), threads=8)
    free = (b.stat[:, 0] != abi.OV_EMPTY) & (b.stat[:, 0] != abi.OV_PINNED)
    live = b.stat[:, 0] != abi.OV_EMPTY
    assert node_rel_err(a.tangents[live], b.tangents[live]) < 1e-12
    assert node_rel_err(a.vels[free], b.vels[free]) < 1e-10
    assert node_rel_err(a.vs[live], b.vs[live]) < 1e-10


@pytest.mark.gpu
def test_split_walk_equals_fp64_walk():
    """The FP64 path's two walks on the fork's geometry: the same visits and
    accepts, velocities a few ulps apart."""
    out = []
    for walk in WALKS:
        t = W.spherical_tangle(n_rings=160, seed=3)
        ctx = gpu.Context(0)
        ctx.set_walk(walk)
        ctx.sph_update(t, params("temperature"), 0.0)
        out.append((t, ctx.stats()))
        ctx.close()
    (a, sa), (b, sb) = out
    assert sa["visits"] == sb["visits"] and sa["accepts"] == sb["accepts"]
    free = (a.stat[:, 0] != abi.OV_EMPTY) & (a.stat[:, 0] != abi.OV_PINNED)
    assert node_rel_err(a.vels[free], b.vels[free]) < 1e-12
