"""FP64 parity at the benchmark configurations' full sizes, against the C
oracle run on the host cores (needs a GB300).

  * precision form: 262,144 nodes (1,024 random-walk loops x 256), theta 0.3
    and 0.5 - every node;
  * large tangle: 1,048,576 nodes (4,096 loops x 256) in D = 0.2 - every node
    of one full update_tangle;
  * batching form: the 48-tangle ensemble at its real member sizes, each
    member with its own alpha, alpha' and v_n - every node of every member;
  * small tangles whose FP64 walks run in parts (1,024 to 12,288 nodes).

Gates: velocities within 1e-10 relative per node of the oracle (the FP64
bar: only summation order differs); and the decisions, node by node: each
target's visited and accepted cell counts equal the reference tree's
(orc_node_interactions).  The GPU builds cell moments bottom-up in child
order while octree.c sums each cell's nodes in index order (octree.c:258-286),
so a centre of mass may differ in the last bit and an opening test
Lm/d < theta (octree.c:319) lying within that bit of theta could go the
other way; a target with such a flip shows up here as a count mismatch.
The number of flipped targets is printed and must be zero.  The mixed
path's per-node counts are compared the same way (it takes the FP64 path's
decisions by construction).
"""
from __future__ import annotations

import os

import numpy as np
import pytest

from openvort_gb300 import abi, gpu, workloads as W
from oracle.pyoracle import Checker

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10
MIXED_L2_TOL = 1e-6
THREADS = os.cpu_count() or 1


@pytest.fixture(scope="module")
def port():
    return Checker("port", fast=False)


def _per_node_rel(a, b):
    num = np.linalg.norm(a - b, axis=1)
    den = np.maximum(np.linalg.norm(b, axis=1), 1e-300)
    return num / den


def _oracle(port, ht, p):
    """Oracle velocities of one update_tangle and per-node counts."""
    p.num_threads = THREADS
    port.set_params(p)
    t = port.tangle(ht)
    port.update_tangle(t, 0.0)
    vels = t.copy("vels")
    vis, acc = port.node_interactions(t, p.bh_resolution, THREADS)
    t.free()
    return vels, vis, acc


def _flips(gv, ga, ov, oa, live):
    return int(np.count_nonzero(((gv != ov) | (ga != oa)) & live))


def _gpu_single(ht, p, precision):
    ctx = gpu.Context(0, params=p, precision=precision)
    ctx.set_node_counting(True)
    ctx.upload(ht)
    ctx.update_tangle(0.0)
    out = ctx.download(ht, abi.OV_F_VELS)
    vis, acc = ctx.node_counts()
    st = ctx.stats()
    ctx.close()
    return np.array(out.vels), vis, acc, st


@pytest.mark.parametrize("loops", [16, 64, 192])
def test_split_walk_parts_every_node(port, loops):
    """Small tangles run each query point's FP64 split walk in parts (32 up to
    2,048 slots, 8 up to 8,192, whole above): 1,024, 4,096 and 12,288 nodes,
    every node and every target's visit/accept counts against the oracle,
    through the counting path and through the default evaluation graph."""
    ht = W.random_walk_tangle(loops, 64, D=0.1, seed=70 + loops)
    p = W.config_params("rw")
    ov, ovis, oacc = _oracle(port, ht, p)
    v64, gvis, gacc, st = _gpu_single(ht, p, abi.OV_PREC_FP64)
    assert st["error_word"] == 0
    assert _flips(gvis, gacc, ovis, oacc, np.ones(ht.n, dtype=bool)) == 0
    assert _per_node_rel(v64, ov).max() < FP64_TOL
    ctx = gpu.Context(0, params=p, precision=abi.OV_PREC_FP64)
    ctx.upload(ht)
    ctx.update_tangle(0.0)
    vg = np.array(ctx.download(ht, abi.OV_F_VELS).vels)
    assert ctx.stats()["accepts"] == int(oacc.sum())
    ctx.close()
    assert _per_node_rel(vg, ov).max() < FP64_TOL


@pytest.mark.parametrize("theta", [0.3, 0.5])
def test_precision_form_262144_every_node(port, theta):
    ht = W.random_walk_tangle(1024, 256, D=0.1, seed=3)
    p = W.config_params("rw", bh_resolution=theta)
    ov, ovis, oacc = _oracle(port, ht, p)
    live = np.ones(ht.n, dtype=bool)
    v64, gvis, gacc, st = _gpu_single(ht, p, abi.OV_PREC_FP64)
    assert st["error_word"] == 0
    flips = _flips(gvis, gacc, ovis, oacc, live)
    err = _per_node_rel(v64, ov)
    print(f"theta {theta}: {ht.n} nodes, flipped targets {flips}, max node rel err {err.max():.2e}, "
          f"visits {gvis.sum()} accepts {gacc.sum()}")
    assert flips == 0
    assert err.max() < FP64_TOL
    vm, mvis, macc, _ = _gpu_single(ht, p, abi.OV_PREC_MIXED)
    assert _flips(mvis, macc, ovis, oacc, live) == 0
    assert np.linalg.norm(vm - ov) / np.linalg.norm(ov) < MIXED_L2_TOL


def test_large_1048576_every_node(port):
    ht = W.random_walk_tangle(4096, 256, D=0.2, seed=5)
    p = W.config_params("large", bh_resolution=0.4)
    ov, ovis, oacc = _oracle(port, ht, p)
    v64, gvis, gacc, st = _gpu_single(ht, p, abi.OV_PREC_FP64)
    assert st["error_word"] == 0
    flips = _flips(gvis, gacc, ovis, oacc, np.ones(ht.n, dtype=bool))
    err = _per_node_rel(v64, ov)
    print(f"large: {ht.n} nodes, flipped targets {flips}, max node rel err {err.max():.2e}")
    assert flips == 0
    assert err.max() < FP64_TOL


def test_ensemble_members_at_real_sizes(port):
    """Every member of the 48-tangle ensemble in one context against the
    oracle run on that member alone with the member's own parameters."""
    ms = W.ensemble(48, 2048, 131072, 256, D=0.1, seed=11)
    hosts = [m.tangle for m in ms]
    params = [W.member_params(m) for m in ms]
    ctx = gpu.Context(0, params=params[0], precision=abi.OV_PREC_FP64)
    ctx.set_node_counting(True)
    ctx.upload_ensemble(hosts, params, headroom=2.0)
    ctx.update_tangle(0.0)
    got = []
    for i, h in enumerate(hosts):
        out = ctx.download_member(i, W.HostTangle(h.pos.copy(), h.conn[:, 0].copy(), h.conn[:, 1].copy(),
                                                  h.box_lo, h.box_hi, n_images=h.n_images), abi.OV_F_VELS)
        vis, acc = ctx.node_counts(i, h.n)
        got.append((np.array(out.vels[:h.n]), vis, acc))
    assert ctx.stats()["error_word"] == 0
    ctx.close()
    total_flips, worst = 0, 0.0
    for i, (h, p) in enumerate(zip(hosts, params)):
        ov, ovis, oacc = _oracle(port, h, p)
        v, gvis, gacc = got[i]
        total_flips += _flips(gvis, gacc, ovis, oacc, np.ones(h.n, dtype=bool))
        worst = max(worst, float(_per_node_rel(v, ov).max()))
    print(f"ensemble: {len(hosts)} members, {sum(h.n for h in hosts)} nodes, flipped targets {total_flips}, "
          f"max node rel err {worst:.2e}")
    assert total_flips == 0
    assert worst < FP64_TOL
