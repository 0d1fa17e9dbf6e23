"""Error paths, made on the host (needs a GB300; no GPU fault is made).

The reference only prints or runs on for these inputs (octree.c:124 and
:147 print and go on, tangle.c:188 and :217 print); the library returns a
status code instead and leaves the caller's tangle as it was:

  * a NaN position                      -> OV_ERR_NAN, host tangle unchanged
  * a forward index out of range        -> OV_ERR_TOPOLOGY at upload, before any launch
  * a forward link onto an EMPTY slot   -> OV_ERR_TOPOLOGY (the filament walk stops)
  * two nodes at the same position      -> OV_ERR_DEPTH under the strict depth policy (the
                                           reference recurses forever); one leaf by default
  * a device allocation that fails      -> OV_ERR_ALLOC; the context frees its buffers, holds
                                           no tangle, and works again after a new upload

Allocation failures are injected by ov_inject_alloc_failure (the allocation
is not attempted), so no real out-of-memory condition is created.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from openvort_gb300 import abi, gpu, workloads as W
from oracle.pyoracle import Checker
from tests._util import node_rel_err
from tests.test_gpu_dropin import dropin, set_globals  # noqa: F401  (fixture)

pytestmark = pytest.mark.gpu

OV_ERR_ALLOC, OV_ERR_DEPTH, OV_ERR_NAN, OV_ERR_TOPOLOGY, OV_ERR_STATE = 3, 4, 6, 8, 10


def _tangle(seed=81):
    return W.random_walk_tangle(8, 64, D=0.1, seed=seed)


def _expect(code, fn, *args):
    with pytest.raises(gpu.OVError) as e:
        fn(*args)
    assert e.value.code == code, str(e.value)


def test_nan_position_context_api():
    ht = _tangle()
    ht.pos[37, 1] = np.nan
    ctx = gpu.Context(0, params=W.config_params("rw"))
    ctx.upload(ht)
    _expect(OV_ERR_NAN, ctx.update_tangle, 0.0)
    # the context stays usable: a clean tangle evaluates
    clean = _tangle()
    ctx.upload(clean)
    ctx.update_tangle(0.0)
    assert np.all(np.isfinite(ctx.download(clean, abi.OV_F_VELS).vels))
    ctx.close()


def test_nan_position_dropin_leaves_caller_tangle_unchanged(dropin):  # noqa: F811
    port = Checker("port")
    ht = _tangle()
    p = W.config_params("rw")
    set_globals(dropin, p)
    port.set_params(p)
    t = port.tangle(ht)
    v = t.views()
    v["pos"][12, 0] = np.nan
    v["vels"][:] = 7.0
    v["vs"][:] = 7.0
    dropin.ovd_update_velocities(C.byref(t.ts), 0.0)
    assert dropin.ovd_last_status() == OV_ERR_NAN
    assert np.all(t.copy("vels") == 7.0) and np.all(t.copy("vs") == 7.0)
    # the next good call succeeds
    v["pos"][12, 0] = ht.pos[12, 0]
    dropin.ovd_update_tangents_normals(C.byref(t.ts))
    dropin.ovd_update_velocities(C.byref(t.ts), 0.0)
    assert dropin.ovd_last_status() == 0
    t.free()


def test_forward_index_out_of_range_refused_before_any_launch():
    ht = _tangle()
    ht.conn[5, 0] = ht.n + 3
    ctx = gpu.Context(0, params=W.config_params("rw"))
    launches = ctx.kernel_launches
    _expect(OV_ERR_TOPOLOGY, ctx.upload, ht)
    assert ctx.kernel_launches == launches
    _expect(OV_ERR_STATE, ctx.update_tangle, 0.0)
    ctx.close()


def test_forward_link_onto_empty_slot():
    base = _tangle()
    n = base.n
    pos = np.vstack([base.pos, np.full((1, 3), 0.05)])
    fwd = np.append(base.conn[:, 0], -1)
    rev = np.append(base.conn[:, 1], -1)
    status = np.append(base.stat[:, 0], abi.OV_EMPTY)
    fwd[9] = n                          # node 9 now points at the EMPTY slot
    ht = W.HostTangle(pos, fwd, rev, base.box_lo, base.box_hi, status=status)
    ctx = gpu.Context(0, params=W.config_params("rw"))
    ctx.upload(ht)
    _expect(OV_ERR_TOPOLOGY, ctx.update_tangle, 0.0)
    ctx.close()


def test_coincident_nodes_report_depth_when_strict():
    ht = _tangle()
    ht.pos[200] = ht.pos[3]             # nodes of two different loops at one point
    ctx = gpu.Context(0, params=W.config_params("rw"))
    ctx.set_depth_policy(True)
    ctx.upload(ht)
    _expect(OV_ERR_DEPTH, ctx.update_tangle, 0.0)
    ctx.close()


def test_coincident_nodes_share_one_leaf_by_default():
    """Default policy: the deepest shared cell is one leaf.  The two nodes at
    one point skip each other (d < 1e-8, octree.c:311); every other target
    sees the leaf's monopole, whose centre of mass is that point."""
    ht = _tangle()
    ht.pos[200] = ht.pos[3]
    ctx = gpu.Context(0, params=W.config_params("rw"))
    ctx.upload(ht)
    ctx.update_tangle(0.0)
    st = ctx.stats()
    out = ctx.download(ht, abi.OV_F_VELS)
    ctx.close()
    assert st["error_word"] & 1            # OV_EW_DEPTH: reported, not fatal
    assert st["max_depth"] == 21
    assert np.all(np.isfinite(out.vels))


@pytest.mark.parametrize("after", [0, 3, 17, 40])
def test_allocation_failure_then_recovery(after):
    """The (after+1)-th allocation of a fresh context fails, wherever that
    falls in upload + evaluation; the call returns OV_ERR_ALLOC, the
    context holds no tangle, and a new upload gives the same velocities as a
    context that never failed."""
    p = W.config_params("rw")
    ht = _tangle()
    ref = gpu.Context(0, params=p)
    ref.upload(ht)
    ref.update_tangle(0.0)
    want = np.array(ref.download(ht, abi.OV_F_VELS).vels)
    ref.close()

    ctx = gpu.Context(0, params=p)
    ctx.inject_alloc_failure(after)
    failed = False
    try:
        ctx.upload(ht)
        ctx.update_tangle(0.0)
    except gpu.OVError as e:
        assert e.code == OV_ERR_ALLOC, str(e)
        failed = True
    if failed:
        _expect(OV_ERR_STATE, ctx.update_tangle, 0.0)
    ctx.inject_alloc_failure(-1)
    ctx.upload(ht)
    ctx.update_tangle(0.0)
    got = np.array(ctx.download(ht, abi.OV_F_VELS).vels)
    ctx.close()
    assert node_rel_err(got, want) == 0.0
    if after == 0:
        assert failed


def test_allocation_failure_inside_a_time_step():
    """A failure among the reconnection pass's buffers in the middle of ov_step."""
    p = W.config_params("rw")
    ht = W.random_walk_tangle(40, 48, D=0.03, seed=61)    # dense: the step reconnects
    ctx = gpu.Context(0, params=p)
    ctx.upload(ht)
    ctx.update_tangle(0.0)
    ctx.inject_alloc_failure(0)
    _expect(OV_ERR_ALLOC, ctx.step, 0.0, 5e-5)
    ctx.upload(ht)
    ctx.step(0.0, 5e-5)
    ctx.close()
