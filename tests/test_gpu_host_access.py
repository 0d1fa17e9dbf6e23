"""Uploads and downloads through the caller's arrays in place (a device that
reads and writes pageable host memory through the host's page tables)
against the staged copies: the same device state and the same host arrays,
bit for bit, for whole-tangle and per-field transfers, in a single context
and in a context whose capacity exceeds the tangle (EMPTY slots past N)."""
from __future__ import annotations

import numpy as np
import pytest

from openvort_gb300 import abi, gpu, workloads as W

pytestmark = pytest.mark.gpu

FIELDS = ("pos", "vels", "vs", "tangents", "normals", "conn", "stat")


def _run(direct: bool):
    ht = W.random_walk_tangle(16, 64, D=0.1, seed=5)
    ctx = gpu.Context(0, params=W.config_params("rw"))
    ctx.set_host_access(direct)
    ctx.upload(ht)
    ctx.update_tangle(0.0)
    ctx.download(ht)
    first = {k: np.array(getattr(ht, k)) for k in FIELDS}
    # positions and topology only, then velocities only
    ht.pos[:] = ht.pos + 1e-6
    ctx.upload_fields(ht, abi.OV_F_POS | abi.OV_F_TOPOLOGY)
    ctx.update_tangle(0.0)
    ctx.download(ht, abi.OV_F_VELS)
    second = {k: np.array(getattr(ht, k)) for k in FIELDS}
    in_place = ctx.host_access_direct
    ctx.close()
    return first, second, in_place


def test_in_place_transfers_equal_staged_copies():
    staged = _run(False)
    direct = _run(True)
    assert not staged[2]
    for a, b in zip(staged[:2], direct[:2]):
        for k in FIELDS:
            assert np.array_equal(a[k], b[k]), k
    assert np.all(np.isfinite(direct[1]["vels"])) and np.abs(direct[1]["vels"]).max() > 0


def test_download_into_a_larger_host_tangle():
    """Host slots past the device's N become EMPTY with zero vectors on both paths."""
    outs = []
    for direct in (False, True):
        ht = W.random_walk_tangle(8, 64, D=0.1, seed=9)
        ctx = gpu.Context(0, params=W.config_params("rw"))
        ctx.set_host_access(direct)
        ctx.upload(ht)
        ctx.update_tangle(0.0)
        big = W.HostTangle(np.vstack([ht.pos, np.ones((7, 3))]), np.append(ht.conn[:, 0], [-1] * 7),
                           np.append(ht.conn[:, 1], [-1] * 7), ht.box_lo, ht.box_hi)
        big.vels[:] = 5.0
        ctx.download(big, abi.OV_F_VELS | abi.OV_F_TOPOLOGY)
        ctx.close()
        outs.append((np.array(big.vels), np.array(big.conn), np.array(big.stat)))
        assert np.all(big.vels[ht.n:] == 0) and np.all(big.stat[ht.n:, 0] == abi.OV_EMPTY)
    for a, b in zip(*outs):
        assert np.array_equal(a, b)
