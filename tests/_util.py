"""Shared helpers for the test-suite."""
from __future__ import annotations

import numpy as np

from openvort_gb300 import abi
from openvort_gb300.workloads import HostTangle


def host_from_arrays(d: dict, prefix: str = "") -> HostTangle:
    """Rebuild a HostTangle from the arrays stored in a golden .npz."""
    conn = d[prefix + "conn"]
    st = d[prefix + "status"]
    ht = HostTangle(d[prefix + "pos"].copy(), conn[:, 0].copy(), conn[:, 1].copy(),
                    d[prefix + "box_lo"].copy(), d[prefix + "box_hi"].copy(),
                    n_images=int(d[prefix + "n_images"]), status=st[:, 0].copy())
    ht.stat[:, 1] = st[:, 1]
    return ht


def rel_err(a, b):
    """max_i |a_i - b_i| / max(|b|), the per-array relative error used by the parity gates."""
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    scale = max(np.abs(b).max(), 1e-300)
    return float(np.abs(a - b).max() / scale)


def rel_l2(a, b):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def node_rel_err(a, b):
    """max over nodes of |a_k - b_k| / |b_k| (per-node vector relative error)."""
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    num = np.linalg.norm(a - b, axis=-1)
    den = np.maximum(np.linalg.norm(b, axis=-1), 1e-300)
    return float((num / den).max())


def used(ht_or_status) -> np.ndarray:
    st = ht_or_status if isinstance(ht_or_status, np.ndarray) else ht_or_status.stat
    return st[:, 0] != abi.OV_EMPTY


def check_event_trajectory(g, step, snapshot, pos_tol, pass_log=None):
    """Run the steps of an event golden (tests/golden/make_golden.py,
    event_trajectory) and compare, step by step, with the reference's run.

    step(s) runs main-loop step s and returns its reconnection count, or
    (count, [(k, l), ...]) when it can log the pairs; snapshot() returns
    (conn, status, pos) of every slot.  Gates: reconnections of every step,
    the (k, l) pairs in order where logged, connections and status after
    every step whose topology changed and at the end (bit-exact), positions
    of live nodes at the stored steps within pos_tol (max-abs relative)."""
    steps = len(g["recs"])
    ev = {int(s): i for i, s in enumerate(g["event_steps"])}
    tr = {int(s): i for i, s in enumerate(g["traj_steps"])}
    pairs = [tuple(int(x) for x in row) for row in g["rec_pairs"]]
    got_recs, got_pairs = [], []
    for s in range(steps):
        r = step(s)
        if isinstance(r, tuple):
            r, log = r
            got_pairs += [(s, int(k), int(l)) for k, l in log]
        got_recs.append(int(r))
        assert got_recs[-1] == int(g["recs"][s]), f"step {s}: {got_recs[-1]} reconnections, reference {g['recs'][s]}"
        if s in ev or s in tr:
            conn, status, pos = snapshot()
            n = int(g["n_slots"][s])
            assert len(conn) == n, f"step {s}: {len(conn)} slots, reference {n}"
            if s in ev:
                np.testing.assert_array_equal(conn, g["event_conn"][ev[s]][:n], err_msg=f"connections after step {s}")
                np.testing.assert_array_equal(status, g["event_status"][ev[s]][:n], err_msg=f"status after step {s}")
            if s in tr:
                m = status[:, 0] != abi.OV_EMPTY
                assert rel_err(pos[m], g["traj"][tr[s]][:n][m]) < pos_tol, f"positions after step {s}"
    if pass_log:
        assert got_pairs == pairs
    conn, status, _ = snapshot()
    np.testing.assert_array_equal(conn, g["conn_final"])
    np.testing.assert_array_equal(status, g["status_final"])
    return got_recs
