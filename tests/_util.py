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
