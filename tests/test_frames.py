"""Frame files in the reference's text format (save_tangle / load_tangle,
utils.c:68-199) - host code, no GPU.

The writer must produce the reference's files byte for byte (including its
loop walk, which treats slot 0 as "no node" in two places), and the reader
must leave the tangle load_tangle leaves: slots, connections, status, the
numbers, and the empty-slot bookkeeping of expand_tangle.  Checked against
the reference compiled here (oracle/_ref) and against a committed frame the
reference wrote (tests/golden/frame_walls.txt, made by make_golden.py).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np
import pytest

from openvort_gb300 import abi, gpu, workloads as W
from oracle.pyoracle import reference_available

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")


def sample_tangle():
    """Closed loops, an open line pinned at both ends, slot 0 inside a loop,
    empty slots, and filled velocities / tangents / normals."""
    ht = W.random_walk_tangle(3, 12, D=0.1, seed=41)
    n = ht.n + 8
    pos = np.zeros((n, 3)); pos[:ht.n] = ht.pos
    fwd = np.full(n, -1); rev = np.full(n, -1); st = np.full(n, abi.OV_EMPTY)
    fwd[:ht.n], rev[:ht.n], st[:ht.n] = ht.conn[:, 0], ht.conn[:, 1], abi.OV_FREE
    # open line in slots n-6 .. n-3 (pinned ends), slots n-8, n-7, n-2, n-1 empty
    line = list(range(n - 6, n - 2))
    for a, b in zip(line[:-1], line[1:]):
        fwd[a], rev[b] = b, a
    st[line] = abi.OV_FREE
    st[line[0]] = st[line[-1]] = abi.OV_PINNED
    pos[line] = [[0.01 * i, 0.02, 0.0] for i in range(len(line))]
    out = W.HostTangle(pos, fwd, rev, np.zeros(3), np.full(3, 0.1), status=st)
    out.stat[line[0], 1], out.stat[line[-1], 1] = 0, 1
    rng = np.random.default_rng(3)
    out.vels[:] = rng.standard_normal((n, 3))
    out.tangents[:] = rng.standard_normal((n, 3))
    out.normals[:] = rng.standard_normal((n, 3)) * 1e-7
    return out


def test_write_then_read_round_trip(tmp_path):
    ht = sample_tangle()
    path = str(tmp_path / "f.txt")
    gpu.write_frame(ht, path, digits=17)
    back, (ne, te) = gpu.read_frame(path, n0=4)
    n = back.n
    assert n >= ht.n
    used = ht.stat[:, 0] != abi.OV_EMPTY
    # save_tangle skips slot 0 when it closes a loop walked from a later start; here slot 0 starts one
    np.testing.assert_array_equal(back.stat[:ht.n][used], ht.stat[used])
    np.testing.assert_array_equal(back.pos[:ht.n][used], ht.pos[used])
    np.testing.assert_array_equal(back.conn[:ht.n][used], ht.conn[used])


@pytest.mark.skipif(not reference_available(), reason="OpenVort checkout not built here")
@pytest.mark.parametrize("digits", [15])
def test_writer_matches_reference_save_tangle(tmp_path, digits):
    from oracle.pyoracle import Checker
    ref = Checker("reference")
    ht = sample_tangle()
    t = ref.tangle(ht)
    v = t.views()
    v["vels"][:] = ht.vels
    v["tangents"][:] = ht.tangents
    v["normals"][:] = ht.normals
    ours, theirs = str(tmp_path / "ours.txt"), str(tmp_path / "theirs.txt")
    ref.lib.save_tangle.argtypes = [C.c_char_p, C.c_void_p]
    ref.lib.save_tangle(theirs.encode(), C.addressof(t.ts))
    gpu.write_frame(ht, ours, digits=digits)
    assert open(ours).read() == open(theirs).read()
    t.free()


@pytest.mark.skipif(not reference_available(), reason="OpenVort checkout not built here")
@pytest.mark.parametrize("n0", [1, 5, 64])
def test_reader_matches_reference_load_tangle(tmp_path, n0):
    ref_lib = C.CDLL(os.path.join(ROOT, "oracle", "_ref", "libovref.so"))
    ht = sample_tangle()
    path = str(tmp_path / "f.txt")
    gpu.write_frame(ht, path)
    ts = abi.TangleState()
    ref_lib.create_tangle.argtypes = [C.c_void_p, C.c_size_t]
    ref_lib.load_tangle.argtypes = [C.c_char_p, C.c_void_p]
    ref_lib.create_tangle(C.addressof(ts), n0)
    ref_lib.load_tangle(path.encode(), C.addressof(ts))
    back, (ne, te) = gpu.read_frame(path, n0=n0)
    assert back.n == ts.N
    assert (ne, te) == (ts.next_empty, ts.total_empty)
    n = ts.N
    conn = np.array([(ts.connections[i].forward, ts.connections[i].reverse) for i in range(n)])
    stat = np.array([(ts.status[i].status, ts.status[i].pin_wall) for i in range(n)])
    np.testing.assert_array_equal(back.conn, conn)
    np.testing.assert_array_equal(back.stat, stat)
    used = stat[:, 0] != abi.OV_EMPTY
    pos = np.array([list(ts.vnodes[i].p) for i in range(n)])
    np.testing.assert_array_equal(back.pos[used], pos[used])


def test_writer_matches_committed_reference_frame(tmp_path, golden):
    """Without the checkout: the frame the reference wrote for the wall-step
    tangle (after enforce_wall_boundaries) equals ours."""
    g = golden("wall_steps.npz")
    n = int(g["enf_N"])
    ht = W.HostTangle(g["enf_pos"].copy(), g["enf_conn"][:, 0].copy(), g["enf_conn"][:, 1].copy(), g["box_lo"],
                      g["box_hi"], n_images=0, status=g["enf_status"][:, 0].copy())
    ht.stat[:, 1] = g["enf_status"][:, 1]
    ht.vels[:], ht.tangents[:], ht.normals[:] = g["enf_vels"], g["enf_tangents"], g["enf_normals"]
    assert ht.n == n
    path = str(tmp_path / "ours.txt")
    gpu.write_frame(ht, path)
    assert open(path).read() == open(os.path.join(GOLDEN, "frame_walls.txt")).read()
