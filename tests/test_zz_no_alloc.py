"""ov_direct_velocities_noalloc: direct-sum velocities for callers that may
not allocate GPU memory (their device memory belongs to a pool or to a host
framework that hands out buffers once), checked against the allocating
ov_direct_velocities on the same tangle.

The caller owns every buffer here: torch allocates the inputs and outputs,
and the entry point itself allocates nothing (the device's free memory is
the same before and after a call).  The reference's own direct-sum golden
vectors are matched with its tangents and normals handed in.  Two calls in a
row with different node lists must both match, which also shows that the
working array the calls share carries nothing over from one call to the next.  An EMPTY slot in the
list gives zeros, as the allocating call gives.  A wall geometry with mirror
images runs with no superfluid-velocity output (d_vs NULL).  This file sorts
last so that a run stopping at the first failure has run every other test
before it.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from openvort_gb300 import abi, gpu, workloads as W
from tests._util import host_from_arrays, node_rel_err

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10          # the FP64 parity tolerance of the other GPU tests
MAX_NODES = 4096          # OV_NOALLOC_MAX_NODES in include/openvort_gpu.h


def _bind(lib):
    fn = lib.ov_direct_velocities_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.POINTER(abi.Params), C.POINTER(abi.DomainBox), C.POINTER(abi.ImageTangle), C.c_int,
                   C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                   C.c_double, C.c_void_p, C.c_void_p, C.c_void_p]
    return fn


def _with_empty_slot(ht: W.HostTangle, **kw) -> W.HostTangle:
    """The same tangle with one EMPTY slot appended (pool slot n)."""
    n = ht.n
    pos = np.vstack([ht.pos, np.zeros((1, 3))])
    fwd = np.append(ht.conn[:, 0], -1)
    rev = np.append(ht.conn[:, 1], -1)
    status = np.append(ht.stat[:, 0], abi.OV_EMPTY)
    out = W.HostTangle(pos, fwd, rev, ht.box_lo, ht.box_hi, status=status, **kw)
    assert out.n == n + 1
    return out


class _Caller:
    """The caller's side: its own device buffers, filled once, and the call."""

    def __init__(self, torch, ht, p):
        self.torch, self.ht, self.p = torch, ht, p
        dev = self.dev = torch.device("cuda:0")
        f64, i32 = torch.float64, torch.int32
        self.pos = torch.tensor(np.ascontiguousarray(ht.pos.T), dtype=f64, device=dev)
        self.tan = torch.tensor(np.ascontiguousarray(ht.tangents.T), dtype=f64, device=dev)
        self.nrm = torch.tensor(np.ascontiguousarray(ht.normals.T), dtype=f64, device=dev)
        self.conn = torch.tensor(np.ascontiguousarray(ht.conn.T), dtype=i32, device=dev)
        self.stat = torch.tensor(np.ascontiguousarray(ht.stat.T), dtype=i32, device=dev)
        self.st = ht.state()
        self.fn = _bind(gpu.load())
        self.stream = torch.cuda.current_stream(dev).cuda_stream

    def buffers(self, nodes, with_vs=True):
        t = self.torch
        d_nodes = t.tensor(nodes, dtype=t.int32, device=self.dev)
        vels = t.full((len(nodes), 3), float("nan"), dtype=t.float64, device=self.dev)
        vs = t.full((len(nodes), 3), float("nan"), dtype=t.float64, device=self.dev) if with_vs else None
        return d_nodes, vels, vs

    def launch(self, d_nodes, n, vels, vs):
        ht = self.ht
        return self.fn(C.byref(self.p), C.byref(self.st.box), ht._images, ht.n_images, ht.n, self.pos.data_ptr(),
                       self.conn.data_ptr(), self.stat.data_ptr(), self.tan.data_ptr(), self.nrm.data_ptr(),
                       d_nodes.data_ptr(), n, 0.0, vels.data_ptr(), None if vs is None else vs.data_ptr(),
                       self.stream)

    def call(self, nodes, with_vs=True):
        d_nodes, vels, vs = self.buffers(nodes, with_vs)
        assert self.launch(d_nodes, len(nodes), vels, vs) == 0
        self.torch.cuda.synchronize(self.dev)
        return vels.cpu().numpy(), None if vs is None else vs.cpu().numpy()


def _reference(ht, p, node_lists):
    """The allocating entry point through a context (tangents and normals first)."""
    ctx = gpu.Context(0, params=p)
    ctx.upload(ht)
    ctx.update_tangents_normals()
    ctx.download(ht, abi.OV_F_TANGENTS | abi.OV_F_NORMALS)
    refs = [ctx.direct_velocities(nodes, 0.0) for nodes in node_lists]
    ctx.close()
    return refs


def test_noalloc_direct_sum_matches_allocating_entry_point():
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    ht = _with_empty_slot(W.random_walk_tangle(8, 64, D=0.1, seed=77))
    p = W.config_params("rw")
    n = ht.n
    empty = n - 1
    nodes_a = np.append(np.arange(0, n - 1, 3, dtype=np.int32), empty).astype(np.int32)
    nodes_b = np.arange(n - 2, 0, -17, dtype=np.int32)
    ref_a, ref_b = _reference(ht, p, [nodes_a, nodes_b])
    assert np.all(ref_a[0][-1] == 0) and np.all(ref_a[1][-1] == 0)   # the allocating call on the EMPTY slot

    c = _Caller(torch, ht, p)
    got_a = c.call(nodes_a)
    got_b = c.call(nodes_b)
    for got, ref in ((got_a, ref_a), (got_b, ref_b)):
        assert np.all(np.isfinite(got[0])) and np.all(np.isfinite(got[1]))
        live = np.linalg.norm(ref[0], axis=1) > 0
        assert node_rel_err(got[0][live], ref[0][live]) < FP64_TOL
        assert node_rel_err(got[1][live], ref[1][live]) < FP64_TOL
        assert np.array_equal(got[0][~live], ref[0][~live]) and np.array_equal(got[1][~live], ref[1][~live])
    assert np.all(got_a[0][-1] == 0) and np.all(got_a[1][-1] == 0)

    # no device allocation: free memory is unchanged across a call whose
    # buffers already exist (the working array was loaded with the library)
    d_nodes, vels, vs = c.buffers(nodes_b)
    torch.cuda.synchronize(c.dev)
    free0, _ = torch.cuda.mem_get_info(c.dev)
    assert c.launch(d_nodes, len(nodes_b), vels, vs) == 0
    torch.cuda.synchronize(c.dev)
    free1, _ = torch.cuda.mem_get_info(c.dev)
    assert free1 == free0
    assert node_rel_err(vels.cpu().numpy(), ref_b[0]) < FP64_TOL

    # a list longer than the fixed working space is refused before any launch
    big = torch.zeros(MAX_NODES + 1, dtype=torch.int32, device=c.dev)
    out = torch.zeros((MAX_NODES + 1, 3), dtype=torch.float64, device=c.dev)
    assert c.launch(big, MAX_NODES + 1, out, None) == 1   # OV_ERR_ARG


def test_noalloc_matches_reference_golden(golden):
    """OpenVort's own direct-sum velocities (147 nodes of the 1,024-node
    random-walk golden, periodic_26), with the reference's tangents and
    normals handed in as the caller's arrays."""
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    g = golden("rw16x64.npz")
    ht = host_from_arrays(g)
    ht.tangents[:] = g["tangents"]
    ht.normals[:] = g["normals"]
    c = _Caller(torch, ht, W.config_params("rw"))
    nodes = np.asarray(g["direct_nodes"], dtype=np.int32)
    v, s = c.call(nodes)
    assert node_rel_err(v, g["direct_vels"]) < FP64_TOL
    assert node_rel_err(s, g["direct_vs"]) < FP64_TOL


def test_noalloc_mirror_images_without_vs_output():
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    base = W.random_walk_tangle(8, 64, D=0.1, seed=91)
    ht = W.HostTangle(base.pos.copy(), base.conn[:, 0].copy(), base.conn[:, 1].copy(), base.box_lo, base.box_hi,
                      image_set="wall_2_4")
    p = W.config_params("rw")
    nodes_a = np.arange(1, ht.n, 5, dtype=np.int32)
    nodes_b = np.arange(0, ht.n, 7, dtype=np.int32)
    ref_a, ref_b = _reference(ht, p, [nodes_a, nodes_b])
    c = _Caller(torch, ht, p)
    for nodes, ref in ((nodes_a, ref_a), (nodes_b, ref_b)):
        v, s = c.call(nodes, with_vs=False)
        assert s is None
        assert np.all(np.isfinite(v))
        assert node_rel_err(v, ref[0]) < FP64_TOL
