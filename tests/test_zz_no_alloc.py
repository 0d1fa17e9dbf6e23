"""ov_direct_velocities_noalloc: direct-sum velocities for callers that may
not allocate GPU memory (their device memory belongs to a pool or to a host
framework that hands out buffers once), checked against the allocating
ov_direct_velocities on the same tangle.

The caller owns every buffer here: torch allocates the inputs and outputs,
and the entry point itself allocates nothing.  Two calls in a row with
different node lists must both match, which also shows that the working
array the calls share carries nothing over from one call to the next.
This file sorts last so that a run stopping at the first failure has run
every other test before it.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from openvort_gb300 import abi, gpu, workloads as W
from tests._util import node_rel_err

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


def test_noalloc_direct_sum_matches_allocating_entry_point():
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    ht = W.random_walk_tangle(8, 64, D=0.1, seed=77)
    p = W.config_params("rw")
    n = ht.n

    # reference: the allocating entry point through its context
    ctx = gpu.Context(0, params=p)
    ctx.upload(ht)
    ctx.update_tangents_normals()
    ctx.download(ht, abi.OV_F_TANGENTS | abi.OV_F_NORMALS)
    nodes_a = np.arange(0, n, 3, dtype=np.int32)
    nodes_b = np.arange(n - 1, 0, -17, dtype=np.int32)
    ref_a = ctx.direct_velocities(nodes_a, 0.0)
    ref_b = ctx.direct_velocities(nodes_b, 0.0)
    ctx.close()

    # caller-owned device buffers (SoA inputs, AoS outputs)
    dev = torch.device("cuda:0")
    pos = torch.tensor(np.ascontiguousarray(ht.pos.T), dtype=torch.float64, device=dev)
    tan = torch.tensor(np.ascontiguousarray(ht.tangents.T), dtype=torch.float64, device=dev)
    nrm = torch.tensor(np.ascontiguousarray(ht.normals.T), dtype=torch.float64, device=dev)
    conn = torch.tensor(np.ascontiguousarray(ht.conn.T), dtype=torch.int32, device=dev)
    stat = torch.tensor(np.ascontiguousarray(ht.stat.T), dtype=torch.int32, device=dev)
    st = ht.state()
    images = abi.image_table(ht.n_images)
    fn = _bind(gpu.load())
    stream = torch.cuda.current_stream(dev).cuda_stream

    def call(nodes):
        d_nodes = torch.tensor(nodes, dtype=torch.int32, device=dev)
        vels = torch.full((len(nodes), 3), float("nan"), dtype=torch.float64, device=dev)
        vs = torch.full((len(nodes), 3), float("nan"), dtype=torch.float64, device=dev)
        rc = fn(C.byref(p), C.byref(st.box), images, ht.n_images, n, pos.data_ptr(), conn.data_ptr(),
                stat.data_ptr(), tan.data_ptr(), nrm.data_ptr(), d_nodes.data_ptr(), len(nodes), 0.0,
                vels.data_ptr(), vs.data_ptr(), stream)
        assert rc == 0
        torch.cuda.synchronize(dev)
        return vels.cpu().numpy(), vs.cpu().numpy()

    got_a = call(nodes_a)
    got_b = call(nodes_b)
    for got, ref in ((got_a, ref_a), (got_b, ref_b)):
        assert np.all(np.isfinite(got[0]))
        assert node_rel_err(got[0], ref[0]) < FP64_TOL
        assert node_rel_err(got[1], ref[1]) < FP64_TOL

    # a list longer than the fixed working space is refused before any launch
    big = torch.zeros(MAX_NODES + 1, dtype=torch.int32, device=dev)
    out = torch.zeros((MAX_NODES + 1, 3), dtype=torch.float64, device=dev)
    rc = fn(C.byref(p), C.byref(st.box), images, ht.n_images, n, pos.data_ptr(), conn.data_ptr(), stat.data_ptr(),
            tan.data_ptr(), nrm.data_ptr(), big.data_ptr(), MAX_NODES + 1, 0.0, out.data_ptr(), None, stream)
    assert rc == 1   # OV_ERR_ARG
