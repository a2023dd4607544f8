"""bg3_outgoing_map_noalloc: the allocation-free map build, for callers that cannot allocate
device memory when they need the map (inside a host runtime that owns all device allocations, in
a loop that must not enter the allocator).  The test owns every device
buffer (torch tensors); the entry point is called through the C-ABI twice in a row and must give
the same map as the existing path (bg3_download_maps), exactly, both times.  This file is
collected last so that a failing run has already run every other test."""
import ctypes

import numpy as np
import pytest

from braingrid_gb300 import lib as bg
from braingrid_gb300 import netgen

pytestmark = pytest.mark.gpu


def _noalloc(L):
    f = L.bg3_outgoing_map_noalloc
    vp = ctypes.c_void_p
    f.argtypes = [vp, vp, ctypes.c_int32, ctypes.c_int32, vp, vp, vp, vp, vp]
    f.restype = ctypes.c_int
    return f


def test_noalloc_map_matches_existing_path_twice():
    import torch
    spec = netgen.lif_network(40, 30, seed=5)
    net = netgen.make_gpu_network(spec, 120, epoch_duration=0.5)
    netgen.pregrow(net, spec, 3.1, weight_scale=0.1, seed=9)
    N, M = net.N, net.max_syn
    syn = net.download_synapses()
    want = net.download_maps()
    T = net.total_synapses()
    assert T > 10000
    dev = torch.device("cuda", torch.cuda.current_device())
    src = torch.from_numpy(syn["src"].astype(np.int32)).to(dev)
    counts = torch.from_numpy(syn["counts"].astype(np.uint32).view(np.int32)).to(dev)
    begin = torch.zeros(N, dtype=torch.int32, device=dev)
    count = torch.zeros(N, dtype=torch.int32, device=dev)
    omap = torch.zeros(T, dtype=torch.int32, device=dev)
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    f = _noalloc(bg.load())
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):
        begin.fill_(-1)
        count.fill_(-1)
        omap.fill_(-1)
        rc = f(src.data_ptr(), counts.data_ptr(), N, M, begin.data_ptr(), count.data_ptr(),
               omap.data_ptr(), status.data_ptr(), stream)
        assert rc == 0
        torch.cuda.synchronize()
        assert int(status.item()) == 0
        np.testing.assert_array_equal(begin.cpu().numpy().view(np.uint32),
                                      want["outgoingSynapseBegin"], err_msg="call %d" % call)
        np.testing.assert_array_equal(count.cpu().numpy().view(np.uint32),
                                      want["outgoingSynapseCount"], err_msg="call %d" % call)
        np.testing.assert_array_equal(omap.cpu().numpy().view(np.uint32),
                                      want["outgoingSynapseIndexMap"], err_msg="call %d" % call)


def test_noalloc_rejects_oversize():
    f = _noalloc(bg.load())
    rc = f(1, 1, 65537, 4, 1, 1, 1, 1, None)
    assert rc == -1  # BG3_EINVAL before touching any pointer


def _small_call(src_rows, counts, max_syn):
    """Runs the entry point on a small caller-made map (src_rows: n x max_syn int32, counts: n)
    and returns (status, begin, count, map)."""
    import torch
    dev = torch.device("cuda", torch.cuda.current_device())
    n = len(counts)
    T = max(int(np.sum(counts)), 1)
    src = torch.from_numpy(np.ascontiguousarray(src_rows, np.int32).reshape(-1)).to(dev)
    cnt = torch.from_numpy(np.asarray(counts, np.int32)).to(dev)
    begin = torch.zeros(n, dtype=torch.int32, device=dev)
    count = torch.zeros(n, dtype=torch.int32, device=dev)
    omap = torch.full((T,), -1, dtype=torch.int32, device=dev)
    status = torch.full((1,), -1, dtype=torch.int32, device=dev)
    f = _noalloc(bg.load())
    rc = f(src.data_ptr(), cnt.data_ptr(), n, max_syn, begin.data_ptr(), count.data_ptr(),
           omap.data_ptr(), status.data_ptr(), torch.cuda.current_stream().cuda_stream)
    assert rc == 0
    torch.cuda.synchronize()
    return (int(status.item()), begin.cpu().numpy(), count.cpu().numpy(), omap.cpu().numpy())


def test_noalloc_flags_source_out_of_range():
    """A source index outside [0, n) sets status bit 0; that synapse is left out of the map and
    the others are placed as usual."""
    src = np.array([[1, 7, 0, 0], [0, 2, 2, 0], [1, 0, 0, 0]], np.int32)  # 7 is out of range
    st, begin, count, omap = _small_call(src, [2, 3, 1], 4)
    assert st & 1 and not st & 2
    np.testing.assert_array_equal(count, [1, 2, 2])
    np.testing.assert_array_equal(begin, [0, 1, 3])
    np.testing.assert_array_equal(omap[:5], [4, 0, 8, 5, 6])


def test_noalloc_flags_fanout_above_limit():
    """A source with more than BG3_NOALLOC_MAX_FANOUT synapses sets status bit 1; its run holds
    all of its slot ids (unsorted), and the other sources' runs are sorted as usual."""
    n, m = 8, 1024
    src = np.zeros((n, m), np.int32)
    src[7, :] = 3                                    # row 7: source 3
    st, begin, count, omap = _small_call(src, [m] * n, m)
    assert st & 2 and not st & 1
    assert count[0] == 7 * m and count[3] == m
    np.testing.assert_array_equal(np.sort(omap[:7 * m]), np.arange(7 * m))
    np.testing.assert_array_equal(omap[begin[3]:begin[3] + m], np.arange(7 * m, 8 * m))


def test_noalloc_rejects_32bit_slot_overflow():
    f = _noalloc(bg.load())
    rc = f(1, 1, 65536, 65537, 1, 1, 1, 1, None)
    assert rc == -1  # BG3_EINVAL before touching any pointer
