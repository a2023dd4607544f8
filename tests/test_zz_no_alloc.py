"""bg3_outgoing_map_noalloc: the allocation-free map build, for callers that cannot allocate
device memory when they need the map (under stream capture, inside a host runtime that owns all
device allocations, in a loop that must not enter the allocator).  The test owns every device
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
