"""orbgpu_knn2_noalloc: the allocation-free k = 2 search.

It serves callers that cannot allocate device memory (a process whose device
memory is reserved up front by its own allocator, a real-time path that cannot
take cudaMalloc's device-wide synchronisation).  Its results must equal
orbgpu_knn2's, call after call, although every call reuses the same fixed
scratch array inside the library.  This file is collected last so that a run
stopping at the first failure has run every other test first.
"""
import ctypes as C

import numpy as np
import pytest

from tests.gpu_util import require_gpu

pytestmark = pytest.mark.gpu


def test_knn_noalloc_equals_knn2_twice():
    torch = require_gpu()
    from oracle import pyoracle
    from orb_slam2_detailed_comments_gb300 import ORBmatcher
    from orb_slam2_detailed_comments_gb300 import synthetic as syn
    from orb_slam2_detailed_comments_gb300._lib import lib, ptr
    qh = syn.random_descriptors(5000, 11)
    th = syn.clustered_descriptors(60000, 300, 0.1, 12)
    q = torch.from_numpy(qh).cuda()
    t = torch.from_numpy(th).cuda()
    ref = [a.cpu().numpy() for a in ORBmatcher().knn2(q, t)]
    # the allocating entry point it is compared with is itself the oracle's
    # result (a loop over DescriptorDistance on the host)
    pyoracle.build(ref=False)
    oref = pyoracle.Oracle().knn2(qh, th)
    for a, b, name in zip(ref, oref, ("idx1", "d1", "idx2", "d2")):
        assert np.array_equal(a, b), f"orbgpu_knn2 vs oracle: {name}"
    for call in range(2):
        outs = [torch.full((5000,), -7, dtype=torch.int32, device="cuda") for _ in range(4)]
        rc = lib().orbgpu_knn2_noalloc(ptr(q), 5000, ptr(t), 60000, *[ptr(o) for o in outs], C.c_void_p(0))
        assert rc == 0, lib().orbgpu_last_error()
        torch.cuda.synchronize()
        for a, b, name in zip(outs, ref, ("idx1", "d1", "idx2", "d2")):
            # integer results: exact equality is the tolerance
            assert np.array_equal(a.cpu().numpy(), b), f"call {call}: {name}"
    # sizes beyond the fixed scratch are rejected, not truncated
    rc = lib().orbgpu_knn2_noalloc(ptr(q), (1 << 20) + 1, ptr(t), 60000, *[ptr(o) for o in outs], C.c_void_p(0))
    assert rc == 1
