"""katoann_gpu_coarse_noalloc, the coarse step for callers that cannot
allocate device memory (a host whose own allocator owns all device memory, or
a latency-bound loop that cannot take cudaMalloc's device-wide sync): called
through the C ABI twice in a row, it must give exactly the probe lists of
katoann_gpu_coarse (integer output, so the tolerance is zero), and it must
refuse batches larger than its static scratch. This file is collected last."""
import ctypes as C

import numpy as np
import pytest

import oracle
from _gpu import check, dptr, gpu
from _util import fixture

pytestmark = pytest.mark.gpu


def _inputs(name):
    import katoann
    import torch
    spec, z, prefix, queries = fixture(name)
    idx = katoann.Index()
    idx.load(prefix)
    ref = oracle.OracleIndex(prefix)
    q = ref.quantize(ref.rotate(queries))
    dev = {k: torch.from_numpy(np.ascontiguousarray(q[k])).cuda() for k in ("hi", "lo", "norm")}
    return idx, ref, dev, len(queries)


@pytest.mark.parametrize("name,nprobe", [("d128", 8), ("d1024", 4)])
def test_noalloc_coarse_equals_coarse_twice(name, nprobe):
    import torch
    lib = gpu()
    lib.katoann_gpu_coarse_noalloc.argtypes = [C.c_void_p] * 4 + [C.c_uint32, C.c_uint32, C.c_void_p,
                                                                   C.c_void_p]
    idx, ref, dev, nq = _inputs(name)
    view = C.c_void_p(idx.device_view)
    dists = torch.empty((nq, ref.nlist), dtype=torch.float32, device="cuda")
    want = torch.empty((nq, nprobe), dtype=torch.int32, device="cuda")
    check(lib.katoann_gpu_coarse(view, dptr(dev["hi"]), dptr(dev["lo"]), dptr(dev["norm"]), nq,
                                 nprobe, dptr(dists), dptr(want), None))
    for _ in range(2):
        got = torch.full((nq, nprobe), -1, dtype=torch.int32, device="cuda")
        check(lib.katoann_gpu_coarse_noalloc(view, dptr(dev["hi"]), dptr(dev["lo"]), dptr(dev["norm"]),
                                             nq, nprobe, dptr(got), None))
        torch.cuda.synchronize()
        assert torch.equal(got, want)


def test_noalloc_coarse_rejects_oversize_batches():
    lib = gpu()
    lib.katoann_gpu_coarse_noalloc.argtypes = [C.c_void_p] * 4 + [C.c_uint32, C.c_uint32, C.c_void_p,
                                                                   C.c_void_p]
    idx, ref, dev, nq = _inputs("d128")
    too_many = (1 << 20) // ref.nlist + 1
    rc = lib.katoann_gpu_coarse_noalloc(C.c_void_p(idx.device_view), dptr(dev["hi"]), dptr(dev["lo"]),
                                        dptr(dev["norm"]), too_many, 8, dptr(dev["hi"]), None)
    assert rc == -1
    assert b"static scratch" in lib.katoann_gpu_last_error()
