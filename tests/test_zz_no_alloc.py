"""katoann_gpu_coarse_noalloc, the coarse step for callers that cannot
allocate device memory (a host whose own allocator owns all device memory, or
a latency-bound loop that cannot take cudaMalloc's device-wide sync): called
through the C ABI twice in a row, it must give exactly the probe lists of
katoann_gpu_coarse and the oracle's probes (integer output, so the tolerance
is zero), also for the largest batch its static scratch takes, and it must
refuse batches larger than that. This file is collected last."""
import ctypes as C

import numpy as np
import pytest

import oracle
from _gpu import check, dptr, gpu
from _util import fixture

pytestmark = pytest.mark.gpu


def _inputs(name, nq=None):
    """The fixture's index, the oracle, and nq of its queries (cycled when nq
    is larger than the fixture's set) quantized by the oracle, on the device."""
    import katoann
    import torch
    spec, z, prefix, queries = fixture(name)
    idx = katoann.Index()
    idx.load(prefix)
    ref = oracle.OracleIndex(prefix)
    if nq is not None:
        queries = queries[np.arange(nq) % len(queries)]
    q = ref.quantize(ref.rotate(queries))
    dev = {k: torch.from_numpy(np.ascontiguousarray(q[k])).cuda() for k in ("hi", "lo", "norm")}
    return idx, ref, dev, q, len(queries)


def _check_twice(idx, ref, dev, q, nq, nprobe):
    import torch
    lib = gpu()
    lib.katoann_gpu_coarse_noalloc.argtypes = [C.c_void_p] * 4 + [C.c_uint32, C.c_uint32, C.c_void_p,
                                                                   C.c_void_p]
    view = C.c_void_p(idx.device_view)
    dists = torch.empty((nq, ref.nlist), dtype=torch.float32, device="cuda")
    want = torch.empty((nq, nprobe), dtype=torch.int32, device="cuda")
    check(lib.katoann_gpu_coarse(view, dptr(dev["hi"]), dptr(dev["lo"]), dptr(dev["norm"]), nq,
                                 nprobe, dptr(dists), dptr(want), None))
    oracle_probes = np.sort(ref.coarse(q["hi"], q["lo"], q["norm"], nprobe), 1)
    for _ in range(2):
        got = torch.full((nq, nprobe), -1, dtype=torch.int32, device="cuda")
        check(lib.katoann_gpu_coarse_noalloc(view, dptr(dev["hi"]), dptr(dev["lo"]), dptr(dev["norm"]),
                                             nq, nprobe, dptr(got), None))
        torch.cuda.synchronize()
        assert torch.equal(got, want)
        assert np.array_equal(np.sort(got.cpu().numpy().astype(np.uint32), 1), oracle_probes)


@pytest.mark.parametrize("name,nprobe", [("d128", 8), ("d1024", 4)])
def test_noalloc_coarse_equals_coarse_twice(name, nprobe):
    _check_twice(*_inputs(name), nprobe)


def test_noalloc_coarse_at_its_largest_batch():
    """nq * nlist exactly the static scratch's 1,048,576 distances."""
    spec, z, prefix, queries = fixture("d128")
    nlist = spec["nlist"]
    _check_twice(*_inputs("d128", (1 << 20) // nlist), 8)


def test_noalloc_coarse_rejects_oversize_batches():
    lib = gpu()
    lib.katoann_gpu_coarse_noalloc.argtypes = [C.c_void_p] * 4 + [C.c_uint32, C.c_uint32, C.c_void_p,
                                                                   C.c_void_p]
    idx, ref, dev, q, nq = _inputs("d128")
    too_many = (1 << 20) // ref.nlist + 1
    rc = lib.katoann_gpu_coarse_noalloc(C.c_void_p(idx.device_view), dptr(dev["hi"]), dptr(dev["lo"]),
                                        dptr(dev["norm"]), too_many, 8, dptr(dev["hi"]), None)
    assert rc == -1
    assert b"static scratch" in lib.katoann_gpu_last_error()
