"""GPU search on the benchmark workloads' shapes, bit for bit against the oracle.

  small: 100,000 x 128, nlist 256, prefix 64, 1,024 queries (full size);
  plain: 1,024 dims, nlist 4,096, prefix 128, nprobe 16 and 128 (fewer rows);
  wide:  3,072 dims (the coarse product in three exact 1,024-dimension chunks
         on the tensor cores), prefix 256, survivors 32 and 64, prefix and
         full ranking (fewer rows and lists).

The oracle and the GPU index load the same arrays (tests/configs.py), so any
difference is a difference of the search."""
import ctypes as C
import os

import numpy as np
import pytest

import configs
import oracle
from _gpu import GpuIndex, check, dptr, gpu

pytestmark = pytest.mark.gpu


def _pair(kind, n, nq, nlist=None, seed=0, dim=None, rotate=True):
    import katoann
    s = configs.SHAPES[kind]
    x, q = configs.vectors(kind, n, nq, seed=seed, dim=dim)
    a = configs.index_arrays(x, nlist or s["nlist"], s["head"], seed=seed, rotate=rotate)
    idx = katoann.Index()
    idx.load_arrays(a["centroids"], a["list_sizes"], a["ids"], a["vectors"], rotation=a["rotation"],
                    head_dims=a["head_dims"], max_batch=max(nq, 1))
    oracle.set_threads(os.cpu_count() or 1)
    ref = oracle.OracleIndex(None, arrays=a)
    return idx, ref, q


def _same(idx, ref, q, **kw):
    ids, dists = idx.search(q, **kw)
    rid, rd = ref.search(q, **kw)
    bad = np.nonzero((ids != rid).any(1) | (dists != rd).any(1))[0]
    assert len(bad) == 0, (kw, len(bad), bad[:5])


@pytest.fixture(scope="module")
def small():
    return _pair("small", 100_000, 1024)


@pytest.fixture(scope="module")
def plain():
    return _pair("plain", 40_000, 256)


@pytest.fixture(scope="module")
def wide():
    return _pair("wide", 8_000, 128, nlist=256)


def test_small_workload_full_size(small):
    idx, ref, q = small
    assert (idx.dim, idx.nlist, idx.size, idx.prefix_dims) == (128, 256, 100_000, 64)
    for kw in (dict(k=10, nprobe=16, ranking="prefix", survivors=32),
               dict(k=10, nprobe=16, ranking="full", survivors=32),
               dict(k=10, nprobe=16, ranking="high", survivors=32)):
        _same(idx, ref, q, **kw)


@pytest.mark.parametrize("nprobe,survivors", [(16, 32), (128, 32), (128, 64)])
def test_plain_workload_shape(plain, nprobe, survivors):
    idx, ref, q = plain
    assert (idx.dim, idx.nlist, idx.prefix_dims) == (1024, 4096, 128)
    _same(idx, ref, q, k=10, nprobe=nprobe, ranking="prefix", survivors=survivors)


@pytest.mark.parametrize("nprobe,survivors,ranking", [(8, 32, "prefix"), (64, 64, "prefix"),
                                                      (64, 32, "full"), (16, 64, "high")])
def test_wide_workload_shape(wide, nprobe, survivors, ranking):
    idx, ref, q = wide
    assert (idx.dim, idx.prefix_dims) == (3072, 256)
    _same(idx, ref, q, k=10, nprobe=nprobe, ranking=ranking, survivors=survivors)


def _coarse_both_paths(idx, ref, queries):
    """The full query x centroid distance matrix from the tensor-core product
    and from the CUDA-core product (a view without the centred planes), each
    bit for bit against the oracle's sq16_l2."""
    import torch
    qc = ref.quantize(ref.rotate(queries))
    cen = ref.centroid_codes()
    want = oracle.sq16_l2(qc["hi"], qc["lo"], cen["hi"], cen["lo"], qc["norm"], cen["norm"],
                          ref.step_sq)
    nq = len(queries)
    qh, ql, qn = (torch.from_numpy(np.ascontiguousarray(qc[k])).cuda() for k in ("hi", "lo", "norm"))
    view = GpuIndex.from_address(idx.device_view)
    plain_view = GpuIndex()
    C.pointer(plain_view)[0] = view
    plain_view.d_chi16 = plain_view.d_clo16 = plain_view.d_cterm = None
    for v in (view, plain_view):
        dists = torch.empty((nq, ref.nlist), dtype=torch.float32, device="cuda")
        probed = torch.empty((nq, 4), dtype=torch.int32, device="cuda")
        check(gpu().katoann_gpu_coarse(C.byref(v), dptr(qh), dptr(ql), dptr(qn), nq, 4,
                                       dptr(dists), dptr(probed), None))
        got = dists.cpu().numpy()
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), bool(v.d_chi16)
        # the probes are the oracle's: the 4 nearest by (distance, list id)
        assert np.array_equal(np.sort(probed.cpu().numpy().astype(np.uint32), 1),
                              np.sort(ref.coarse(qc["hi"], qc["lo"], qc["norm"], 4), 1))


def test_coarse_product_at_3072_dims(wide):
    idx, ref, q = wide
    assert ref.dc == 3072
    _coarse_both_paths(idx, ref, q)


@pytest.mark.parametrize("dim", [1088, 2048, 4096])
def test_coarse_product_beyond_1024_dims(dim):
    """Chunk boundaries: one chunk and a 64-dimension remainder, two whole
    chunks, and the widest rows the reference takes (kMaxDim = 4096)."""
    idx, ref, q = _pair("wide", 1500, 70, nlist=200, dim=dim, rotate=False)
    assert ref.dc == dim
    _coarse_both_paths(idx, ref, q)
