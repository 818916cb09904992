"""The index build on the device (katoann_gpu_kmeans_*, katoann_gpu_covariance,
Index::build / katoann.build_partition) against numpy in float64.

The assignment runs on the tensor cores in TF32 (10 mantissa bits per
operand), so it must equal the exact argmin wherever the two nearest
centroids are further apart than that resolution; the other kernels are
checked to float/double rounding."""
import ctypes as C

import numpy as np
import pytest

import oracle
from _gpu import check, dptr, gpu

pytestmark = pytest.mark.gpu

P, U32, U64, D = C.c_void_p, C.c_uint32, C.c_uint64, C.c_double


@pytest.fixture(scope="module")
def torch():
    import torch
    assert torch.cuda.is_available()
    g = gpu()
    g.katoann_gpu_kmeans_assign.argtypes = [P, U32, U32, P, P, U32, P, P, P, P]
    g.katoann_gpu_row_norms.argtypes = [P, U32, U32, P, P]
    g.katoann_gpu_kmeans_update.argtypes = [P, U32, U32, P, U32, P, P, P, P, P]
    g.katoann_gpu_kmeanspp_scratch.restype = C.c_size_t
    g.katoann_gpu_kmeanspp_scratch.argtypes = [U32]
    g.katoann_gpu_kmeanspp.argtypes = [P, U32, U32, U32, U32, P, P, P, P, P, P]
    g.katoann_gpu_covariance.argtypes = [P, U32, U32, U32, P, P, P]
    g.katoann_gpu_gather_rows.argtypes = [P, U32, P, U32, U32, P, P]
    return torch


def _padded(torch, x, ld):
    t = torch.zeros((x.shape[0], ld), dtype=torch.float32, device="cuda")
    t[:, :x.shape[1]] = torch.from_numpy(np.ascontiguousarray(x, np.float32)).cuda()
    return t


def _assign(torch, x, c):
    ld = (x.shape[1] + 31) // 32 * 32
    xd, cd = _padded(torch, x, ld), _padded(torch, c, ld)
    cn = torch.empty(len(c), dtype=torch.float32, device="cuda")
    check(gpu().katoann_gpu_row_norms(dptr(cd), len(c), ld, dptr(cn), None))
    a = torch.empty(len(x), dtype=torch.int32, device="cuda")
    best = torch.empty(len(x), dtype=torch.float32, device="cuda")
    tmo = torch.zeros(4, dtype=torch.int32, device="cuda")
    check(gpu().katoann_gpu_kmeans_assign(dptr(xd), len(x), ld, dptr(cd), dptr(cn), len(c), dptr(a),
                                          dptr(best), dptr(tmo), None))
    torch.cuda.synchronize()
    assert int(tmo[0]) == 0
    return a.cpu().numpy().astype(np.int64), best.cpu().numpy()


@pytest.mark.parametrize("n,d,L", [(1, 64, 1), (5000, 64, 37), (3000, 100, 300), (4097, 1024, 1000),
                                   (700, 3072, 257)])
def test_assignment_is_the_nearest_centroid(torch, n, d, L):
    rng = np.random.default_rng(n + d + L)
    x = rng.standard_normal((n, d)).astype(np.float32)
    c = (rng.standard_normal((L, d)) * 0.7).astype(np.float32)
    got, best = _assign(torch, x, c)
    x64, c64 = x.astype(np.float64), c.astype(np.float64)
    part = (c64 * c64).sum(1)[None, :] - 2.0 * x64 @ c64.T  # |c|^2 - 2 x.c
    order = np.argsort(part, axis=1, kind="stable")
    want = order[:, 0]
    scale = np.linalg.norm(x64, axis=1) * np.linalg.norm(c64, axis=1).max()
    tol = 8.0 * 2.0 ** -10 * scale  # TF32 rounding of both operands, with margin
    if L > 1:
        gap = part[np.arange(n), order[:, 1]] - part[np.arange(n), want]
        clear = gap > tol
        assert np.array_equal(got[clear], want[clear])
        # a row inside the resolution goes to one of its near-ties
        near = part[np.arange(n), got] - part[np.arange(n), want]
        assert np.all(near <= tol)
    else:
        assert np.all(got == 0)
    assert np.all(np.abs(best - part[np.arange(n), got]) <= tol)


def test_update_is_the_cluster_mean(torch):
    rng = np.random.default_rng(5)
    n, d, L = 6000, 100, 50
    ld = 128
    x = rng.standard_normal((n, d)).astype(np.float32)
    a = rng.integers(0, L - 3, n).astype(np.int32)  # the last three clusters stay empty
    c0 = rng.standard_normal((L, d)).astype(np.float32)
    xd, cd = _padded(torch, x, ld), _padded(torch, c0, ld)
    ad = torch.from_numpy(a).cuda()
    sums = torch.empty((L, ld), dtype=torch.float64, device="cuda")
    cnt = torch.empty(L, dtype=torch.int32, device="cuda")
    cn = torch.empty(L, dtype=torch.float32, device="cuda")
    check(gpu().katoann_gpu_kmeans_update(dptr(xd), n, ld, dptr(ad), L, dptr(sums), dptr(cnt), dptr(cd),
                                          dptr(cn), None))
    got = cd.cpu().numpy()[:, :d]
    for c in range(L):
        m = a == c
        want = x[m].astype(np.float64).mean(0) if m.any() else c0[c]
        assert np.allclose(got[c], want, rtol=1e-6, atol=1e-7), c
    assert np.allclose(cn.cpu().numpy(), (got.astype(np.float64) ** 2).sum(1), rtol=1e-5)
    assert np.array_equal(cnt.cpu().numpy(), np.bincount(a, minlength=L))


def _kmeanspp(torch, x, L, first, u):
    n, d = x.shape
    ld = (d + 31) // 32 * 32
    xd = _padded(torch, x, ld)
    ud = torch.from_numpy(np.asarray(u, np.float64)).cuda()
    cen = torch.empty((L, ld), dtype=torch.float32, device="cuda")
    dist = torch.empty(n, dtype=torch.float32, device="cuda")
    part = torch.empty(gpu().katoann_gpu_kmeanspp_scratch(n), dtype=torch.uint8, device="cuda")
    chosen = torch.empty(L, dtype=torch.int32, device="cuda")
    check(gpu().katoann_gpu_kmeanspp(dptr(xd), n, ld, L, first, dptr(ud), dptr(cen), dptr(dist),
                                     dptr(part), dptr(chosen), None))
    torch.cuda.synchronize()
    return chosen.cpu().numpy(), cen.cpu().numpy()[:, :d], dist.cpu().numpy()


def test_kmeanspp_picks_distinct_far_rows(torch):
    rng = np.random.default_rng(9)
    n, d, L = 20000, 48, 200
    centres = rng.standard_normal((L, d)) * 4
    x = (centres[rng.integers(0, L, n)] + rng.standard_normal((n, d)) * 0.2).astype(np.float32)
    u = rng.random(L)
    chosen, cen, dist = _kmeanspp(torch, x, L, 17, u)
    assert chosen[0] == 17 and len(set(chosen.tolist())) == L
    assert np.array_equal(cen, x[chosen])
    # the same draws give the same seeds
    again, _, _ = _kmeanspp(torch, x, L, 17, u)
    assert np.array_equal(chosen, again)
    # every row's running distance is its distance to the nearest of the
    # first L - 1 centres (the last pick is not folded in)
    x64 = x.astype(np.float64)
    cc = x64[chosen[:-1]]
    near = ((x64 * x64).sum(1)[:, None] + (cc * cc).sum(1)[None, :] - 2.0 * x64 @ cc.T).min(1)
    assert np.allclose(dist, near, rtol=1e-4, atol=1e-5)
    # D^2 sampling covers the well-separated components far better than a
    # uniform draw of the same size
    comp_of = np.argmin(((x64[chosen][:, None, :] - centres[None]) ** 2).sum(-1), 1)
    assert len(set(comp_of.tolist())) >= 0.85 * L


def test_covariance_in_double(torch):
    rng = np.random.default_rng(11)
    n, d, ld = 3001, 70, 96
    x = (rng.standard_normal((n, d)) * np.linspace(0.1, 3, d) + 5.0).astype(np.float32)
    xd = _padded(torch, x, ld)
    mean = torch.empty(d, dtype=torch.float64, device="cuda")
    cov = torch.empty((d, d), dtype=torch.float64, device="cuda")
    check(gpu().katoann_gpu_covariance(dptr(xd), n, ld, d, dptr(mean), dptr(cov), None))
    x64 = x.astype(np.float64)
    want = np.cov(x64, rowvar=False, bias=True)
    assert np.allclose(mean.cpu().numpy(), x64.mean(0), rtol=1e-12)
    assert np.allclose(cov.cpu().numpy(), want, rtol=1e-9, atol=1e-12)


def test_gather_rows_pads_with_zeros(torch):
    rng = np.random.default_rng(2)
    x = rng.standard_normal((500, 45)).astype(np.float32)
    rows = np.array([499, 0, 7, 7, 250], np.int32)
    out = torch.full((5, 64), 9.0, dtype=torch.float32, device="cuda")
    xd, rd = torch.from_numpy(x).cuda(), torch.from_numpy(rows).cuda()  # alive until the copy ran
    check(gpu().katoann_gpu_gather_rows(dptr(xd), 45, dptr(rd), 5, 64, dptr(out), None))
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    assert np.array_equal(got[:, :45], x[rows]) and np.all(got[:, 45:] == 0)


def test_build_partition_and_files(torch, tmp_path):
    """katoann.build writes files the oracle and the GPU index load; the
    partition is each vector's nearest centroid (to TF32 resolution), lists
    hold ascending ids, the rotation is orthonormal and sorted by variance, and
    the device-array path gives the same partition as the host-array path."""
    import katoann
    import configs
    x, q = configs.vectors("plain", 30000, 200, dim=256)
    L = 64
    prefix = str(tmp_path / "b")
    katoann.build(x, prefix, nlist=L, train_size=20000, kmeans_iters=8, seed=7, rotation_sample=8000)
    ref = oracle.OracleIndex(prefix)
    assert (ref.dim, ref.nlist, ref.npts, ref.head_dims) == (256, L, 30000, 64)
    cen, assign, rot, head = katoann.build_partition(x, nlist=L, train_size=20000, kmeans_iters=8,
                                                     seed=7, rotation_sample=8000)
    cen_d, assign_d, rot_d, _ = katoann.build_partition(torch.from_numpy(x).cuda(), nlist=L,
                                                        train_size=20000, kmeans_iters=8, seed=7,
                                                        rotation_sample=8000)
    assert np.array_equal(cen, cen_d) and np.array_equal(assign, assign_d) and np.array_equal(rot, rot_d)
    assert head == 64
    # the files hold this partition
    stored = np.fromfile(prefix + ".centroids", np.float32).reshape(L, 256)
    assert np.array_equal(stored, cen)
    off = ref.list_offsets()
    assert np.array_equal(np.diff(off), np.bincount(assign, minlength=L))
    ids = ref.codes()["ids"]
    for c in range(L):
        li = ids[off[c]:off[c + 1]]
        assert np.all(np.diff(li.astype(np.int64)) > 0) and np.all(assign[li] == c)
    # nearest centroid to TF32 resolution
    x64, c64 = x.astype(np.float64), cen.astype(np.float64)
    part = (c64 * c64).sum(1)[None, :] - 2.0 * x64 @ c64.T
    near = part[np.arange(len(x)), assign] - part.min(1)
    assert np.all(near <= 8.0 * 2.0 ** -10 * np.linalg.norm(c64, axis=1).max())
    # the rotation: orthonormal rows, variance along them descending
    r64 = rot.astype(np.float64)
    assert np.allclose(r64 @ r64.T, np.eye(256), atol=1e-5)
    var = ((x64 - x64.mean(0)) @ r64.T).var(0)
    top = np.sort(np.linalg.eigvalsh(np.cov(x64, rowvar=False, bias=True)))[::-1]
    assert var[:8].sum() >= 0.97 * top[:8].sum() and var[0] >= var[-1]
    # and the index searches: recall against exact float search
    idx = katoann.Index()
    idx.load(prefix)
    ids_g, _ = idx.search(q, k=10, nprobe=16, survivors=64)
    q64 = q.astype(np.float64)
    d2 = (q64 * q64).sum(1)[:, None] + (x64 * x64).sum(1)[None, :] - 2.0 * q64 @ x64.T
    gt = np.argsort(d2, 1)[:, :10]
    rec = np.mean([len(set(a) & set(b)) / 10 for a, b in zip(ids_g, gt)])
    assert rec >= 0.9, rec
    rid, rd = ref.search(q, k=10, nprobe=16, survivors=64)
    assert np.array_equal(ids_g, rid)
