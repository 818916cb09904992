"""Kernel-level checks through the C ABI of libkatoann_gpu.so: the exact
SQ16 distance kernels on the reference's own test grid
(tests/test_kernels.cpp:151-154), the float rotation in the reference's
arithmetic, the 16-bit coding of the lists and centroids, and the coarse
probes, each against the oracle."""
import ctypes as C

import numpy as np
import pytest

import oracle
from _gpu import check, dptr, gpu, to_host, view_of
from _util import FIXTURES, fixture

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    import torch
    assert torch.cuda.is_available()
    return torch


def _draw(rng, shape):
    c = rng.integers(0, 4, shape)
    return np.where(c == 0, 0, np.where(c == 1, 255, rng.integers(0, 256, shape))).astype(np.uint8)


def test_sq16_kernels_on_reference_grid(torch):
    rng = np.random.default_rng(7)
    step_sq = 1.0 / (65535.0 * 65535.0)
    keep = []

    def dev(a):  # device copy kept alive until the kernel has run
        t = torch.from_numpy(np.ascontiguousarray(a)).cuda()
        keep.append(t)
        return t

    for dc in (64, 128, 1024, 3072):
        for m in (1, 5, 16, 70):
            for n in (1, 15, 16, 17, 70, 256):
                qh, ql, xh, xl = _draw(rng, (m, dc)), _draw(rng, (m, dc)), _draw(rng, (n, dc)), _draw(rng, (n, dc))
                code = lambda h, l: h.astype(np.int64) * 256 + l
                qn = (code(qh, ql) ** 2).sum(1)
                xn = (code(xh, xl) ** 2).sum(1)
                out = torch.empty((m, n), dtype=torch.float32, device="cuda")
                check(gpu().katoann_gpu_sq16_l2(dptr(dev(qh)), dptr(dev(ql)), dptr(dev(xh)), dptr(dev(xl)),
                                               dptr(dev(qn)), dptr(dev(xn)), step_sq, m, n, dc, dptr(out), None))
                want = oracle.sq16_l2(qh, ql, xh, xl, qn, xn, step_sq)
                assert np.array_equal(out.cpu().numpy(), want), ("full", dc, m, n)
                # high bytes, and the leading pd dims of the dc-wide rows in place
                pds = [dc] + [pd for pd in (64, 128, 256, 512, 1024) if pd < dc]
                for pd in pds:
                    qp = np.ascontiguousarray(qh[:, :pd])
                    qpn = (qp.astype(np.int64) ** 2).sum(1)
                    xpn = (xh[:, :pd].astype(np.int64) ** 2).sum(1)
                    out = torch.empty((m, n), dtype=torch.float32, device="cuda")
                    check(gpu().katoann_gpu_sq16_high_l2(dptr(dev(qp)), dptr(dev(xh)), dptr(dev(qpn)),
                                                        dptr(dev(xpn)), step_sq, m, n, pd, dc, dptr(out), None))
                    want = oracle.sq16_high_l2(qp, xh, qpn, xpn, step_sq, dims=pd)
                    assert np.array_equal(out.cpu().numpy(), want), ("high", dc, m, n, pd)
                keep.clear()


def test_dist_values_on_device(torch):
    """The device's conversion (its single-precision path and the integer path
    it falls back to) against float(double(l2) * step_sq), on random values and
    on values a few units from float rounding midpoints."""
    from test_dist_value_single import SCALES, near_midpoints
    rng = np.random.default_rng(3)
    for step_sq in SCALES + [1.0 / 65535.0 ** 2 * 3.7]:
        top = (1 << 46) - 1
        l2 = np.concatenate([rng.integers(0, 1 << 45, 1 << 20, dtype=np.int64),
                             np.exp2(rng.uniform(0, 46, 1 << 18)).astype(np.int64),
                             near_midpoints(rng, step_sq, 1 << 16, max(step_sq * 64, 1e-30),
                                            min(top * step_sq, 3e38))])
        l2 = np.clip(l2, 0, top)
        l2[:64] = np.arange(64)
        d = torch.from_numpy(l2).cuda()
        out = torch.empty(len(l2), dtype=torch.float32, device="cuda")
        check(gpu().katoann_gpu_dist_values(dptr(d), len(l2), step_sq, dptr(out), None))
        assert np.array_equal(out.cpu().numpy(), (l2.astype(np.float64) * step_sq).astype(np.float32))


@pytest.mark.parametrize("d", [4, 5, 7, 9, 15, 16, 17, 19, 31, 33, 47, 63, 64, 65, 100, 102, 127,
                               128, 129, 255, 1023, 1024])
def test_rotation_matches_reference_arithmetic(torch, d):
    rng = np.random.default_rng(d)
    for nrows in (1, 3, 33, 100):
        x = (rng.standard_normal((nrows, d)) * rng.uniform(0.01, 3.0, d)).astype(np.float32)
        r = rng.standard_normal((d, d)).astype(np.float32) / np.float32(np.sqrt(d))
        out = torch.empty((nrows, d), dtype=torch.float32, device="cuda")
        xd, rd = torch.from_numpy(x).cuda(), torch.from_numpy(r).cuda()
        check(gpu().katoann_gpu_rotate_rows(dptr(xd), nrows, d, dptr(rd), dptr(out), None))
        assert np.array_equal(out.cpu().numpy(), oracle.rotate_with(x, r)), nrows


def _lround_clamped(x, lo, inv_step):
    """The reference's code of a value: (double(x) - lo) * inv_step in double,
    rounded half away from zero, clamped to [0, 65535]."""
    t = (x.astype(np.float64) - np.float64(lo)) * np.float64(inv_step)
    f = np.floor(t)
    return np.clip(f + (t - f >= 0.5), 0, 65535).astype(np.int64)


@pytest.mark.parametrize("lo,inv_step", [(-0.3712, 65535.0 / 0.8093),  # a generic index scale
                                         (0.0, 4096.0),                # exact halves: the double path
                                         (-1.0, 32767.5)])
def test_quantization_at_rounding_ties(torch, lo, inv_step):
    """The single-precision quantizer against the reference's double arithmetic
    at and around half-integers (the float neighbours of each tie), at integers,
    at the clamps and on random values."""
    lo = float(np.float32(lo))
    rng = np.random.default_rng(11)
    k = np.concatenate([np.arange(0, 40), rng.integers(0, 65535, 3000), np.arange(65495, 65536)])
    ties = (np.float64(lo) + (k + 0.5) / inv_step).astype(np.float32)
    near = [ties]
    for step in (1, 2, 3):
        near.append(np.nextafter(near[-1], np.float32(np.inf)))
    down = [ties]
    for step in (1, 2, 3):
        down.append(np.nextafter(down[-1], np.float32(-np.inf)))
    ints = (np.float64(lo) + k / inv_step).astype(np.float32)
    span = 65535.0 / inv_step
    rand = rng.uniform(lo - 0.2 * span, lo + 1.2 * span, 20000).astype(np.float32)
    edge = np.array([lo, np.nextafter(np.float32(lo), np.float32(-1)), lo + span, -1e30, 1e30, 0.0],
                    np.float32)
    x = np.concatenate(near + down[1:] + [ints, rand, edge])
    d = 64
    x = np.concatenate([x, np.zeros((-len(x)) % d, np.float32)]).reshape(-1, d)
    n = x.shape[0]
    xd = torch.from_numpy(x).cuda()
    hi = torch.zeros((n, d), dtype=torch.uint8, device="cuda")
    lp = torch.zeros((n, d), dtype=torch.uint8, device="cuda")
    nrm = torch.zeros(n, dtype=torch.int64, device="cuda")
    hn = torch.zeros(n, dtype=torch.int64, device="cuda")
    check(gpu().katoann_gpu_quantize_rows(dptr(xd), n, d, d, lo, inv_step, 0, dptr(hi), dptr(lp),
                                          dptr(nrm), dptr(hn), None, None))
    got = hi.cpu().numpy().astype(np.int64) * 256 + lp.cpu().numpy()
    want = _lround_clamped(x, lo, inv_step)
    bad = np.argwhere(got != want)
    assert len(bad) == 0, (len(bad), [(x[i, j], got[i, j], want[i, j]) for i, j in bad[:5]])
    assert np.array_equal(nrm.cpu().numpy(), (want * want).sum(1))
    assert np.array_equal(hn.cpu().numpy(), ((want >> 8) ** 2).sum(1))


@pytest.mark.parametrize("d", [64, 1024])
def test_rotation_into_an_unaligned_buffer(torch, d):
    """Rows of 16-dimension multiples are stored four outputs at a time when
    the destination is 16-byte aligned; an output pointer one float off takes
    the scalar stores and gives the same bits."""
    rng = np.random.default_rng(d + 1)
    x = rng.standard_normal((40, d)).astype(np.float32)
    r = rng.standard_normal((d, d)).astype(np.float32) / np.float32(np.sqrt(d))
    xd, rd = torch.from_numpy(x).cuda(), torch.from_numpy(r).cuda()
    buf = torch.zeros(40 * d + 1, dtype=torch.float32, device="cuda")
    check(gpu().katoann_gpu_rotate_rows(dptr(xd), 40, d, dptr(rd), buf.data_ptr() + 4, None))
    got = buf[1:].cpu().numpy().reshape(40, d)
    assert np.array_equal(got, oracle.rotate_with(x, r)) and buf[0].item() == 0.0


def test_rotation_kmajor_layout(torch):
    """katoann_gpu_rotation_kmajor: entry [k][j] = rot[j][k] for k < d & ~15,
    j < d & ~3, rows padded with zeros to a multiple of 32 (both the 16-byte
    and the 4-byte transpose)."""
    g = gpu()
    g.katoann_gpu_rotation_kmajor_bytes.restype = C.c_size_t
    g.katoann_gpu_rotation_kmajor_bytes.argtypes = [C.c_uint32]
    g.katoann_gpu_rotation_kmajor.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p]
    rng = np.random.default_rng(7)
    for d in (4, 15, 16, 17, 33, 64, 100, 102, 1024):
        r = rng.standard_normal((d, d)).astype(np.float32)
        d4, d16 = d & ~3, d & ~15
        ldr = (d4 + 31) // 32 * 32
        nb = g.katoann_gpu_rotation_kmajor_bytes(d)
        assert nb == ldr * d16 * 4, d
        if nb == 0:
            continue
        rd = torch.from_numpy(r).cuda()
        out = torch.full((nb // 4,), float("nan"), dtype=torch.float32, device="cuda")
        check(g.katoann_gpu_rotation_kmajor(dptr(rd), d, dptr(out), None))
        want = np.zeros((d16, ldr), np.float32)
        want[:, :d4] = r[:d4, :d16].T
        assert np.array_equal(out.cpu().numpy().reshape(d16, ldr), want), d


@pytest.mark.parametrize("name", ["d1024", "d100", "d102", "pca"])
def test_search_with_and_without_kmajor_rotation(torch, name):
    """The host library gives the kernels the rotation's k-major copy; a view
    without it (NULL) transposes per search. Both give the same bits."""
    import katoann
    spec, z, prefix, queries = fixture(name)
    idx = katoann.Index()
    idx.load(prefix)
    v = view_of(idx)
    assert v.rotated and v.d_rotation_t
    bare = type(v).from_buffer_copy(v)
    bare.d_rotation_t = None
    nq, k, S = len(queries), 10, 32
    p = min(8, v.nlist)
    q = torch.from_numpy(np.ascontiguousarray(queries, np.float32)).cuda()
    got = []
    for view in (v, bare):
        ws_bytes = gpu().katoann_gpu_search_workspace(C.addressof(view), nq, k, p, 1, S)
        ws = torch.empty(ws_bytes, dtype=torch.uint8, device="cuda")
        ids = torch.empty((nq, k), dtype=torch.int32, device="cuda")
        dists = torch.empty((nq, k), dtype=torch.float32, device="cuda")
        check(gpu().katoann_gpu_search(C.addressof(view), dptr(q), nq, k, p, 1, S, nq, dptr(ws),
                                       ws_bytes, dptr(ids), dptr(dists), None))
        torch.cuda.synchronize()
        got.append((ids.cpu().numpy(), dists.cpu().numpy()))
    assert np.array_equal(got[0][0], got[1][0]) and np.array_equal(got[0][1], got[1][1])


@pytest.mark.parametrize("name", FIXTURES)
def test_load_codes_match_oracle(name):
    import katoann
    spec, z, prefix, queries = fixture(name)
    idx = katoann.Index()
    idx.load(prefix)
    v = view_of(idx)
    ref = oracle.OracleIndex(prefix)
    c = ref.codes()
    n, dc = ref.npts, ref.dc
    assert (v.npts, v.dc, v.head_dims) == (n, dc, ref.head_dims)
    assert (float(v.lo), float(v.inv_step), float(v.step_sq)) == (np.float32(ref.lo), ref.inv_step, ref.step_sq)
    assert np.array_equal(to_host(v.d_hi, n * dc, np.uint8).reshape(n, dc), c["hi"])
    assert np.array_equal(to_host(v.d_lo, n * dc, np.uint8).reshape(n, dc), c["lo"])
    assert np.array_equal(to_host(v.d_norm, n * 8, np.int64), c["norm"])
    assert np.array_equal(to_host(v.d_hinorm, n * 8, np.int64), c["hinorm"])
    if ref.head_dims:
        assert np.array_equal(to_host(v.d_headnorm, n * 8, np.int64), c["headnorm"])
    assert np.array_equal(to_host(v.d_ids, n * 4, np.uint32), c["ids"])
    cc = ref.centroid_codes()
    L = ref.nlist
    assert np.array_equal(to_host(v.d_chi, L * dc, np.uint8).reshape(L, dc), cc["hi"])
    assert np.array_equal(to_host(v.d_clo, L * dc, np.uint8).reshape(L, dc), cc["lo"])
    assert np.array_equal(to_host(v.d_cnorm, L * 8, np.int64), cc["norm"])


@pytest.mark.parametrize("name", ["d128", "d1024", "pca", "d100"])
def test_coarse_probes_match_reference(torch, name):
    import katoann
    spec, z, prefix, queries = fixture(name)
    idx = katoann.Index()
    idx.load(prefix)
    ref = oracle.OracleIndex(prefix)
    q = ref.quantize(ref.rotate(queries))
    nprobe = int(z["probed"].shape[1])
    nq = len(queries)
    qh, ql, qn = (torch.from_numpy(np.ascontiguousarray(q[k])).cuda() for k in ("hi", "lo", "norm"))
    dists = torch.empty((nq, ref.nlist), dtype=torch.float32, device="cuda")
    probed = torch.empty((nq, nprobe), dtype=torch.int32, device="cuda")
    check(gpu().katoann_gpu_coarse(C.c_void_p(idx.device_view), dptr(qh), dptr(ql), dptr(qn), nq,
                                   nprobe, dptr(dists), dptr(probed), None))
    got = probed.cpu().numpy().astype(np.uint32)
    assert np.array_equal(np.sort(got, 1), np.sort(z["probed"], 1))
    # ascending by (distance, list)
    d = dists.cpu().numpy()
    rows = np.arange(nq)[:, None]
    dd = d[rows, got]
    assert np.all((dd[:, 1:] > dd[:, :-1]) | ((dd[:, 1:] == dd[:, :-1]) & (got[:, 1:] > got[:, :-1])))


@pytest.mark.parametrize("name", FIXTURES)
def test_coarse_distances_match_oracle_on_both_paths(torch, name):
    """The full query x centroid distance matrix, bit for bit, from the
    tensor-core product and from the CUDA-core product (view without the
    centred planes)."""
    import ctypes as C
    import katoann
    from _gpu import GpuIndex
    spec, z, prefix, queries = fixture(name)
    idx = katoann.Index()
    idx.load(prefix)
    ref = oracle.OracleIndex(prefix)
    q = ref.quantize(ref.rotate(queries))
    cen = ref.centroid_codes()
    want = oracle.sq16_l2(q["hi"], q["lo"], cen["hi"], cen["lo"], q["norm"], cen["norm"], ref.step_sq)
    nq = len(queries)
    qh, ql, qn = (torch.from_numpy(np.ascontiguousarray(q[k])).cuda() for k in ("hi", "lo", "norm"))
    view = GpuIndex.from_address(idx.device_view)
    plain = GpuIndex()
    C.pointer(plain)[0] = view
    plain.d_chi16 = plain.d_clo16 = plain.d_cterm = None
    for v in (view, plain):
        dists = torch.empty((nq, ref.nlist), dtype=torch.float32, device="cuda")
        probed = torch.empty((nq, 1), dtype=torch.int32, device="cuda")
        check(gpu().katoann_gpu_coarse(C.byref(v), dptr(qh), dptr(ql), dptr(qn), nq, 1, dptr(dists),
                                       dptr(probed), None))
        got = dists.cpu().numpy()
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), v.d_chi16
