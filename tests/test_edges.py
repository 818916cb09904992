"""Edge cases of the additions: empty batches, budgets beyond the candidates,
models deeper than the index, bad server requests and graph searches with a
timer - each gives the documented result or error, never a wrong answer."""
import numpy as np
import pytest

import oracle
import synth

pytestmark = pytest.mark.gpu

SPEC = dict(seed=81, n=3000, dim=64, ncomp=6, nlist=24, nq=50, rotation="random")


@pytest.fixture(scope="module")
def small(tmp_path_factory):
    import katoann
    prefix = str(tmp_path_factory.mktemp("edge") / "x")
    queries, _ = synth.materialize(SPEC, prefix)
    idx = katoann.Index()
    idx.load(prefix)
    return prefix, queries, idx


def test_empty_batches(small):
    import katoann
    _, queries, idx = small
    ids, dists, used = idx.search(queries[:0], k=10, nprobe=4,
                                  nprobe_per_query=np.zeros(0, np.uint32), return_nprobe=True)
    assert ids.shape == (0, 10) and used.shape == (0,)
    z = katoann.ProbeModel.features(idx, queries[:0], 16)
    assert z.shape == (0, 64)


def test_budgets_and_k_beyond_the_candidates(small):
    """k larger than what a one-list budget can supply: padded like the
    reference (UINT32_MAX / FLT_MAX), equal to the oracle at that nprobe."""
    prefix, queries, idx = small
    ref = oracle.OracleIndex(prefix)
    sizes = idx.list_sizes()
    k = int(sizes.max()) + 5
    budget = np.ones(len(queries), np.uint32)
    ids, dists, used = idx.search(queries, k=k, nprobe=24, survivors=k, ranking="prefix",
                                  nprobe_per_query=budget, return_nprobe=True)
    assert (used == 1).all()
    rid, rd = ref.search(queries, k=k, nprobe=1, survivors=k, ranking="prefix")
    assert np.array_equal(ids, rid) and np.array_equal(dists, rd)
    assert (ids[:, -1] == 0xFFFFFFFF).all() and (dists[:, -1] == np.float32(3.402823466e+38)).all()


def test_model_deeper_than_the_index_is_refused(small, tmp_path):
    import katoann
    _, queries, idx = small
    rng = np.random.default_rng(0)
    deep = katoann.ProbeModel.fit(rng.normal(size=(64, 64)).astype(np.float32),
                                  rng.integers(0, 3, 64).astype(np.uint8), ladder=(1, 2, 4),
                                  depth=64, epochs=1, batch=32)
    with pytest.raises(ValueError, match="depth exceeds nlist"):
        idx.search(queries, nprobe=8, budget=deep)
    with pytest.raises(ValueError, match="depth"):
        katoann.ProbeModel.features(idx, queries, 64)


def test_server_refuses_bad_requests(small):
    import katoann
    _, queries, idx = small
    server = katoann.Server(idx, max_batch=16, max_in_flight=1, max_k=20, nprobe=4)
    with pytest.raises(ValueError, match="k must be"):
        server.submit(queries[0], k=21)
    with pytest.raises(ValueError, match="dim"):
        server.submit(queries[0][:10], k=10)
    rid = server.submit(queries[0], k=20)
    ids, dists, nprobe, ms = server.wait(rid)
    want = idx.search(queries[:1], k=20, nprobe=4)
    assert np.array_equal(ids, want[0][0]) and np.array_equal(dists, want[1][0]) and nprobe == 4
    with pytest.raises(ValueError, match="max_in_flight"):
        katoann.Server(idx, max_in_flight=0)
    with pytest.raises(ValueError, match="nprobe"):
        katoann.Server(idx, nprobe=25)


def test_graph_search_refuses_a_timer(small):
    torch = pytest.importorskip("torch")
    import katoann
    _, queries, idx = small
    q = torch.from_numpy(queries).cuda()
    ids = torch.empty((len(queries), 10), dtype=torch.int32, device="cuda")
    dists = torch.empty((len(queries), 10), dtype=torch.float32, device="cuda")
    timer = katoann.PhaseTimer(4)
    st = torch.cuda.Stream()
    with pytest.raises(ValueError, match="phase events"):
        idx.search_device(q, ids, dists, nprobe=4, stream=st.cuda_stream, timer=timer, graph=True)


def test_phase_timer_brackets_the_top_kernels(small):
    """Two timed searches: every phase and each of the three bracketed kernels
    is counted once per pass, and a kernel takes no longer than its phase."""
    torch = pytest.importorskip("torch")
    import katoann
    _, queries, idx = small
    q = torch.from_numpy(queries).cuda()
    ids = torch.empty((len(queries), 10), dtype=torch.int32, device="cuda")
    dists = torch.empty((len(queries), 10), dtype=torch.float32, device="cuda")
    timer = katoann.PhaseTimer(4)
    st = torch.cuda.Stream()
    for _ in range(2):
        idx.search_device(q, ids, dists, nprobe=4, survivors=32, stream=st.cuda_stream, timer=timer)
    phases, passes = timer.read()
    kern = timer.kernels()
    assert passes == 2 and set(kern) == set(katoann.TIMED_KERNELS)
    for name, phase in (("rotation", "rotate+quantize"), ("coarse_tc_kernel", "coarse product"),
                        ("rank_tc_kernel", "ranking pass")):
        ms, n = kern[name]
        assert n == 2 and 0 < ms <= phases[phase] + 1e-3, (name, kern, phases)
    # a read with no passes since clears the kernel sums too
    assert timer.read()[1] == 0 and all(n == 0 for _, n in timer.kernels().values())


def test_host_search_replayed_as_a_graph(small):
    """Index.search with graph=True (each pass's kernels a captured graph of
    the index's own buffers, the copies outside it) gives the plain search's
    results and the oracle's: repeated calls, another k, a batch split into
    passes of 16 queries, and per-query budgets."""
    import katoann
    prefix, queries, idx = small
    ref = oracle.OracleIndex(prefix)
    for k, nprobe in ((10, 4), (5, 6), (10, 4)):
        got = idx.search(queries, k=k, nprobe=nprobe, survivors=32, graph=True)
        plain = idx.search(queries, k=k, nprobe=nprobe, survivors=32)
        want = ref.search(queries, k=k, nprobe=nprobe, survivors=32)
        for a, b, c in zip(got, plain, want):
            assert np.array_equal(a, b) and np.array_equal(a, c), (k, nprobe)
    passes = katoann.Index()
    passes.load(prefix, max_batch=16)
    for _ in range(2):
        ids, dists = passes.search(queries, k=10, nprobe=4, survivors=32, graph=True)
        want = ref.search(queries, k=10, nprobe=4, survivors=32)
        assert np.array_equal(ids, want[0]) and np.array_equal(dists, want[1])
    npq = (np.arange(len(queries)) % 5 + 1).astype(np.uint32)
    ids, dists, used = idx.search(queries, k=10, nprobe=6, survivors=32, nprobe_per_query=npq,
                                  return_nprobe=True, graph=True)
    assert np.array_equal(used, npq)
    for p in np.unique(npq):
        sel = np.nonzero(npq == p)[0]
        want = ref.search(queries[sel], k=10, nprobe=int(p), survivors=32)
        assert np.array_equal(ids[sel], want[0]) and np.array_equal(dists[sel], want[1]), p
