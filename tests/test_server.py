"""The continuous-batching server (katoann.Server, csrc/server.cpp): requests
with their own k, submitted from several threads while earlier batches are on
the device, come back exactly as a search of that query alone gives them,
with a fixed or a learned nprobe and under an HBM budget that forces small
batches."""
import threading

import numpy as np
import pytest

import synth

SPEC = dict(seed=61, n=20000, dim=64, ncomp=24, nlist=96, nq=400, rotation="random")


def test_server_before_load_is_a_logic_error():
    import katoann
    with pytest.raises(RuntimeError, match="logic error: server before load"):
        katoann.Server(katoann.Index())


def _index(tmp_path):
    import katoann
    prefix = str(tmp_path / "x")
    queries, _ = synth.materialize(SPEC, prefix)
    idx = katoann.Index()
    idx.load(prefix)
    return queries, idx


def _serve(server, queries, ks, threads=3, seed=0):
    """Submits queries[i] with ks[i] from several threads with random pauses;
    returns every result by request index."""
    ids = [None] * len(queries)
    rng = np.random.default_rng(seed)
    pauses = rng.exponential(2e-5, len(queries))

    def client(part):
        import time
        for i in part:
            time.sleep(pauses[i])
            ids[i] = server.submit(queries[i], int(ks[i]))

    parts = np.array_split(np.arange(len(queries)), threads)
    ts = [threading.Thread(target=client, args=(p,)) for p in parts]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    return [server.wait(r) for r in ids]


def _padded(n, max_batch):
    """The batch size the server's graphs run a batch of n at."""
    b = 1
    while b < n and b < 16:
        b <<= 1
    if n > 16:
        octave = 16
        while 2 * octave < n:
            octave <<= 1
        step = octave // 8
        b = -(-n // step) * step
    return min(b, max_batch)


def _check_alone(idx, queries, ks, results, **kw):
    for k in np.unique(ks):
        sel = np.nonzero(ks == k)[0]
        out = idx.search(queries[sel], k=int(k), return_nprobe=True, **kw)
        for j, i in enumerate(sel):
            ids, dists, npb, _ = results[i]
            assert np.array_equal(ids, out[0][j]) and np.array_equal(dists, out[1][j]), (i, k)
            assert npb == out[2][j]


@pytest.mark.gpu
@pytest.mark.parametrize("learned", [False, True])
def test_results_in_the_mix_equal_alone(tmp_path, learned):
    import katoann
    queries, idx = _index(tmp_path)
    model = None
    if learned:
        train = synth.to_f32(synth.mixture_ints(SPEC["seed"], 30, 2000, SPEC["dim"], SPEC["ncomp"]))
        model = katoann.ProbeModel.train(idx, train, ladder=(2, 4, 8, 16, 32), depth=32,
                                         label_nprobe=96, survivors=32, epochs=10, batch=256)
    ks = np.random.default_rng(3).choice([10, 100], len(queries))
    # learned: the graphs of k = 10 captured up front (3 slots x the padded
    # sizes up to 64: 1, 2, 4, 8, 16, 18, 20, .., 32, 36, 40, .., 64)
    server = katoann.Server(idx, max_batch=64, max_in_flight=3, max_k=100, nprobe=32,
                            survivors=32, budget=model, threshold=0.9,
                            warm_k=(10,) if learned else ())
    if learned:
        assert server.stats()["graphs"] == 3 * len({_padded(n, 64) for n in range(1, 65)}) == 3 * 21
    res = _serve(server, queries, ks)
    stats = server.stats()
    assert stats["requests"] == len(queries) and stats["batches"] >= len(queries) / 64
    assert stats["peak_in_flight"] >= 1
    assert stats["max_batch_gpu_ms"] > 0 and stats["max_enqueue_ms"] > 0
    # every batch replayed a captured search, its queries padded to a power of two
    assert stats["graph_batches"] == stats["batches"] and stats["graphs"] >= 2
    assert all(r[3] > 0 for r in res)
    _check_alone(idx, queries, ks, res, nprobe=32, survivors=32, budget=model, threshold=0.9)


@pytest.mark.gpu
def test_hbm_budget_cuts_batches(tmp_path):
    import katoann
    queries, idx = _index(tmp_path)
    ks = np.full(len(queries), 10)
    # the device memory of a 16-query batch, from a server capped at 16
    probe = katoann.Server(idx, max_batch=16, max_in_flight=1, max_k=10, nprobe=16)
    res16 = _serve(probe, queries, ks, threads=1)
    budget = probe.stats()["peak_hbm_bytes"]
    del probe
    # a server allowed 4096-query batches, but with only that much memory:
    # too little for a slot of its own per batch, so no graphs either
    small = katoann.Server(idx, max_batch=4096, max_in_flight=2, max_k=10, nprobe=16,
                           hbm_budget=budget)
    res = _serve(small, queries, ks, threads=2)
    st = small.stats()
    assert st["peak_hbm_bytes"] <= budget and st["graph_batches"] == 0
    assert st["batches"] >= len(queries) // 16 and st["mean_batch"] <= 16
    for a, b in zip(res, res16):
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    _check_alone(idx, queries, ks, res, nprobe=16)


@pytest.mark.gpu
@pytest.mark.parametrize("graphs", [True, False])
def test_burst_overlaps_batches_and_matches_the_oracle(tmp_path, graphs):
    """1,200 requests submitted at once: the dispatcher launches a batch and
    forms the next while it runs, so at least two batches are on the device
    together; every result is the oracle's for that query, bit for bit."""
    import katoann
    import oracle
    queries, idx = _index(tmp_path)
    ref = oracle.OracleIndex(str(tmp_path / "x"))
    qs = np.concatenate([queries] * 3)
    server = katoann.Server(idx, max_batch=64, max_in_flight=3, max_k=10, nprobe=96, survivors=256,
                            graphs=graphs)
    tickets = [server.submit(q, 10) for q in qs]
    res = [server.wait(t) for t in tickets]
    st = server.stats()
    assert st["requests"] == len(qs) and st["peak_in_flight"] >= 2, st
    want_ids, want_d = ref.search(qs, k=10, nprobe=96, survivors=256)
    for i, r in enumerate(res):
        assert np.array_equal(r[0], want_ids[i]) and np.array_equal(r[1], want_d[i]), i
