"""The learned per-query probe budget (katoann.ProbeModel, csrc/probe.cu):

* a search with per-query nprobe gives, for every query, exactly the fixed-
  nprobe result at that query's nprobe (checked against the oracle, which
  only knows fixed nprobe), on all three rankings and through the rescan path;
* the features, the MLP and the training gradients match plain numpy / torch
  fp32 restatements within the tolerances stated in each test;
* labels follow their definition, the model file round-trips, and a trained
  model's search is again exactly the oracle at the budgets it chose."""
import ctypes as C

import numpy as np
import pytest

import oracle
import synth

SPEC = dict(seed=51, n=20000, dim=64, ncomp=24, nlist=96, nq=300, rotation="random")
LADDER = (1, 2, 4, 8, 16, 32, 48)


def _index(tmp_path, spec=SPEC):
    import katoann
    prefix = str(tmp_path / "x")
    queries, _ = synth.materialize(spec, prefix)
    idx = katoann.Index()
    idx.load(prefix)
    return prefix, queries, idx


def _train_queries(spec, n, stream=30):
    return synth.to_f32(synth.mixture_ints(spec["seed"], stream, n, spec["dim"], spec["ncomp"]))


def _check_against_oracle(ref, queries, ids, dists, used, **kw):
    for v in np.unique(used):
        sel = np.nonzero(used == v)[0]
        rid, rd = ref.search(queries[sel], nprobe=int(v), **kw)
        assert np.array_equal(ids[sel], rid) and np.array_equal(dists[sel], rd), (int(v), kw)


# ------------------------------------------------------------------ on CPU
def test_model_file_errors(tmp_path):
    import katoann
    with pytest.raises(RuntimeError, match="cannot open"):
        katoann.ProbeModel.load(str(tmp_path / "none.kprb"))
    bad = tmp_path / "bad.kprb"
    bad.write_bytes(b"\x00" * 64)
    with pytest.raises(RuntimeError, match="bad header"):
        katoann.ProbeModel.load(str(bad))
    short = tmp_path / "short.kprb"
    short.write_bytes(np.array([0x4252504B, 1, 4, 64], np.uint32).tobytes() + b"\x00" * 40)
    with pytest.raises(RuntimeError, match="truncated"):
        katoann.ProbeModel.load(str(short))


def test_fit_argument_errors():
    import katoann
    z = np.zeros((10, 64), np.float32)
    with pytest.raises(ValueError, match="ladder"):
        katoann.ProbeModel.fit(z, np.zeros(10, np.uint8), ladder=(4,))
    with pytest.raises(ValueError, match="ladder"):
        katoann.ProbeModel.fit(z, np.zeros(10, np.uint8), ladder=(8, 4))
    with pytest.raises(ValueError, match="not a ladder class"):
        katoann.ProbeModel.fit(z, np.full(10, 7, np.uint8), ladder=(1, 2, 4))


# ------------------------------------------------------------------ on GPU
@pytest.mark.gpu
@pytest.mark.parametrize("ranking", ["prefix", "high", "full"])
def test_per_query_nprobe_equals_fixed_nprobe(tmp_path, ranking):
    prefix, queries, idx = _index(tmp_path)
    ref = oracle.OracleIndex(prefix)
    rng = np.random.default_rng(7)
    want = rng.integers(0, 40, len(queries)).astype(np.uint32)  # 0 is clamped to 1
    ids, dists, used = idx.search(queries, k=10, nprobe=24, ranking=ranking, survivors=32,
                                  nprobe_per_query=want, return_nprobe=True)
    assert np.array_equal(used, np.clip(want, 1, 24))
    _check_against_oracle(ref, queries, ids, dists, used, k=10, ranking=ranking, survivors=32)
    # no budget: every query reports the fixed nprobe, results unchanged
    i2, d2, u2 = idx.search(queries, k=10, nprobe=24, ranking=ranking, survivors=32,
                            return_nprobe=True)
    assert (u2 == 24).all()
    rid, rd = idx.search(queries, k=10, nprobe=24, ranking=ranking, survivors=32)
    assert np.array_equal(i2, rid) and np.array_equal(d2, rd)


@pytest.mark.gpu
def test_per_query_nprobe_through_the_rescans(tmp_path):
    """Tiny candidate buffers: overflowing queries are rescanned over their own
    probes only."""
    from _gpu import gpu
    spec = dict(seed=24, n=40000, dim=128, ncomp=8, nlist=8, nq=64, rotation="random")
    prefix, queries, idx = _index(tmp_path, spec)
    ref = oracle.OracleIndex(prefix)
    want = (np.arange(len(queries)) % 4 + 1).astype(np.uint32)
    lib = gpu()
    try:
        assert lib.katoann_gpu_set_candidate_cap(16) == 0
        ids, dists, used = idx.search(queries, k=10, nprobe=4, ranking="prefix", survivors=16,
                                      nprobe_per_query=want, return_nprobe=True)
        assert idx.search_stats()["ranking_rescans"] > 0
    finally:
        assert lib.katoann_gpu_set_candidate_cap(32768) == 0
    _check_against_oracle(ref, queries, ids, dists, used, k=10, ranking="prefix", survivors=16)


def _numpy_features(ref, queries, depth, ranks):
    """The features from the oracle's codes: exact coarse distances, sorted by
    (distance, list), then the logs (tolerance: float32 logf)."""
    q = ref.quantize(ref.rotate(queries) if ref.rotated else queries)
    c = ref.centroid_codes()
    d = oracle.sq16_l2(q["hi"], q["lo"], c["hi"], c["lo"], q["norm"], c["norm"], ref.step_sq)
    out = np.zeros((len(queries), 64), np.float32)
    for i, row in enumerate(d):
        order = np.lexsort((np.arange(len(row)), row))[:depth]
        s = row[order].astype(np.float32)
        e = np.float32(1e-4) * s[ranks[63]] + np.float32(1e-30)
        l0 = np.log(s[0] + e)
        out[i] = np.log(s[ranks] + e) - l0
        out[i, 0] = l0
    return out


@pytest.mark.gpu
def test_trained_model_search_equals_oracle_at_its_budgets(tmp_path):
    import katoann
    prefix, queries, idx = _index(tmp_path)
    ref = oracle.OracleIndex(prefix)
    train = _train_queries(SPEC, 3000)
    model = katoann.ProbeModel.train(idx, train, ladder=LADDER, depth=48, k=10, label_nprobe=96,
                                     ranking="prefix", survivors=32, epochs=40, batch=256, seed=3)
    assert model.classes == len(LADDER) and model.depth == 48
    assert np.array_equal(model.ladder, LADDER)
    loss = model.loss
    assert len(loss) == 40 and np.all(np.isfinite(loss)) and loss[-1] < loss[0]
    labels = model.labels
    assert labels.shape == (3000,) and labels.max() < len(LADDER)
    # labels by their definition, on a sample: the smallest ladder value whose
    # search recovers as much of the exact top-10 (kFull, 96 lists) as any value
    sample = train[:60]
    exact, _ = ref.search(sample, k=10, nprobe=96, ranking="full", survivors=10)
    hits = np.zeros((60, len(LADDER)), np.int64)
    for c, v in enumerate(LADDER):
        got, _ = ref.search(sample, k=10, nprobe=v, ranking="prefix", survivors=32)
        hits[:, c] = [len(set(a) & set(b)) for a, b in zip(exact, got)]
    assert np.array_equal(labels[:60], hits.argmax(1))
    # the learned search: every query's result is the oracle's at its nprobe
    for thr in (0.5, 0.9, 0.99):
        ids, dists, used = idx.search(queries, k=10, nprobe=48, ranking="prefix", survivors=32,
                                      budget=model, threshold=thr, return_nprobe=True)
        assert set(np.unique(used)) <= set(LADDER)
        _check_against_oracle(ref, queries, ids, dists, used, k=10, ranking="prefix",
                              survivors=32)
    # a higher threshold never probes less
    _, _, lo = idx.search(queries, nprobe=48, budget=model, threshold=0.5, return_nprobe=True)
    _, _, hi = idx.search(queries, nprobe=48, budget=model, threshold=0.99, return_nprobe=True)
    assert np.all(hi >= lo)
    # the cap applies
    _, _, capped = idx.search(queries, nprobe=8, budget=model, threshold=0.99, return_nprobe=True)
    assert capped.max() <= 8
    # the file round-trips: same weights, same budgets
    path = str(tmp_path / "m.kprb")
    model.save(path)
    again = katoann.ProbeModel.load(path)
    for key, v in model.weights().items():
        assert np.array_equal(v, again.weights()[key]), key
    _, _, u2 = idx.search(queries, nprobe=48, budget=again, threshold=0.9, return_nprobe=True)
    _, _, u1 = idx.search(queries, nprobe=48, budget=model, threshold=0.9, return_nprobe=True)
    assert np.array_equal(u1, u2)
    # features shallower than the cap: the queries whose budget exceeds the
    # feature depth take a second, deeper selection
    # (uniform labels: a flat distribution puts the 0.95 point in the deep classes)
    flat = np.random.default_rng(9).integers(0, len(LADDER), len(train)).astype(np.uint8)
    shallow = katoann.ProbeModel.fit(katoann.ProbeModel.features(idx, train, 16), flat,
                                     ladder=LADDER, depth=16, epochs=2, batch=256, seed=5)
    ids, dists, used = idx.search(queries, k=10, nprobe=48, survivors=32, budget=shallow,
                                  threshold=0.95, return_nprobe=True)
    assert (used > 16).any()
    _check_against_oracle(ref, queries, ids, dists, used, k=10, ranking="prefix", survivors=32)


@pytest.mark.gpu
def test_features_and_mlp_match_numpy_and_torch(tmp_path):
    torch = pytest.importorskip("torch")
    import katoann
    prefix, queries, idx = _index(tmp_path)
    ref = oracle.OracleIndex(prefix)
    depth = 64
    z = katoann.ProbeModel.features(idx, queries, depth)
    rng = np.random.default_rng(5)
    model = katoann.ProbeModel.fit(z, rng.integers(0, len(LADDER), len(z)).astype(np.uint8),
                                   ladder=LADDER, depth=depth, epochs=3, batch=64, seed=1)
    ranks = model.feature_ranks
    assert ranks[0] == 0 and ranks[-1] == depth - 1 and np.all(np.diff(ranks.astype(int)) >= 0)
    want = _numpy_features(ref, queries, depth, ranks)
    np.testing.assert_allclose(z, want, rtol=1e-5, atol=1e-5)
    # the MLP: torch fp32 on the bf16 weights (tolerance 1e-5 on probabilities)
    w = model.weights()
    f32 = lambda h: torch.from_numpy((h.astype(np.uint32) << 16).view(np.float32).copy())
    x = (torch.from_numpy(z) - torch.from_numpy(w["shift"])) * torch.from_numpy(w["scale"])
    h1 = torch.relu(x @ f32(w["w1"]) + torch.from_numpy(w["b1"]))
    h2 = torch.relu(h1 @ f32(w["w2"]) + torch.from_numpy(w["b2"]))
    probs_t = torch.softmax(h2 @ f32(w["w3"]) + torch.from_numpy(w["b3"]), dim=1).numpy()
    for thr in (0.3, 0.8, 0.97):
        probs, nprobe = model.predict(z, threshold=thr, cap=40)
        np.testing.assert_allclose(probs, probs_t, rtol=0, atol=1e-5)
        cum = np.cumsum(probs_t, axis=1)
        pick = np.where((cum >= thr).any(1), (cum >= thr).argmax(1), len(LADDER) - 1)
        clear = np.abs(cum - thr).min(1) > 1e-4  # decisions not on the threshold
        assert np.array_equal(nprobe[clear], np.minimum(np.array(LADDER)[pick[clear]], 40))


class _DevModel(C.Structure):
    """Mirror of katoann_gpu_probe_model (include/katoann_gpu.h)."""
    _fields_ = [("nclass", C.c_uint32), ("depth", C.c_uint32), ("threshold", C.c_float),
                ("reserved", C.c_uint32)] + [(n, C.c_void_p) for n in (
                    "d_rank", "d_shift", "d_scale", "d_w1", "d_b1", "d_w2", "d_b2", "d_w3", "d_b3",
                    "d_ladder")]


@pytest.mark.gpu
def test_training_gradients_match_torch():
    """katoann_gpu_probe_grads against torch autograd on the same bf16 weights
    (fp32 arithmetic; tolerance 1e-4 relative to each gradient's scale)."""
    torch = pytest.importorskip("torch")
    from _gpu import gpu
    lib = gpu()
    rng = np.random.default_rng(11)
    n, C_ = 300, 6
    bf = lambda a: torch.from_numpy(np.asarray(a, np.float32)).to(torch.bfloat16)
    w1, w2, w3 = bf(rng.normal(0, 0.2, (64, 256))), bf(rng.normal(0, 0.08, (256, 256))), \
        bf(rng.normal(0, 0.1, (256, C_)))
    b1, b2, b3 = (torch.from_numpy(rng.normal(0, 0.1, s).astype(np.float32)) for s in (256, 256, C_))
    shift = torch.from_numpy(rng.normal(0, 1, 64).astype(np.float32))
    scale = torch.from_numpy(rng.uniform(0.5, 2, 64).astype(np.float32))
    z = torch.from_numpy(rng.normal(0, 1.5, (n, 64)).astype(np.float32))
    y = torch.from_numpy(rng.integers(0, C_, n).astype(np.uint8))
    dev = lambda t: t.contiguous().cuda()
    d = {k: dev(v) for k, v in dict(w1=w1.view(torch.int16), w2=w2.view(torch.int16),
                                     w3=w3.view(torch.int16), b1=b1, b2=b2, b3=b3, shift=shift,
                                     scale=scale, z=z, y=y,
                                     rank=torch.arange(64, dtype=torch.int32),
                                     ladder=torch.arange(1, C_ + 1, dtype=torch.int32)).items()}
    m = _DevModel(C_, 64, 0.9, 0, *(C.c_void_p(d[k].data_ptr()) for k in (
        "rank", "shift", "scale", "w1", "b1", "w2", "b2", "w3", "b3", "ladder")))
    grads = {k: torch.zeros(s, device="cuda") for k, s in dict(
        w1=(64, 256), b1=(256,), w2=(256, 256), b2=(256,), w3=(256, C_), b3=(C_,)).items()}
    loss = C.c_float()
    P = C.c_void_p
    lib.katoann_gpu_probe_grads.argtypes = [P, P, P, C.c_uint32, P] + [P] * 6
    rc = lib.katoann_gpu_probe_grads(C.byref(m), P(d["z"].data_ptr()), P(d["y"].data_ptr()), n,
                                     C.byref(loss), *(P(grads[k].data_ptr()) for k in (
                                         "w1", "b1", "w2", "b2", "w3", "b3")))
    assert rc == 0, lib.katoann_gpu_last_error()
    # torch fp32 reference
    params = {k: v.float().clone().requires_grad_(True) for k, v in dict(
        w1=w1, b1=b1, w2=w2, b2=b2, w3=w3, b3=b3).items()}
    x = (z - shift) * scale
    h1 = torch.relu(x @ params["w1"] + params["b1"])
    h2 = torch.relu(h1 @ params["w2"] + params["b2"])
    ref_loss = torch.nn.functional.cross_entropy(h2 @ params["w3"] + params["b3"], y.long())
    ref_loss.backward()
    assert abs(loss.value - ref_loss.item()) <= 1e-5 * max(1.0, abs(ref_loss.item()))
    for k, p in params.items():
        g, want = grads[k].cpu(), p.grad
        tol = 1e-4 * float(want.abs().max()) + 1e-7
        assert float((g - want).abs().max()) <= tol, k


@pytest.mark.gpu
def test_graph_replay_equals_plain_search(tmp_path):
    """search_device(graph=True): captured once per call signature, replayed
    with whatever the query buffer holds; results equal the plain search."""
    torch = pytest.importorskip("torch")
    import katoann
    prefix, queries, idx = _index(tmp_path)
    train = _train_queries(SPEC, 1500)
    model = katoann.ProbeModel.fit(katoann.ProbeModel.features(idx, train, 48),
                                   np.random.default_rng(2).integers(0, len(LADDER), 1500)
                                   .astype(np.uint8), ladder=LADDER, depth=48, epochs=2, seed=4)
    nq = 128
    q = torch.empty((nq, queries.shape[1]), dtype=torch.float32, device="cuda")
    ids = torch.empty((nq, 10), dtype=torch.int32, device="cuda")
    dists = torch.empty((nq, 10), dtype=torch.float32, device="cuda")
    used = torch.empty(nq, dtype=torch.int32, device="cuda")
    st = torch.cuda.Stream()
    for kw in (dict(nprobe=24, ranking="prefix", survivors=32),
               dict(nprobe=24, ranking="full"),
               dict(nprobe=48, ranking="prefix", survivors=32, budget=model, threshold=0.8)):
        for rep in range(3):  # capture, then two replays on new contents
            block = queries[(rep * 37) % 150:][:nq]
            q.copy_(torch.from_numpy(block))
            torch.cuda.synchronize()
            extra = dict(nprobe_out=used) if "budget" in kw else {}
            idx.search_device(q, ids, dists, k=10, stream=st.cuda_stream, graph=True, **kw, **extra)
            st.synchronize()
            want = idx.search(block, k=10, return_nprobe="budget" in kw, **kw)
            assert np.array_equal(ids.cpu().numpy().view(np.uint32), want[0]), (kw, rep)
            assert np.array_equal(dists.cpu().numpy(), want[1]), (kw, rep)
            if "budget" in kw:
                assert np.array_equal(used.cpu().numpy().view(np.uint32), want[2])
