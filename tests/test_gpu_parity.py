"""GPU search against the reference's own outputs (golden fixtures) and the
oracle: ids and distances must be bit-identical. Runs through the public API
(katoann.Index over libkatoann.so / libkatoann_gpu.so)."""
import numpy as np
import pytest

import oracle
from _util import FIXTURES, fixture, same, searches

pytestmark = pytest.mark.gpu


def _load(prefix, pd, **kw):
    import katoann
    idx = katoann.Index()
    idx.load(prefix, prefix_dims=pd, **kw)
    return idx


@pytest.mark.parametrize("name", FIXTURES)
def test_search_matches_reference_bit_exact(name):
    spec, z, prefix, queries = fixture(name)
    loaded = {}
    for i, s in enumerate(searches(z)):
        pd = s["prefix_dims"]
        if pd not in loaded:
            loaded[pd] = _load(prefix, pd)
        ids, dists = loaded[pd].search(queries, k=s["k"], nprobe=s["nprobe"], ranking=s["ranking"],
                                       survivors=s["survivors"], selection=s["selection"])
        rid, rd = z[f"ids_{i}"], z[f"dists_{i}"]
        assert same(rid, rd, ids, dists), f"{name} search {i} {s}: not same()"
        bad = np.nonzero((ids != rid).any(1) | (dists != rd).any(1))[0]
        assert len(bad) == 0, f"{name} search {i} {s}: {len(bad)} queries differ, first {bad[:5]}"


@pytest.mark.parametrize("name", ["d128", "d1024", "pca"])
def test_search_matches_oracle_on_other_settings(name):
    spec, z, prefix, queries = fixture(name)
    idx = _load(prefix, 0)
    ref = oracle.OracleIndex(prefix)
    for k, nprobe, ranking, surv in [(10, 2, "prefix", 32), (5, 3, "high", 7), (16, 5, "full", 0),
                                     (10, spec["nlist"], "prefix", 64), (3, 1, "prefix", 1)]:
        ids, dists = idx.search(queries, k=k, nprobe=nprobe, ranking=ranking, survivors=surv)
        rid, rd = ref.search(queries, k=k, nprobe=nprobe, ranking=ranking, survivors=surv)
        assert np.array_equal(ids, rid) and np.array_equal(dists, rd), (k, nprobe, ranking, surv)


def test_errors_match_reference():
    import json
    for name in ("d128", "nodimc"):
        spec, z, prefix, queries = fixture(name)
        idx = _load(prefix, 0)
        errs = json.loads(str(z["errors"]))
        cases = {"k0": dict(k=0, nprobe=1), "np0": dict(k=1, nprobe=0),
                 "np_gt_nlist": dict(k=1, nprobe=spec["nlist"] + 1),
                 "prefix": dict(k=1, nprobe=1, ranking="prefix")}
        for label, kw in cases.items():
            if errs[label] == "ok":
                idx.search(queries[:1], **kw)
            else:
                with pytest.raises(ValueError) as e:
                    idx.search(queries[:1], **kw)
                assert errs[label].split(": ", 1)[1] in str(e.value)


def test_results_do_not_depend_on_batch_composition():
    """Every stage is per query, so a query's answer is the same alone, in any
    batch and across device passes (max_batch)."""
    import katoann
    spec, z, prefix, queries = fixture("d128")
    full = _load(prefix, 0)
    ids, dists = full.search(queries, k=10, nprobe=8)
    small = katoann.Index()
    small.load(prefix, max_batch=7)
    i2, d2 = small.search(queries, k=10, nprobe=8)
    assert np.array_equal(ids, i2) and np.array_equal(dists, d2)
    perm = np.random.default_rng(0).permutation(len(queries))
    i3, d3 = full.search(queries[perm], k=10, nprobe=8)
    assert np.array_equal(ids[perm], i3) and np.array_equal(dists[perm], d3)
    for q in (0, 17, len(queries) - 1):
        i4, d4 = full.search(queries[q:q + 1], k=10, nprobe=8)
        assert np.array_equal(ids[q:q + 1], i4) and np.array_equal(dists[q:q + 1], d4)


def test_empty_batch_returns_nothing():
    spec, z, prefix, queries = fixture("d128")
    idx = _load(prefix, 0)
    ids, dists = idx.search(queries[:0], k=10, nprobe=8)
    assert ids.shape == (0, 10)


def test_invalid_prefix_dims_rejected():
    spec, z, prefix, queries = fixture("d100")
    import katoann
    for pd in (32, 192):
        with pytest.raises(ValueError, match="prefix_dims"):
            katoann.Index().load(prefix, prefix_dims=pd)


def test_normalized_index_normalizes_queries(tmp_path):
    """The module scales queries of a normalized index to unit length first
    (python/katoann_module.cpp:97-110), in double as the reference does."""
    import katoann
    import synth
    prefix = str(tmp_path / "n")
    spec = dict(seed=5, n=3000, dim=64, ncomp=6, nlist=8, nq=40, rotation="random")
    queries, _ = synth.materialize(spec, prefix)
    meta = np.fromfile(prefix + ".meta", np.uint32)
    meta[4] = 1
    meta.tofile(prefix + ".meta")
    idx = _load(prefix, 0)
    assert idx.normalized
    ids, dists = idx.search(queries, k=10, nprobe=4)
    ref = oracle.OracleIndex(prefix)
    rid, rd = ref.search(katoann.normalize_rows(queries), k=10, nprobe=4)
    assert np.array_equal(ids, rid) and np.array_equal(dists, rd)


@pytest.mark.parametrize("spec,searches_", [
    # few long lists: several 1024-row chunks per list, > 64 queries per list
    (dict(seed=21, n=20000, dim=128, ncomp=8, nlist=4, nq=300, rotation="random"),
     [(10, 2, "prefix", 32), (10, 1, "high", 64), (100, 2, "prefix", 32), (10, 3, "prefix", 256)]),
    # h = 1024 in the high-byte mode (four 256-dimension chunks)
    (dict(seed=22, n=3000, dim=1024, ncomp=8, nlist=8, nq=40, rotation="random"),
     [(10, 2, "high", 32), (10, 3, "prefix", 48)]),
    # h = 2048: two accumulators of 1024 dimensions
    (dict(seed=23, n=1500, dim=2048, ncomp=6, nlist=6, nq=24, rotation="none", head_dims=2048),
     [(10, 2, "high", 32), (5, 2, "prefix", 16)]),
])
def test_tensor_core_ranking_shapes_match_oracle(tmp_path, spec, searches_):
    import katoann
    import synth
    prefix = str(tmp_path / "x")
    queries, _ = synth.materialize(spec, prefix)
    idx = _load(prefix, 0)
    ref = oracle.OracleIndex(prefix)
    for k, nprobe, ranking, surv in searches_:
        ids, dists = idx.search(queries, k=k, nprobe=nprobe, ranking=ranking, survivors=surv)
        rid, rd = ref.search(queries, k=k, nprobe=nprobe, ranking=ranking, survivors=surv)
        bad = np.nonzero((ids != rid).any(1) | (dists != rd).any(1))[0]
        assert len(bad) == 0, (k, nprobe, ranking, surv, bad[:5])
        assert idx.search_stats()["coarse_boundary_ties"] >= 0


@pytest.mark.gpu
def test_candidate_buffer_overflow_is_rescanned_exactly(tmp_path):
    """A candidate buffer far too small: every query overflows and is rescanned;
    the results stay those of the oracle."""
    import katoann
    import synth
    from _gpu import gpu
    # long lists: the seed bound comes from 1024 of a query's ~10,000 nearest rows
    spec = dict(seed=24, n=40000, dim=128, ncomp=8, nlist=4, nq=64, rotation="random")
    prefix = str(tmp_path / "x")
    queries, _ = synth.materialize(spec, prefix)
    idx = _load(prefix, 0)
    ref = oracle.OracleIndex(prefix)
    lib = gpu()
    idx.search(queries, k=10, nprobe=2, ranking="prefix", survivors=10)
    most = idx.search_stats()["ranking_max_candidates"]
    assert most > 16
    try:
        # cap = survivors: the bound-tightening rounds rarely converge and the
        # rescan ends in the full selection; a cap a third of the largest
        # candidate count with survivors 10: the rounds converge
        for cap, ranking, surv in ((16, "prefix", 16), (16, "high", 16),
                                   (max(16, most // 3), "prefix", 10)):
            assert lib.katoann_gpu_set_candidate_cap(cap) == 0
            ids, dists = idx.search(queries, k=10, nprobe=2, ranking=ranking, survivors=surv)
            stats = idx.search_stats()
            rid, rd = ref.search(queries, k=10, nprobe=2, ranking=ranking, survivors=surv)
            assert np.array_equal(ids, rid) and np.array_equal(dists, rd), (cap, ranking)
            assert stats["ranking_rescans"] > 0 and stats["ranking_timeouts"] == 0, (cap, stats)
    finally:
        assert lib.katoann_gpu_set_candidate_cap(32768) == 0
