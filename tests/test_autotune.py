"""The ranking pass's knobs (seed rows, CTA split weight, item width) and the
autotuner that picks them: every setting gives the oracle's results bit for
bit; the autotuner returns one of its candidates and leaves results alone."""
import ctypes as C

import numpy as np
import pytest

import oracle
import synth

SPEC = dict(seed=71, n=30000, dim=128, ncomp=12, nlist=64, nq=256, rotation="random")


def test_knob_setters_check_their_ranges():
    from _gpu import gpu
    lib = gpu()
    assert lib.katoann_gpu_set_rank_width(24) == -1
    assert lib.katoann_gpu_set_rank_schedule(9) == -1
    knobs = (C.c_uint32 * 3)()
    lib.katoann_gpu_rank_knobs(knobs)
    assert lib.katoann_gpu_set_rank_width(32) == 0 and lib.katoann_gpu_set_rank_schedule(3) == 0
    mine = (C.c_uint32 * 3)()
    lib.katoann_gpu_rank_knobs(mine)
    assert list(mine)[1:] == [3, 32]
    assert lib.katoann_gpu_set_rank_width(knobs[2]) == 0
    assert lib.katoann_gpu_set_rank_schedule(knobs[1]) == 0


@pytest.mark.gpu
def test_every_knob_setting_matches_the_oracle(tmp_path):
    import katoann
    from _gpu import gpu
    lib = gpu()
    prefix = str(tmp_path / "x")
    queries, _ = synth.materialize(SPEC, prefix)
    idx = katoann.Index()
    idx.load(prefix)
    ref = oracle.OracleIndex(prefix)
    want = ref.search(queries, k=10, nprobe=12, survivors=32)
    try:
        for beta in (0, 1, 4, 8):
            for width in (0, 16, 32):
                for seed in (0, 64, 2048, 4096):
                    assert lib.katoann_gpu_set_rank_schedule(beta) == 0
                    assert lib.katoann_gpu_set_rank_width(width) == 0
                    assert lib.katoann_gpu_set_seed_rows(seed) == 0
                    got = idx.search(queries, k=10, nprobe=12, survivors=32)
                    assert np.array_equal(got[0], want[0]) and np.array_equal(got[1], want[1]), \
                        (beta, width, seed)
    finally:
        lib.katoann_gpu_set_rank_schedule(0)
        lib.katoann_gpu_set_rank_width(0)
        lib.katoann_gpu_set_seed_rows(0)


@pytest.mark.gpu
def test_autotune_keeps_results(tmp_path):
    import katoann
    from _gpu import gpu
    lib = gpu()
    prefix = str(tmp_path / "x")
    queries, _ = synth.materialize(SPEC, prefix)
    idx = katoann.Index()
    idx.load(prefix)
    ref = oracle.OracleIndex(prefix)
    try:
        t = idx.autotune(queries, k=10, nprobe=12, survivors=32)
        assert t["seed_rows"] in (1024, 2048, 4096) and t["schedule"] in (0, 1, 2, 4)
        assert t["width"] in (0, 32) and t["us_per_search"] > 0
        got = idx.search(queries, k=10, nprobe=12, survivors=32)
        want = ref.search(queries, k=10, nprobe=12, survivors=32)
        assert np.array_equal(got[0], want[0]) and np.array_equal(got[1], want[1])
    finally:
        lib.katoann_gpu_set_rank_schedule(0)
        lib.katoann_gpu_set_rank_width(0)
        lib.katoann_gpu_set_seed_rows(0)


@pytest.mark.gpu
@pytest.mark.parametrize("width", [64, 32])
def test_tile_histogram_counts_every_item(tmp_path, width):
    """search_stats()["ranking_tiles_by_queries"]: the ranking pass's tiles by
    the query count of their work item, recomputed from the oracle's probes
    (an item is up to `width` of the queries probing one list; every item
    scores all of its list's 128-row tiles)."""
    import katoann
    from _gpu import gpu
    lib = gpu()
    prefix = str(tmp_path / "x")
    queries, _ = synth.materialize(SPEC, prefix)
    idx = katoann.Index()
    idx.load(prefix)
    ref = oracle.OracleIndex(prefix)
    knobs = (C.c_uint32 * 3)()
    lib.katoann_gpu_rank_knobs(knobs)
    p = 12
    try:
        assert lib.katoann_gpu_set_rank_width(width) == 0
        idx.search(queries, k=10, nprobe=p, survivors=32)
        st = idx.search_stats()
    finally:
        assert lib.katoann_gpu_set_rank_width(knobs[2]) == 0
    q = ref.quantize(ref.rotate(queries))
    probed = ref.coarse(q["hi"], q["lo"], q["norm"], p)
    cnt = np.bincount(probed.ravel().astype(np.int64), minlength=ref.nlist)
    sizes = np.diff(ref.list_offsets().astype(np.int64))
    want = np.zeros(6, np.int64)
    for c in range(ref.nlist):
        if sizes[c] == 0:
            continue
        tiles = -(-sizes[c] // 128)
        for j in range(-(-cnt[c] // width)):
            ne = min(width, cnt[c] - j * width)
            want[0 if ne <= 2 else 1 if ne <= 4 else 2 if ne <= 8 else 3 if ne <= 16 else
                 4 if ne <= 32 else 5] += tiles
    got = np.array(list(st["ranking_tiles_by_queries"].values()), np.int64)
    assert np.array_equal(got, want), (got, want)
    assert got.sum() == st["ranking_tiles"]
    # the distinct probed lists and their rows: what the pass reads once each
    hit = (cnt > 0) & (sizes > 0)
    assert st["lists_probed"] == int(hit.sum()) and st["probed_rows"] == int(sizes[hit].sum())
