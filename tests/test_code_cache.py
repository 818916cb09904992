"""The device-code cache (Index.save_codes / load_codes / load(code_cache=True)):
an index loaded from the cache searches exactly like the one loaded from the
reference's files, and a cache made from other files or settings is not used."""
import os

import numpy as np
import pytest

import oracle
import synth

SPEC = dict(seed=41, n=5000, dim=100, ncomp=10, nlist=24, nq=120, rotation="random")


def _search(idx, q, **kw):
    return idx.search(q, k=10, nprobe=6, survivors=32, **kw)


def test_bad_cache_files_are_refused(tmp_path):
    import katoann
    idx = katoann.Index()
    with pytest.raises(RuntimeError, match="cannot open"):
        idx.load_codes(str(tmp_path / "none.gpucodes"))
    bad = tmp_path / "bad.gpucodes"
    bad.write_bytes(b"not a code cache" * 8)
    with pytest.raises(RuntimeError, match="bad header"):
        idx.load_codes(str(bad))


@pytest.mark.gpu
def test_saved_codes_search_like_the_files(tmp_path):
    import katoann
    prefix = str(tmp_path / "x")
    queries, _ = synth.materialize(SPEC, prefix)
    a = katoann.Index()
    a.load(prefix)
    path = str(tmp_path / "x.codes")
    a.save_codes(path)
    b = katoann.Index()
    b.load_codes(path)
    assert (b.dim, b.nlist, b.size, b.prefix_dims, b.rotated) == (a.dim, a.nlist, a.size,
                                                                 a.prefix_dims, a.rotated)
    ref = oracle.OracleIndex(prefix)
    for ranking in ("prefix", "high", "full"):
        ia, da = _search(a, queries, ranking=ranking)
        ib, db = _search(b, queries, ranking=ranking)
        ir, dr = _search(ref, queries, ranking=ranking)
        assert np.array_equal(ia, ib) and np.array_equal(da, db)
        assert np.array_equal(ib, ir) and np.array_equal(db, dr)
    # a truncated file is refused
    blob = open(path, "rb").read()
    cut = str(tmp_path / "cut.codes")
    with open(cut, "wb") as f:
        f.write(blob[: len(blob) // 2])
    with pytest.raises(RuntimeError, match="truncated|bad array"):
        katoann.Index().load_codes(cut)


@pytest.mark.gpu
def test_load_through_the_cache(tmp_path):
    import katoann
    prefix = str(tmp_path / "x")
    queries, _ = synth.materialize(SPEC, prefix)
    cache = prefix + ".gpucodes"
    first = katoann.Index()
    first.load(prefix, code_cache=True)
    assert os.path.exists(cache)
    stamp = os.stat(cache).st_mtime_ns
    second = katoann.Index()
    second.load(prefix, code_cache=True)  # from the cache: the file is not rewritten
    assert os.stat(cache).st_mtime_ns == stamp
    ref = oracle.OracleIndex(prefix)
    want = _search(ref, queries)
    for idx in (first, second):
        got = _search(idx, queries)
        assert np.array_equal(got[0], want[0]) and np.array_equal(got[1], want[1])
    # another prefix_dims: the cache does not apply; the load codes the files again
    third = katoann.Index()
    third.load(prefix, code_cache=True, prefix_dims=128)
    assert third.prefix_dims == 128
    ref128 = oracle.OracleIndex(prefix, prefix_dims=128)
    got, want = _search(third, queries), _search(ref128, queries)
    assert np.array_equal(got[0], want[0]) and np.array_equal(got[1], want[1])
    # rewritten index files (another partition): the old cache is not used
    synth.materialize(dict(SPEC, seed=42), prefix)
    fourth = katoann.Index()
    fourth.load(prefix, code_cache=True)
    got, want = _search(fourth, queries), _search(oracle.OracleIndex(prefix), queries)
    assert np.array_equal(got[0], want[0]) and np.array_equal(got[1], want[1])
