"""Failure detection without a GPU fault: every pipeline wait of the
tensor-core ranking pass is bounded, and a CTA whose wait runs out sets its
error flag, lets its copies and MMAs in flight finish, frees its tensor memory
and returns. Here the bound is set far below one pipeline step, so waits run
out on purpose: the search must fail with TimeoutError (the host reads the
count of such CTAs after each device pass), and the next search at the default
bound must be the oracle's again, bit for bit."""
import numpy as np
import pytest

import oracle
from _util import fixture

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("cycles", [200, 1000])
def test_short_wait_limit_fails_cleanly_then_search_recovers(cycles):
    import katoann
    spec, z, prefix, queries = fixture("d128")
    idx = katoann.Index()
    idx.load(prefix)
    ref = oracle.OracleIndex(prefix)
    want = ref.search(queries, k=10, nprobe=8, survivors=32)
    try:
        katoann.set_wait_limit(cycles)
        with pytest.raises(TimeoutError, match="bounded pipeline wait"):
            idx.search(queries, k=10, nprobe=8, survivors=32)
        assert idx.search_stats()["ranking_timeouts"] > 0
    finally:
        katoann.set_wait_limit(0)
    for _ in range(2):
        got = idx.search(queries, k=10, nprobe=8, survivors=32)
        assert np.array_equal(got[0], want[0]) and np.array_equal(got[1], want[1])
        assert idx.search_stats()["ranking_timeouts"] == 0


def test_wait_limit_range():
    import katoann
    with pytest.raises(ValueError):
        katoann.set_wait_limit(1 << 41)
    katoann.set_wait_limit(0)
