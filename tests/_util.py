"""Shared helpers of the test suite (fixture materialisation, parity predicates)."""
from __future__ import annotations

import json
import os
import tempfile

import numpy as np

import synth

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FIXTURES = ["d128", "d100", "d102", "d1024", "norot", "tinyq", "pca", "nodimc"]
_CACHE: dict = {}
_TMP = tempfile.mkdtemp(prefix="katoann_fixtures_")


def fixture(name: str):
    """(spec, npz, prefix, queries): index files written under a temp dir, once."""
    if name not in _CACHE:
        spec, z = synth.load_fixture(os.path.join(GOLDEN, f"{name}.npz"))
        stored = None
        if spec["rotation"] == "stored":
            stored = dict(centroids=z["stored_centroids"], assign=z["stored_assign"],
                          rotation=z["stored_rotation"])
        prefix = os.path.join(_TMP, name)
        queries, dig = synth.materialize(spec, prefix, stored)
        assert dig == str(z["digest"]), f"{name}: regenerated index files differ from the fixture"
        _CACHE[name] = (spec, z, prefix, queries)
    return _CACHE[name]


def searches(z):
    return json.loads(str(z["searches"]))


def same(a_ids, a_d, b_ids, b_d) -> bool:
    """The reference's parity predicate (tests/test_index.cpp:203-213): equal
    distances at every rank; ids equal wherever the distance is strictly below
    that query's k-th distance."""
    if not np.array_equal(a_d, b_d):
        return False
    last = a_d[:, -1:]
    strict = a_d < last
    return bool(np.all(a_ids[strict] == b_ids[strict]))
