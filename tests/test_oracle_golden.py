"""The CPU restatement (oracle) against the reference's golden outputs.

This pins the oracle: every search of every fixture must match the reference
bit for bit (ids and distances), and the intermediate stages (codes, scale,
rotation, coarse probes) must match the reference's digests."""
import hashlib

import numpy as np
import pytest

import oracle
from _util import FIXTURES, fixture, same, searches


def _digest(*arrays):
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


@pytest.mark.parametrize("name", FIXTURES)
def test_oracle_search_matches_reference(name):
    spec, z, prefix, queries = fixture(name)
    loaded = {}
    for i, s in enumerate(searches(z)):
        pd = s["prefix_dims"]
        if pd not in loaded:
            loaded[pd] = oracle.OracleIndex(prefix, prefix_dims=pd)
        ids, dists = loaded[pd].search(queries, k=s["k"], nprobe=s["nprobe"], ranking=s["ranking"],
                                       survivors=s["survivors"])
        rid, rd = z[f"ids_{i}"], z[f"dists_{i}"]
        assert same(rid, rd, ids, dists), f"{name} search {i} {s}: not same()"
        assert np.array_equal(ids, rid) and np.array_equal(dists, rd), f"{name} search {i} {s}"


@pytest.mark.parametrize("name", FIXTURES)
def test_oracle_stages_match_reference(name):
    spec, z, prefix, queries = fixture(name)
    o = oracle.OracleIndex(prefix)
    scale = z["scale"]
    assert (o.lo, o.inv_step, o.step, o.step_sq) == tuple(float(v) for v in scale)
    c = o.codes()
    assert _digest(c["hi"], c["lo"], c["norm"], c["hinorm"], c["ids"]) == str(z["codes_digest"])
    if o.head_dims:
        assert _digest(c["headnorm"]) == str(z["headnorm_digest"])
    cc = o.centroid_codes()
    assert _digest(cc["hi"], cc["lo"], cc["norm"]) == str(z["centroid_digest"])
    fq = o.rotate(queries)
    assert _digest(fq) == str(z["qrot_digest"])
    q = o.quantize(fq)
    probed = o.coarse(q["hi"], q["lo"], q["norm"], searches(z)[0]["nprobe"])
    ref = z["probed"]
    assert np.array_equal(np.sort(probed, 1), np.sort(ref, 1))


@pytest.mark.parametrize("name", FIXTURES)
def test_oracle_errors_match_reference(name):
    import json
    spec, z, prefix, queries = fixture(name)
    o = oracle.OracleIndex(prefix)
    errs = json.loads(str(z["errors"]))
    cases = {"k0": dict(k=0, nprobe=1), "np0": dict(k=1, nprobe=0),
             "np_gt_nlist": dict(k=1, nprobe=spec["nlist"] + 1),
             "prefix": dict(k=1, nprobe=1, ranking="prefix")}
    for label, kw in cases.items():
        if errs[label] == "ok":
            o.search(queries[:1], **kw)
        else:
            with pytest.raises(ValueError) as e:
                o.search(queries[:1], **kw)
            assert errs[label].split(": ", 1)[1] in str(e.value)
