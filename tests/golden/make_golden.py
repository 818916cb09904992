"""Writes the golden fixtures tests/golden/*.npz from the reference itself.

Run where the reference builds (x86-64 with AVX-512 VNNI/AMX):
    make -C oracle ref && python tests/golden/make_golden.py
Each fixture holds a spec (tests/golden/synth.py turns it back into the same
index files on any host), the sha256 of those files, the reference's code
digests and scale, one coarse probe set, and the reference's search outputs
(ids, distances) for a list of parameter sets. Only fixtures with a stored
rotation/partition (the one built by the reference's own k-means and PCA)
carry arrays beyond the spec.
"""
from __future__ import annotations

import hashlib
import json
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import refbind  # noqa: E402
import synth  # noqa: E402

# (load prefix_dims, ranking, selection, k, nprobe, survivors)
FIXTURES = {
    "d128": dict(spec=dict(seed=11, n=20000, dim=128, ncomp=50, nlist=64, nq=250, rotation="random"),
                 searches=[(0, "prefix", "threshold", 10, 8, 32), (0, "prefix", "local", 10, 8, 32),
                           (0, "prefix", "threshold", 100, 16, 32), (0, "high", "threshold", 10, 8, 16),
                           (0, "full", "threshold", 10, 8, 0), (0, "full", "threshold", 10, 64, 0),
                           (0, "prefix", "local", 1, 4, 5), (128, "prefix", "local", 10, 8, 32),
                           (0, "prefix", "threshold", 10, 1, 32), (0, "prefix", "local", 20, 12, 4000)]),
    "d100": dict(spec=dict(seed=12, n=5000, dim=100, ncomp=20, nlist=32, nq=77, rotation="random",
                           far_list=5),
                 searches=[(0, "prefix", "threshold", 10, 6, 32), (0, "prefix", "local", 10, 6, 32),
                           (0, "high", "local", 10, 6, 32), (0, "full", "threshold", 10, 6, 0),
                           (0, "prefix", "local", 50, 32, 64), (128, "prefix", "local", 10, 6, 32)]),
    "d102": dict(spec=dict(seed=13, n=3000, dim=102, ncomp=10, nlist=16, nq=40, rotation="random"),
                 searches=[(0, "prefix", "local", 10, 4, 32), (0, "full", "threshold", 10, 4, 0),
                           (0, "high", "local", 10, 3, 16)]),
    "d1024": dict(spec=dict(seed=14, n=6000, dim=1024, ncomp=16, nlist=32, nq=64, rotation="random"),
                  searches=[(0, "prefix", "threshold", 10, 4, 32), (0, "prefix", "local", 10, 4, 32),
                            (0, "full", "threshold", 10, 4, 0), (128, "prefix", "local", 10, 4, 32),
                            (0, "high", "local", 10, 2, 32), (1024, "prefix", "local", 10, 3, 64)]),
    "norot": dict(spec=dict(seed=15, n=600, dim=64, ncomp=8, nlist=16, nq=3, rotation="none",
                            head_dims=64),
                  searches=[(0, "prefix", "local", 100, 1, 32), (0, "full", "threshold", 100, 2, 0),
                            (0, "high", "local", 10, 16, 32)]),
    "tinyq": dict(spec=dict(seed=18, n=2000, dim=48, ncomp=6, nlist=8, nq=2, rotation="random"),
                  searches=[(0, "prefix", "local", 10, 4, 32), (0, "full", "threshold", 5, 4, 0)]),
    "pca": dict(spec=dict(seed=16, n=10000, dim=128, ncomp=30, nlist=32, nq=100, rotation="stored"),
                searches=[(0, "prefix", "threshold", 10, 4, 32), (0, "prefix", "local", 10, 4, 32),
                          (0, "full", "threshold", 10, 4, 0), (0, "high", "local", 10, 4, 32)]),
    "nodimc": dict(spec=dict(seed=17, n=2000, dim=64, ncomp=8, nlist=8, nq=20, rotation="none",
                             dimc=False),
                   searches=[(0, "high", "local", 10, 4, 32), (0, "full", "threshold", 10, 4, 0)]),
}


def lround_half_away(x: np.ndarray) -> np.ndarray:
    t = np.trunc(x)
    f = x - t
    return (t + np.where(np.abs(f) >= 0.5, np.sign(x), 0.0)).astype(np.int64)


def quantize(idx: refbind.RefIndex, rows: np.ndarray):
    v = lround_half_away((rows.astype(np.float64) - idx.lo) * idx.inv_step)
    v = np.clip(v, 0, 65535)
    dc = idx.dc
    hi = np.zeros((len(rows), dc), np.uint8)
    lo = np.zeros((len(rows), dc), np.uint8)
    hi[:, :rows.shape[1]] = (v >> 8).astype(np.uint8)
    lo[:, :rows.shape[1]] = (v & 255).astype(np.uint8)
    return hi, lo, (v * v).sum(1)


def digest(*arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def read_stored(prefix: str, spec: dict) -> dict:
    """Reads back the partition and rotation that the reference build wrote."""
    d, nlist = spec["dim"], spec["nlist"]
    cen = np.fromfile(prefix + ".centroids", np.float32).reshape(nlist, d)
    assign = np.zeros(spec["n"], np.uint16)
    with open(prefix + ".invlist", "rb") as f:
        for c in range(nlist):
            sz = int(np.frombuffer(f.read(4), np.uint32)[0])
            ids = np.frombuffer(f.read(4 * sz), np.uint32)
            f.read(4 * sz * d)
            assign[ids] = c
    raw = np.fromfile(prefix + ".dimc", np.uint32)
    assert raw[6] == 1
    rot = raw[8:].view(np.float32).reshape(d, d).copy()
    return dict(centroids=cen, assign=assign, rotation=rot)


def make(name: str, cfg: dict, tmp: str) -> None:
    spec = dict(cfg["spec"])
    prefix = os.path.join(tmp, name)
    stored = None
    if spec["rotation"] == "stored":
        seed, n, d = spec["seed"], spec["n"], spec["dim"]
        data = synth.to_f32(synth.mixture_ints(seed, 10, n, d, spec["ncomp"]))
        refbind.build(data, prefix + "_refbuild", spec["nlist"], seed=1, rotation_sample=20000)
        stored = read_stored(prefix + "_refbuild", spec)
        ref_digest = synth.file_digest(prefix + "_refbuild")
    queries, dig = synth.materialize(spec, prefix, stored)
    if stored is not None:
        assert dig == ref_digest, "stored partition does not reproduce the reference build"
    out = dict(spec=json.dumps(spec), digest=dig)
    if stored is not None:
        out.update(stored_centroids=stored["centroids"], stored_assign=stored["assign"],
                   stored_rotation=stored["rotation"])
    searches = []
    loaded = {}
    for si, (pd, ranking, selection, k, nprobe, surv) in enumerate(cfg["searches"]):
        if pd not in loaded:
            loaded[pd] = refbind.RefIndex(prefix, prefix_dims=pd)
        idx = loaded[pd]
        ids, dists = idx.search(queries, k=k, nprobe=nprobe, ranking=ranking, survivors=surv,
                                selection=selection)
        out[f"ids_{si}"] = ids
        out[f"dists_{si}"] = dists
        searches.append(dict(prefix_dims=pd, ranking=ranking, selection=selection, k=k,
                             nprobe=nprobe, survivors=surv))
    idx = loaded[0] if 0 in loaded else next(iter(loaded.values()))
    codes = idx.codes()
    cc = idx.centroid_codes()
    out["codes_digest"] = digest(codes["hi"], codes["lo"], codes["norm"], codes["hinorm"],
                                 codes["ids"])
    out["headnorm_digest"] = digest(codes["headnorm"])
    out["centroid_digest"] = digest(cc["hi"], cc["lo"], cc["norm"])
    out["scale"] = np.array([idx.lo, idx.inv_step, idx.step, idx.step_sq], np.float64)
    out["info"] = np.array([idx.dim, idx.nlist, idx.npts, idx.dc, idx.head_dims, int(idx.rotated)],
                           np.uint32)
    # Intermediate stages of the first search: rotated queries and coarse probes.
    fq = idx.rotate_rows(queries) if idx.rotated else queries
    out["qrot_digest"] = digest(fq)
    qh, ql, qn = quantize(idx, fq)
    np0 = cfg["searches"][0][4]
    out["probed"] = idx.coarse(qh, ql, qn, np0)
    out["searches"] = json.dumps(searches)
    # Error behaviour of the reference for this index.
    errs = {}
    for label, kw in [("k0", dict(k=0, nprobe=1)), ("np0", dict(k=1, nprobe=0)),
                      ("np_gt_nlist", dict(k=1, nprobe=spec["nlist"] + 1)),
                      ("prefix", dict(k=1, nprobe=1, ranking="prefix"))]:
        try:
            idx.search(queries[:1], **kw)
            errs[label] = "ok"
        except ValueError as e:
            errs[label] = str(e)
    out["errors"] = json.dumps(errs)
    path = os.path.join(HERE, f"{name}.npz")
    np.savez_compressed(path, **out)
    print(f"{name}: {len(searches)} searches, {os.path.getsize(path)} bytes, engine {idx.engine}")


def main() -> None:
    if not refbind.available():
        sys.exit("oracle/_ref/libkatoann_ref.so is missing: run `make -C oracle ref` first")
    names = sys.argv[1:] or list(FIXTURES)
    with tempfile.TemporaryDirectory() as tmp:
        for name in names:
            make(name, FIXTURES[name], tmp)


if __name__ == "__main__":
    main()
