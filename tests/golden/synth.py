"""Deterministic, platform-independent index fixtures (test infrastructure).

Every number here comes from integer arithmetic on numpy uint64/int64 arrays
(a counter-based splitmix64 stream), and every float is an integer times a
power of two that float32 holds exactly. The same spec therefore yields
byte-identical index files on any host (x86-64 here, aarch64 on the GPU machine),
which lets the reference's outputs, computed once where the reference builds,
serve as golden vectors everywhere.

The files follow the reference's on-disk format (src/index.cpp:482-505 for
.meta/.centroids/.invlist/.norms, :535-545 for .dimc). The partition is made
by a small exact-integer Lloyd iteration instead of the reference's k-means:
search parity is defined over the index files, whatever made them.
"""
from __future__ import annotations

import hashlib
import json
import os

import numpy as np

MASK = (1 << 64) - 1
SCALE_BITS = 20          # data value = int * 2^-20
ROT_BITS = 15            # rotation entry = int * 2^-15
DIMC_MAGIC = 0x434D4944  # "DIMC"


def _u64(x: int) -> np.uint64:
    return np.uint64(x & MASK)


def splitmix64(x: np.ndarray) -> np.ndarray:
    x = x.astype(np.uint64) + _u64(0x9E3779B97F4A7C15)
    z = (x ^ (x >> np.uint64(30))) * _u64(0xBF58476D1CE4E5B9)
    z = (z ^ (z >> np.uint64(27))) * _u64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


def uniform_int(seed: int, stream: int, count: int, lo: int, hi: int) -> np.ndarray:
    """count integers in [lo, hi] from stream `stream` of `seed`."""
    base = _u64(seed * 0x632BE59BD9B4E019 + stream * 0xD1B54A32D192ED03)
    r = splitmix64(np.arange(count, dtype=np.uint64) + base)
    span = np.uint64(hi - lo + 1)
    return ((r >> np.uint64(16)) % span).astype(np.int64) + lo


def dim_scale(d: int) -> np.ndarray:
    """Per-dimension integer scale decaying with the dimension index."""
    j = np.arange(d, dtype=np.int64)
    return np.maximum(1, 1024 // (1 + j // 4))


def mixture_ints(seed: int, stream: int, n: int, d: int, ncomp: int) -> np.ndarray:
    """n x d int64 vectors around ncomp integer centres, |v| < 2^24."""
    centres = uniform_int(seed, 1, ncomp * d, -1024, 1024).reshape(ncomp, d)
    comp = uniform_int(seed, stream, n, 0, ncomp - 1)
    noise = np.zeros(n * d, dtype=np.int64)
    for t in range(4):
        noise += uniform_int(seed, stream + 1 + t, n * d, -128, 128)
    v = (centres[comp] + noise.reshape(n, d)) * dim_scale(d)[None, :]
    return v


def to_f32(v: np.ndarray) -> np.ndarray:
    out = v.astype(np.float32) * np.float32(2.0 ** -SCALE_BITS)
    return np.ascontiguousarray(out, dtype=np.float32)


def nearest(x: np.ndarray, c: np.ndarray) -> np.ndarray:
    """Index of the nearest centre by exact int64 squared L2 (first on ties)."""
    xx = (x * x).sum(1)
    cc = (c * c).sum(1)
    out = np.empty(len(x), dtype=np.int64)
    for s in range(0, len(x), 4096):
        xs = x[s:s + 4096]
        d2 = xx[s:s + 4096, None] + cc[None, :] - 2 * (xs @ c.T)
        out[s:s + 4096] = d2.argmin(1)
    return out


def partition(x: np.ndarray, nlist: int, iters: int, far_list: int | None):
    n = len(x)
    cen = x[(np.arange(nlist, dtype=np.int64) * n) // nlist].copy()
    for _ in range(iters):
        a = nearest(x, cen)
        for c in range(nlist):
            m = a == c
            cnt = int(m.sum())
            if cnt:
                cen[c] = x[m].sum(0) // cnt
    if far_list is not None:
        cen[far_list] = (1 << 22)  # no vector is nearest: an empty list
    return cen, nearest(x, cen)


def rotation_ints(seed: int, d: int) -> np.ndarray:
    """A general (not orthogonal) d x d matrix with exact float32 entries; it
    exercises every rounding step of the query and list rotation."""
    return uniform_int(seed, 7, d * d, -32767, 32767).reshape(d, d)


def default_head(d: int) -> int:
    dc = (d + 63) // 64 * 64
    return min(max(64, (d // 4 + 63) // 64 * 64), dc)


def write_index(prefix: str, data: np.ndarray, centroids: np.ndarray, assign: np.ndarray,
                rotation: np.ndarray | None, head_dims: int | None, normalized: bool = False,
                dimc: bool = True) -> None:
    n, d = data.shape
    nlist = len(centroids)
    with open(prefix + ".meta", "wb") as f:
        np.array([d, nlist, n, 0, 1 if normalized else 0], dtype=np.uint32).tofile(f)
    with open(prefix + ".centroids", "wb") as f:
        np.ascontiguousarray(centroids, dtype=np.float32).tofile(f)
    with open(prefix + ".invlist", "wb") as f, open(prefix + ".norms", "wb") as g:
        for c in range(nlist):
            ids = np.nonzero(assign == c)[0].astype(np.uint32)
            np.array([len(ids)], dtype=np.uint32).tofile(f)
            ids.tofile(f)
            np.ascontiguousarray(data[ids], dtype=np.float32).tofile(f)
            np.array([len(ids)], dtype=np.uint32).tofile(g)
    if dimc:
        rotated = rotation is not None
        hdr = [DIMC_MAGIC, 2, d, nlist, n, head_dims or 0, 1 if rotated else 0, 0]
        with open(prefix + ".dimc", "wb") as f:
            np.array(hdr, dtype=np.uint32).tofile(f)
            if rotated:
                np.ascontiguousarray(rotation, dtype=np.float32).tofile(f)


def file_digest(prefix: str) -> str:
    h = hashlib.sha256()
    for ext in (".meta", ".centroids", ".invlist", ".dimc"):
        if os.path.exists(prefix + ext):
            with open(prefix + ext, "rb") as f:
                h.update(f.read())
    return h.hexdigest()


def materialize(spec: dict, prefix: str, stored: dict | None = None) -> tuple[np.ndarray, str]:
    """Writes the index files of `spec` under `prefix`; returns (queries, digest).

    `stored` supplies arrays that are not derived from the spec (a rotation and
    partition made by the reference's own build, kept in the fixture)."""
    seed, n, d = spec["seed"], spec["n"], spec["dim"]
    xi = mixture_ints(seed, 10, n, d, spec["ncomp"])
    qi = mixture_ints(seed, 20, spec["nq"], d, spec["ncomp"])
    data, queries = to_f32(xi), to_f32(qi)
    if stored is not None and "centroids" in stored:
        centroids = stored["centroids"]
        assign = stored["assign"].astype(np.int64)
    else:
        cen, assign = partition(xi, spec["nlist"], spec.get("iters", 2), spec.get("far_list"))
        centroids = to_f32(cen)
    rot = None
    if spec["rotation"] == "random":
        rot = rotation_ints(seed, d).astype(np.float32) * np.float32(2.0 ** -ROT_BITS)
    elif spec["rotation"] == "stored":
        rot = stored["rotation"]
    head = spec.get("head_dims", default_head(d))
    write_index(prefix, data, centroids, assign, rot, head, dimc=spec.get("dimc", True))
    return queries, file_digest(prefix)


def load_fixture(path: str):
    z = np.load(path, allow_pickle=False)
    spec = json.loads(str(z["spec"]))
    return spec, z
