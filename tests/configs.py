"""Seeded stand-ins for the benchmark workloads, at any size (test infrastructure).

The reference measures on public datasets that are not available here; these
generators draw vectors with the shapes and value distributions the workloads
are quoted on, with numpy on the host so that the oracle and the GPU index
load the very same arrays:

  small: a 100-component Gaussian mixture, centres N(0, 1), per-component
         sigma 0.3, dimension j scaled by 1/sqrt(j + 1), L2-normalised
         (100,000 x 128, nlist 256, 1,024 queries at full size);
  plain: an anisotropic power-law spectrum (eigenvalue_i ~ i^-1.2) in a random
         orthogonal basis plus a 1,000-component mixture offset, unit norm
         (1,000,000 x 1,024, nlist 4,096 at full size);
  wide:  the same with spectrum i^-1.0 and 2,000 components (990,000 x 3,072).

`index_arrays` partitions the vectors with a few Lloyd iterations and a PCA
rotation (float BLAS; the partition only has to be reasonable, since parity is
defined over whatever index both sides load) and returns the arrays that
katoann.Index.load_arrays and oracle.OracleIndex(arrays=...) take.
"""
from __future__ import annotations

import numpy as np

SHAPES = {
    "small": dict(dim=128, nlist=256, head=64, ncomp=100),
    "plain": dict(dim=1024, nlist=4096, head=128, ncomp=1000, power=1.2),
    "wide": dict(dim=3072, nlist=4096, head=256, ncomp=2000, power=1.0),
}


def _unit(x: np.ndarray) -> np.ndarray:
    return (x / np.linalg.norm(x, axis=1, keepdims=True)).astype(np.float32)


def vectors(kind: str, n: int, nq: int, seed: int = 0, dim: int | None = None):
    """(base n x dim, queries nq x dim) float32, unit norm."""
    s = SHAPES[kind]
    d = dim or s["dim"]
    rng = np.random.default_rng(seed)
    ncomp = s["ncomp"]
    if kind == "small":
        centres = rng.standard_normal((ncomp, d))
        scale = 1.0 / np.sqrt(np.arange(d) + 1.0)

        def draw(m, g):
            comp = g.integers(0, ncomp, m)
            return _unit((centres[comp] + 0.3 * g.standard_normal((m, d))) * scale)
    else:
        q, r = np.linalg.qr(rng.standard_normal((d, d)))
        q *= np.sign(np.diag(r))[None, :]
        lam = np.arange(1, d + 1, dtype=np.float64) ** -s["power"]
        basis = (np.sqrt(lam / lam.sum())[:, None] * q.T).astype(np.float32)
        centres = rng.standard_normal((ncomp, d)).astype(np.float32) @ basis

        def draw(m, g):
            comp = g.integers(0, ncomp, m)
            return _unit(centres[comp] + 0.5 * (g.standard_normal((m, d)).astype(np.float32) @ basis))
    return draw(n, np.random.default_rng(seed + 1)), draw(nq, np.random.default_rng(seed + 2))


def _nearest(x: np.ndarray, c: np.ndarray) -> np.ndarray:
    cn = (c * c).sum(1)
    out = np.empty(len(x), np.int64)
    for s in range(0, len(x), 8192):
        xs = x[s:s + 8192]
        out[s:s + 8192] = (cn[None, :] - 2.0 * (xs @ c.T)).argmin(1)
    return out


def index_arrays(x: np.ndarray, nlist: int, head: int, iters: int = 3, seed: int = 0,
                 rotate: bool = True) -> dict:
    """Lloyd partition (initial centres: a seeded sample of rows), lists in
    ascending-id order, and the PCA rotation of a sample (row j = the axis of
    the j-th largest variance)."""
    rng = np.random.default_rng(seed + 3)
    c = x[rng.choice(len(x), nlist, replace=False)].copy()
    for _ in range(iters):
        a = _nearest(x, c)
        cnt = np.bincount(a, minlength=nlist)
        sums = np.zeros_like(c, dtype=np.float64)
        np.add.at(sums, a, x)
        nz = cnt > 0
        c[nz] = (sums[nz] / cnt[nz, None]).astype(np.float32)
    a = _nearest(x, c)
    order = np.argsort(a, kind="stable").astype(np.uint32)
    sizes = np.bincount(a, minlength=nlist).astype(np.uint32)
    rot = None
    if rotate:
        smp = x[rng.choice(len(x), min(len(x), 20000), replace=False)].astype(np.float64)
        smp -= smp.mean(0, keepdims=True)
        w, v = np.linalg.eigh(smp.T @ smp / len(smp))
        rot = np.ascontiguousarray(v[:, np.argsort(-w, kind="stable")].T, dtype=np.float32)
    return dict(centroids=np.ascontiguousarray(c, np.float32), list_sizes=sizes, ids=order,
                vectors=np.ascontiguousarray(x[order], np.float32), rotation=rot, head_dims=head)
