"""ctypes binding of the CPU restatement (oracle/liboracle.so).

TEST INFRASTRUCTURE: imported only by tests/, by __graft_entry__.smoke() and
by bench.py's CPU-baseline / reference leg, always as the checker or the timed
CPU baseline, never as part of the product path. `python -c "import
__graft_entry__ as g; g.build()"` compiles the library.
"""
from __future__ import annotations

import ctypes as C
import os
import platform

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, f"liboracle-{platform.machine()}.so")
RANKING = {"full": 0, "high": 1, "prefix": 2}

_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: run __graft_entry__.build() first")
        _lib = C.CDLL(LIB_PATH)
        P, U32, I32, D = C.c_void_p, C.c_uint32, C.c_int, C.c_double
        _lib.oracle_last_error.restype = C.c_char_p
        _lib.oracle_load.argtypes = [C.c_char_p, U32]
        _lib.oracle_load.restype = P
        _lib.oracle_free.argtypes = [P]
        _lib.oracle_code_begin.argtypes = [U32, U32, U32, P, P, P, P, U32]
        _lib.oracle_code_begin.restype = P
        _lib.oracle_code_rows.argtypes = [P, U32, U32, P]
        _lib.oracle_code_finish.argtypes = [P]
        _lib.oracle_code_finish.restype = P
        _lib.oracle_load_codes.argtypes = [P] * 13
        _lib.oracle_load_codes.restype = P
        _lib.oracle_load_arrays.argtypes = [U32, U32, U32, P, P, P, P, P, U32]
        _lib.oracle_load_arrays.restype = P
        _lib.oracle_search.argtypes = [P, P, U32, U32, U32, I32, U32, P, P]
        _lib.oracle_info.argtypes = [P, P, P]
        _lib.oracle_list_offsets.argtypes = [P, P]
        _lib.oracle_codes.argtypes = [P, P, P, P, P, P, P]
        _lib.oracle_centroid_codes.argtypes = [P, P, P, P]
        _lib.oracle_rotate.argtypes = [P, P, U32, P]
        _lib.oracle_rotate_with.argtypes = [P, U32, U32, P, P]
        _lib.oracle_quantize.argtypes = [P, P, U32, P, P, P, P, P]
        _lib.oracle_coarse.argtypes = [P, P, P, P, U32, U32, P]
        _lib.oracle_sq16_l2.argtypes = [P, P, P, P, P, P, D, U32, U32, U32, P]
        _lib.oracle_sq16_high_l2.argtypes = [P, P, P, P, D, U32, U32, U32, U32, P]
        _lib.oracle_to_dist.argtypes = [C.c_int64, D]
        _lib.oracle_to_dist.restype = C.c_float
        _lib.oracle_set_threads.argtypes = [I32]
        _lib.oracle_max_threads.restype = I32
    return _lib


def _p(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def set_threads(n: int) -> None:
    lib().oracle_set_threads(n)


def max_threads() -> int:
    return lib().oracle_max_threads()


class OracleIndex:
    """The restated reference index: codes, norms and search on the CPU."""

    def __init__(self, prefix: str | None, prefix_dims: int = 0, codes: dict | None = None,
                 arrays: dict | None = None, pieces=None):
        """From index files (prefix), coded arrays (codes), arrays in the file
        layout (arrays: centroids, list_sizes, ids, vectors, rotation,
        head_dims), or the same with the vectors handed over in pieces
        (arrays without "vectors", pieces: an iterable of (first row, rows))."""
        keep = []
        if pieces is not None:
            self.h = self._from_pieces(arrays, pieces)
        elif codes is not None:
            self.h = self._from_codes(codes)
        elif arrays is not None:
            a = {k: (np.ascontiguousarray(v) if isinstance(v, np.ndarray) else v)
                 for k, v in arrays.items()}
            keep.append(a)
            self.h = lib().oracle_load_arrays(
                a["centroids"].shape[1], a["centroids"].shape[0], a["vectors"].shape[0],
                _p(a["centroids"].astype(np.float32)), _p(a["list_sizes"].astype(np.uint32)),
                _p(a["ids"].astype(np.uint32)), _p(a["vectors"].astype(np.float32, copy=False)),
                _p(a["rotation"].astype(np.float32)) if a.get("rotation") is not None else None,
                int(a.get("head_dims", 0)))
        else:
            self.h = lib().oracle_load(prefix.encode(), prefix_dims)
        if not self.h:
            raise RuntimeError(lib().oracle_last_error().decode())
        self._read_info()

    @staticmethod
    def _from_pieces(a: dict, pieces):
        cen = np.ascontiguousarray(a["centroids"], dtype=np.float32)
        sizes = np.ascontiguousarray(a["list_sizes"], dtype=np.uint32)
        ids = np.ascontiguousarray(a["ids"], dtype=np.uint32)
        rot = a.get("rotation")
        rot = np.ascontiguousarray(rot, dtype=np.float32) if rot is not None else None
        h = lib().oracle_code_begin(cen.shape[1], cen.shape[0], len(ids), _p(cen), _p(sizes), _p(ids),
                                    _p(rot) if rot is not None else None, int(a.get("head_dims", 0)))
        if not h:
            raise RuntimeError(lib().oracle_last_error().decode())
        for row0, rows in pieces:
            rows = np.ascontiguousarray(rows, dtype=np.float32)
            if lib().oracle_code_rows(h, int(row0), rows.shape[0], _p(rows)):
                lib().oracle_code_finish(h)
                raise RuntimeError(lib().oracle_last_error().decode())
        return lib().oracle_code_finish(h)

    @staticmethod
    def _from_codes(c: dict):
        """c: info (u32[6]), scale (f64[4]), rotation, list_off, ids, hi, lo, norm,
        hinorm, headnorm, chi, clo, cnorm as numpy arrays (host)."""
        keys = ("info", "scale", "rotation", "list_off", "ids", "hi", "lo", "norm", "hinorm",
                "headnorm", "chi", "clo", "cnorm")
        arrs = [np.ascontiguousarray(c[k]) if c.get(k) is not None else None for k in keys]
        return lib().oracle_load_codes(*[_p(a) if a is not None else None for a in arrs])

    def _read_info(self):
        info = np.zeros(8, np.uint32)
        scale = np.zeros(4, np.float64)
        lib().oracle_info(self.h, _p(info), _p(scale))
        (self.dim, self.nlist, self.npts, self.dc, self.head_dims, rot, norm, dimc) = map(int, info)
        self.rotated, self.normalized, self.has_dimc = bool(rot), bool(norm), bool(dimc)
        self.lo, self.inv_step, self.step, self.step_sq = map(float, scale)

    def __del__(self):
        if getattr(self, "h", None):
            lib().oracle_free(self.h)
            self.h = None

    def search(self, q, k=10, nprobe=64, ranking="prefix", survivors=32):
        q = np.ascontiguousarray(q, dtype=np.float32)
        nq = q.shape[0]
        ids = np.zeros((nq, k), np.uint32)
        dists = np.zeros((nq, k), np.float32)
        rc = lib().oracle_search(self.h, _p(q), nq, k, nprobe, RANKING[ranking], survivors,
                                 _p(ids), _p(dists))
        if rc:
            raise ValueError(f"oracle error {rc}: {lib().oracle_last_error().decode()}")
        return ids, dists

    def list_offsets(self) -> np.ndarray:
        off = np.zeros(self.nlist + 1, np.uint32)
        lib().oracle_list_offsets(self.h, _p(off))
        return off

    def codes(self) -> dict:
        n, dc = self.npts, self.dc
        out = dict(hi=np.zeros((n, dc), np.uint8), lo=np.zeros((n, dc), np.uint8),
                   norm=np.zeros(n, np.int64), hinorm=np.zeros(n, np.int64),
                   headnorm=np.zeros(n, np.int64), ids=np.zeros(n, np.uint32))
        lib().oracle_codes(self.h, _p(out["hi"]), _p(out["lo"]), _p(out["norm"]),
                           _p(out["hinorm"]), _p(out["headnorm"]), _p(out["ids"]))
        return out

    def centroid_codes(self) -> dict:
        out = dict(hi=np.zeros((self.nlist, self.dc), np.uint8),
                   lo=np.zeros((self.nlist, self.dc), np.uint8),
                   norm=np.zeros(self.nlist, np.int64))
        lib().oracle_centroid_codes(self.h, _p(out["hi"]), _p(out["lo"]), _p(out["norm"]))
        return out

    def rotate(self, x) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.float32)
        out = np.zeros_like(x)
        lib().oracle_rotate(self.h, _p(x), x.shape[0], _p(out))
        return out

    def quantize(self, fq) -> dict:
        fq = np.ascontiguousarray(fq, dtype=np.float32)
        nq = fq.shape[0]
        out = dict(hi=np.zeros((nq, self.dc), np.uint8), lo=np.zeros((nq, self.dc), np.uint8),
                   norm=np.zeros(nq, np.int64), hinorm=np.zeros(nq, np.int64),
                   h0norm=np.zeros(nq, np.int64))
        lib().oracle_quantize(self.h, _p(fq), nq, _p(out["hi"]), _p(out["lo"]), _p(out["norm"]),
                              _p(out["hinorm"]), _p(out["h0norm"]))
        return out

    def coarse(self, qhi, qlo, qnorm, nprobe: int) -> np.ndarray:
        nq = qhi.shape[0]
        probed = np.zeros((nq, nprobe), np.uint32)
        rc = lib().oracle_coarse(self.h, _p(np.ascontiguousarray(qhi)), _p(np.ascontiguousarray(qlo)),
                                 _p(np.ascontiguousarray(qnorm, dtype=np.int64)), nq, nprobe,
                                 _p(probed))
        if rc:
            raise ValueError(lib().oracle_last_error().decode())
        return probed


def rotate_with(x: np.ndarray, rot: np.ndarray) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.float32)
    rot = np.ascontiguousarray(rot, dtype=np.float32)
    out = np.zeros_like(x)
    lib().oracle_rotate_with(_p(x), x.shape[0], x.shape[1], _p(rot), _p(out))
    return out


def sq16_l2(qh, ql, xh, xl, qn, xn, step_sq):
    m, dims = qh.shape
    n = xh.shape[0]
    out = np.zeros((m, n), np.float32)
    lib().oracle_sq16_l2(_p(np.ascontiguousarray(qh)), _p(np.ascontiguousarray(ql)),
                         _p(np.ascontiguousarray(xh)), _p(np.ascontiguousarray(xl)),
                         _p(np.ascontiguousarray(qn, dtype=np.int64)),
                         _p(np.ascontiguousarray(xn, dtype=np.int64)), step_sq, m, n, dims, _p(out))
    return out


def sq16_high_l2(qh, xh, qn, xn, step_sq, dims=None):
    m = qh.shape[0]
    n, plane_dim = xh.shape
    dims = dims or qh.shape[1]
    out = np.zeros((m, n), np.float32)
    lib().oracle_sq16_high_l2(_p(np.ascontiguousarray(qh)), _p(np.ascontiguousarray(xh)),
                              _p(np.ascontiguousarray(qn, dtype=np.int64)),
                              _p(np.ascontiguousarray(xn, dtype=np.int64)), step_sq, m, n, dims,
                              plane_dim, _p(out))
    return out


def to_dist(l2: int, step_sq: float) -> float:
    return float(lib().oracle_to_dist(int(l2), step_sq))
