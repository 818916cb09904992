"""ctypes binding of the reference build in oracle/_ref (test infrastructure).

The library exists only where the reference compiles (x86-64 with AVX-512
VNNI/AMX, and the reference sources present); `available()` says whether it
does. It is used to make the golden fixtures and to pin the oracle
restatement, never by the product.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_ref", "libkatoann_ref.so")
RANKING = {"full": 0, "high": 1, "prefix": 2}
SELECTION = {"threshold": 0, "local": 1}

_lib = None


def available() -> bool:
    return os.path.exists(LIB_PATH)


def lib():
    global _lib
    if _lib is None:
        os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")
        _lib = C.CDLL(LIB_PATH)
        P, U32, I32, U64, D = C.c_void_p, C.c_uint32, C.c_int, C.c_uint64, C.c_double
        _lib.ref_last_error.restype = C.c_char_p
        _lib.ref_build.argtypes = [P, U32, U32, U32, U32, U32, U64, I32, U32, U32, C.c_char_p]
        _lib.ref_load.argtypes = [C.c_char_p, I32, U32, I32]
        _lib.ref_load.restype = P
        _lib.ref_free.argtypes = [P]
        _lib.ref_search.argtypes = [P, P, U32, U32, U32, I32, U32, I32, P, P]
        _lib.ref_info.argtypes = [P, P, P]
        _lib.ref_list_sizes.argtypes = [P, P]
        _lib.ref_dump_codes.argtypes = [P, P, P, P, P, P, P]
        _lib.ref_dump_centroids.argtypes = [P, P, P, P]
        _lib.ref_rotate_rows.argtypes = [P, P, U32, P]
        _lib.ref_rotate_rows_serial.argtypes = [P, P, U32, P]
        _lib.ref_coarse.argtypes = [P, P, P, P, U32, U32, P]
        _lib.ref_pack_plane.argtypes = [P, U32, U32, P]
        _lib.ref_plane_bytes.argtypes = [U32, U32]
        _lib.ref_plane_bytes.restype = C.c_size_t
        _lib.ref_sq16_l2.argtypes = [I32, P, P, P, P, P, P, D, U32, U32, U32, P]
        _lib.ref_sq16_high_l2.argtypes = [I32, P, P, P, P, D, U32, U32, U32, P, U32]
    return _lib


def _p(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def build(data: np.ndarray, prefix: str, nlist: int, seed: int = 1, train_size: int = 256000,
          iters: int = 12, normalized: bool = False, rotation_sample: int = 100000,
          jacobi_sweeps: int = 8) -> None:
    data = np.ascontiguousarray(data, dtype=np.float32)
    rc = lib().ref_build(_p(data), data.shape[0], data.shape[1], nlist, train_size, iters, seed,
                         int(normalized), rotation_sample, jacobi_sweeps, prefix.encode())
    if rc:
        raise RuntimeError(lib().ref_last_error().decode())


class RefIndex:
    def __init__(self, prefix: str, prefix_dims: int = 0, use_amx: bool = True,
                 batched_coarse: bool = True):
        self.h = lib().ref_load(prefix.encode(), int(use_amx), prefix_dims, int(batched_coarse))
        if not self.h:
            raise RuntimeError(lib().ref_last_error().decode())
        info = np.zeros(8, np.uint32)
        scale = np.zeros(4, np.float64)
        lib().ref_info(self.h, _p(info), _p(scale))
        (self.dim, self.nlist, self.npts, self.dc, self.head_dims, rot, eng, _b) = map(int, info)
        self.rotated = bool(rot)
        self.engine = "amx" if eng == 0 else "avx512"
        self.lo, self.inv_step, self.step, self.step_sq = map(float, scale)

    def __del__(self):
        if getattr(self, "h", None):
            lib().ref_free(self.h)
            self.h = None

    def search(self, q: np.ndarray, k=10, nprobe=64, ranking="prefix", survivors=32,
               selection="threshold"):
        q = np.ascontiguousarray(q, dtype=np.float32)
        nq = q.shape[0]
        ids = np.zeros((nq, k), np.uint32)
        dists = np.zeros((nq, k), np.float32)
        rc = lib().ref_search(self.h, _p(q), nq, k, nprobe, RANKING[ranking], survivors,
                              SELECTION[selection], _p(ids), _p(dists))
        if rc:
            raise ValueError(f"reference error {rc}: {lib().ref_last_error().decode()}")
        return ids, dists

    def list_sizes(self) -> np.ndarray:
        s = np.zeros(self.nlist, np.uint32)
        lib().ref_list_sizes(self.h, _p(s))
        return s

    def codes(self) -> dict:
        n, dc = self.npts, self.dc
        out = dict(hi=np.zeros((n, dc), np.uint8), lo=np.zeros((n, dc), np.uint8),
                   norm=np.zeros(n, np.int64), hinorm=np.zeros(n, np.int64),
                   headnorm=np.zeros(n, np.int64), ids=np.zeros(n, np.uint32))
        lib().ref_dump_codes(self.h, _p(out["hi"]), _p(out["lo"]), _p(out["norm"]),
                             _p(out["hinorm"]), _p(out["headnorm"]), _p(out["ids"]))
        return out

    def centroid_codes(self) -> dict:
        out = dict(hi=np.zeros((self.nlist, self.dc), np.uint8),
                   lo=np.zeros((self.nlist, self.dc), np.uint8),
                   norm=np.zeros(self.nlist, np.int64))
        lib().ref_dump_centroids(self.h, _p(out["hi"]), _p(out["lo"]), _p(out["norm"]))
        return out

    def rotate_rows(self, x: np.ndarray, serial: bool = False) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.float32)
        out = np.zeros_like(x)
        f = lib().ref_rotate_rows_serial if serial else lib().ref_rotate_rows
        f(self.h, _p(x), x.shape[0], _p(out))
        return out

    def coarse(self, qhi, qlo, qnorm, nprobe: int) -> np.ndarray:
        nq = qhi.shape[0]
        probed = np.zeros((nq, nprobe), np.uint32)
        rc = lib().ref_coarse(self.h, _p(np.ascontiguousarray(qhi)), _p(np.ascontiguousarray(qlo)),
                              _p(np.ascontiguousarray(qnorm, dtype=np.int64)), nq, nprobe,
                              _p(probed))
        if rc:
            raise ValueError(lib().ref_last_error().decode())
        return probed


def sq16_l2(qh, ql, xh, xl, qn, xn, step_sq, amx=True):
    """The reference's public sq16_l2 on row-major planes (packed here)."""
    m, dc = qh.shape
    n = xh.shape[0]
    pb = lib().ref_plane_bytes(n, dc)
    ph, pl = np.zeros(pb, np.uint8), np.zeros(pb, np.uint8)
    lib().ref_pack_plane(_p(np.ascontiguousarray(xh)), n, dc, _p(ph))
    lib().ref_pack_plane(_p(np.ascontiguousarray(xl)), n, dc, _p(pl))
    out = np.zeros((m, n), np.float32)
    lib().ref_sq16_l2(int(amx), _p(np.ascontiguousarray(qh)), _p(np.ascontiguousarray(ql)),
                      _p(ph), _p(pl), _p(np.ascontiguousarray(qn, dtype=np.int64)),
                      _p(np.ascontiguousarray(xn, dtype=np.int64)), step_sq, m, n, dc, _p(out))
    return out
