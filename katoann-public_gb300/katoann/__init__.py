"""KatoANN's Python module on one GB300.

Mirrors the reference module (python/katoann_module.cpp:34-129): ``build``,
``Index().load(...)``, ``Index.search(...) -> (ids, dists)``, the read-only
properties and ``amx_available``. Searches run as sm_103a kernels through
libkatoann.so / libkatoann_gpu.so (bound here with ctypes, which releases the
GIL during each call, as the reference's module does). There is no CPU
fallback: importing fails loudly when the libraries are missing.

Additions: ``Index.load_arrays`` (an index from numpy arrays or CUDA tensors),
``Index.search_device`` (CUDA tensors in and out, no host copies) and
``Index.search_stats``.
"""
from __future__ import annotations

import ctypes as C
import os
import platform

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIBDIR = os.path.join(_HERE, "_lib", platform.machine())
_RANKING = {"full": 0, "high": 1, "prefix": 2}
_SELECTION = {"threshold": 0, "local": 1}


def _load():
    path = os.path.join(_LIBDIR, "libkatoann.so")
    if not os.path.exists(path):
        raise ImportError(f"{path} is missing: build with `python -c 'import __graft_entry__ as g; g.build()'`")
    C.CDLL(os.path.join(_LIBDIR, "libkatoann_gpu.so"), mode=C.RTLD_GLOBAL)
    lib = C.CDLL(path)
    P, U32, I32, U64, D, S = C.c_void_p, C.c_uint32, C.c_int, C.c_uint64, C.c_double, C.c_size_t
    lib.katoann_last_error.restype = C.c_char_p
    lib.katoann_build.argtypes = [P, U32, U32, U32, U32, U32, U64, I32, U32, U32, C.c_char_p]
    lib.katoann_index_new.restype = P
    lib.katoann_index_free.argtypes = [P]
    lib.katoann_index_load.argtypes = [P, C.c_char_p, I32, I32, U32, I32, U32]
    lib.katoann_index_load_arrays.argtypes = [P, U32, U32, U32, I32, P, P, P, P, P, I32, U32, I32,
                                              U32, U32]
    lib.katoann_index_search.argtypes = [P, P, U32, U32, U32, I32, U32, I32, P, P]
    lib.katoann_index_search_device.argtypes = [P, P, U32, U32, U32, I32, U32, I32, P, P, P]
    lib.katoann_index_info.argtypes = [P, P]
    lib.katoann_index_memory_bytes.argtypes = [P]
    lib.katoann_index_memory_bytes.restype = S
    lib.katoann_index_list_sizes.argtypes = [P, P]
    lib.katoann_index_stats.argtypes = [P, P, U32]
    lib.katoann_index_device_view.argtypes = [P]
    lib.katoann_index_device_view.restype = P
    lib.katoann_normalize_rows.argtypes = [P, S, U32]
    lib.katoann_dist_value.argtypes = [C.c_int64, D]
    lib.katoann_dist_value.restype = C.c_float
    return lib


_lib = _load()


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def _check(rc: int) -> None:
    if rc == 0:
        return
    msg = _lib.katoann_last_error().decode()
    if rc == -1:
        raise ValueError(msg)
    if rc == -3:
        raise RuntimeError(f"logic error: {msg}")
    raise RuntimeError(msg)


def amx_available() -> bool:
    """False: this build uses no CPU matrix engine."""
    return False


def build(data, prefix: str, nlist: int = 2048, train_size: int = 256000, kmeans_iters: int = 12,
          seed: int = 0, normalized: bool = False, rotation_sample: int = 100000,
          jacobi_sweeps: int = 8) -> None:
    """Partition data (n x dim float32) and write the index files under prefix."""
    data = np.ascontiguousarray(data, dtype=np.float32)
    if data.ndim != 2:
        raise ValueError("data must be a 2-D float32 array")
    _check(_lib.katoann_build(_ptr(data), data.shape[0], data.shape[1], nlist, train_size,
                              kmeans_iters, seed, int(normalized), rotation_sample, jacobi_sweeps,
                              prefix.encode()))


def normalize_rows(x: np.ndarray) -> np.ndarray:
    """Unit-length rows, computed as the reference's module does (double sum)."""
    out = np.array(x, dtype=np.float32, order="C", copy=True)
    _lib.katoann_normalize_rows(_ptr(out), out.shape[0], out.shape[1])
    return out


def dist_value(l2: int, step_sq: float) -> float:
    """float(double(l2) * step_sq), by the integer method of the kernels."""
    return float(_lib.katoann_dist_value(int(l2), float(step_sq)))


class Index:
    def __init__(self):
        self._h = _lib.katoann_index_new()

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            _lib.katoann_index_free(h)
            self._h = None

    def load(self, prefix: str, precision: str = "sq16", use_amx: bool = True, prefix_dims: int = 0,
             batched_coarse: bool = True, max_batch: int = 4096) -> None:
        if precision not in ("sq16", "bf16"):
            raise ValueError("precision is 'sq16' or 'bf16'")
        _check(_lib.katoann_index_load(self._h, prefix.encode(), 1 if precision == "bf16" else 0,
                                       int(use_amx), prefix_dims, int(batched_coarse), max_batch))

    def load_arrays(self, centroids, list_sizes, ids, vectors, rotation=None, head_dims: int = 0,
                    has_dimc: bool | None = None, normalized: bool = False, prefix_dims: int = 0,
                    max_batch: int = 4096) -> None:
        """An index from arrays, lists concatenated in list order: centroids
        (nlist x dim), list_sizes (nlist), ids (n), vectors (n x dim),
        rotation (dim x dim or None). numpy arrays, or CUDA tensors (then the
        vectors never leave the device)."""
        sizes = np.ascontiguousarray(np.asarray(list_sizes), dtype=np.uint32)
        on_device = hasattr(vectors, "is_cuda") and vectors.is_cuda
        keep = []

        def ptr(a, dtype):
            if a is None:
                return None
            if on_device:
                t = a.contiguous()
                keep.append(t)
                return C.c_void_p(t.data_ptr())
            arr = np.ascontiguousarray(a, dtype=dtype)
            keep.append(arr)
            return _ptr(arr)

        nlist, dim = int(centroids.shape[0]), int(centroids.shape[1])
        npts = int(vectors.shape[0])
        if has_dimc is None:
            has_dimc = rotation is not None or head_dims > 0
        _check(_lib.katoann_index_load_arrays(
            self._h, dim, nlist, npts, int(normalized), ptr(centroids, np.float32), _ptr(sizes),
            ptr(ids, np.uint32), ptr(vectors, np.float32), ptr(rotation, np.float32), int(has_dimc),
            head_dims, int(on_device), prefix_dims, max_batch))

    def search(self, queries, k: int = 10, nprobe: int = 64, ranking: str = "prefix",
               survivors: int = 32, selection: str = "threshold"):
        """Search all queries together; returns (ids uint32 [nq, k], squared
        L2 distances float32 [nq, k]), nearest first. Queries are normalized
        when the index was built with normalized=True."""
        if ranking not in _RANKING:
            raise ValueError("ranking is 'prefix', 'high' or 'full'")
        if selection not in _SELECTION:
            raise ValueError("selection is 'threshold' or 'local'")
        q = np.ascontiguousarray(queries, dtype=np.float32)
        if q.ndim != 2 or q.shape[1] != self.dim:
            raise ValueError("queries must be (n, dim) float32")
        if self.normalized:
            q = normalize_rows(q)
        nq = q.shape[0]
        ids = np.zeros((nq, k), np.uint32)
        dists = np.zeros((nq, k), np.float32)
        _check(_lib.katoann_index_search(self._h, _ptr(q), nq, k, nprobe, _RANKING[ranking],
                                         survivors, _SELECTION[selection], _ptr(ids), _ptr(dists)))
        return ids, dists

    def search_into(self, q_ptr: int, nq: int, ids_ptr: int, dists_ptr: int, k: int = 10,
                    nprobe: int = 64, ranking: str = "prefix", survivors: int = 32,
                    selection: str = "threshold") -> None:
        """search() on raw host pointers (e.g. pinned buffers); no normalisation."""
        _check(_lib.katoann_index_search(self._h, C.c_void_p(q_ptr), nq, k, nprobe,
                                         _RANKING[ranking], survivors, _SELECTION[selection],
                                         C.c_void_p(ids_ptr), C.c_void_p(dists_ptr)))

    def search_device(self, queries, ids, dists, k: int = 10, nprobe: int = 64,
                      ranking: str = "prefix", survivors: int = 32, selection: str = "threshold",
                      stream: int = 0) -> None:
        """CUDA tensors in (nq x dim float32) and out (nq x k uint32/int32,
        float32) on `stream` (a cudaStream_t as int; 0 = the index's stream).
        Asynchronous."""
        nq = int(queries.shape[0])
        _check(_lib.katoann_index_search_device(
            self._h, C.c_void_p(queries.data_ptr()), nq, k, nprobe, _RANKING[ranking], survivors,
            _SELECTION[selection], C.c_void_p(ids.data_ptr()), C.c_void_p(dists.data_ptr()),
            C.c_void_p(stream) if stream else None))

    def search_stats(self) -> dict:
        s = np.zeros(3, np.uint64)
        _check(_lib.katoann_index_stats(self._h, _ptr(s), 3))
        return dict(coarse_boundary_ties=int(s[0]), survivor_boundary_ties=int(s[1]))

    def _info(self):
        info = np.zeros(8, np.uint32)
        _lib.katoann_index_info(self._h, _ptr(info))
        return info

    @property
    def dim(self) -> int:
        return int(self._info()[0])

    @property
    def nlist(self) -> int:
        return int(self._info()[1])

    @property
    def size(self) -> int:
        return int(self._info()[2])

    @property
    def prefix_dims(self) -> int:
        return int(self._info()[3])

    @property
    def rotated(self) -> bool:
        return bool(self._info()[4])

    @property
    def normalized(self) -> bool:
        return bool(self._info()[5])

    @property
    def engine(self) -> str:
        return "gpu"

    @property
    def memory_bytes(self) -> int:
        return int(_lib.katoann_index_memory_bytes(self._h))

    def list_sizes(self) -> np.ndarray:
        out = np.zeros(self.nlist, np.uint32)
        _lib.katoann_index_list_sizes(self._h, _ptr(out))
        return out

    @property
    def device_view(self) -> int:
        """Address of the katoann_gpu_index the kernels read (for direct C ABI calls)."""
        return int(_lib.katoann_index_device_view(self._h) or 0)
