"""KatoANN's Python module on one GB300.

Mirrors the reference module (python/katoann_module.cpp:34-129): ``build``,
``Index().load(...)``, ``Index.search(...) -> (ids, dists)``, the read-only
properties and ``amx_available``. Searches run as sm_103a kernels through
libkatoann.so / libkatoann_gpu.so (bound here with ctypes, which releases the
GIL during each call, as the reference's module does). There is no CPU
fallback: importing fails loudly when the libraries are missing.

Additions: ``Index.load_arrays`` (an index from numpy arrays or CUDA tensors),
``Index.search_device`` (CUDA tensors in and out, no host copies),
``Index.search_stats``, the device-code cache (``save_codes`` / ``load_codes``)
and the learned per-query probe budget (``ProbeModel``; ``search(...,
budget=model)`` or ``nprobe_per_query=``).
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
    gpu = C.CDLL(os.path.join(_LIBDIR, "libkatoann_gpu.so"), mode=C.RTLD_GLOBAL)
    gpu.katoann_gpu_timer_create.argtypes = [C.c_uint32]
    gpu.katoann_gpu_timer_create.restype = C.c_void_p
    gpu.katoann_gpu_timer_destroy.argtypes = [C.c_void_p]
    gpu.katoann_gpu_timer_read.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
    gpu.katoann_gpu_timer_kernels.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
    gpu.katoann_gpu_timer_kernels.restype = None
    gpu.katoann_gpu_last_error.restype = C.c_char_p
    gpu.katoann_gpu_copy_to_host.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t]
    gpu.katoann_gpu_set_wait_limit.argtypes = [C.c_uint64]
    gpu.katoann_gpu_last_launches.restype = C.c_uint32
    lib = C.CDLL(path)
    lib.gpu = gpu
    P, U32, I32, U64, D, S = C.c_void_p, C.c_uint32, C.c_int, C.c_uint64, C.c_double, C.c_size_t
    lib.katoann_last_error.restype = C.c_char_p
    lib.katoann_build.argtypes = [P, U32, U32, U32, U32, U32, U64, I32, U32, U32, C.c_char_p]
    lib.katoann_build_partition.argtypes = [P, I32, U32, U32, U32, U32, U32, U64, U32, U32, P, P, P,
                                            P, P]
    lib.katoann_index_new.restype = P
    lib.katoann_index_free.argtypes = [P]
    lib.katoann_index_load.argtypes = [P, C.c_char_p, I32, I32, U32, I32, U32]
    lib.katoann_index_load_cached.argtypes = [P, C.c_char_p, U32, U32]
    lib.katoann_index_save_codes.argtypes = [P, C.c_char_p]
    lib.katoann_index_load_codes.argtypes = [P, C.c_char_p, U32]
    lib.katoann_index_load_arrays.argtypes = [P, U32, U32, U32, I32, P, P, P, P, P, I32, U32, I32,
                                              U32, U32]
    lib.katoann_index_search.argtypes = [P, P, U32, U32, U32, I32, U32, I32, P, P]
    lib.katoann_index_search_device.argtypes = [P, P, U32, U32, U32, I32, U32, I32, P, P, P, P]
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
    F = C.c_float
    lib.katoann_index_search_budget.argtypes = [P, P, U32, U32, U32, I32, U32, I32, P, F, P, P, P, P,
                                                I32]
    lib.katoann_index_search_device_budget.argtypes = [P, P, U32, U32, U32, I32, U32, I32, P, F, P,
                                                       P, P, P, P, P, I32]
    lib.katoann_probe_train.argtypes = [P, P, U32, P, U32, U32, U32, U32, I32, U32, I32, U32, U32,
                                        U32, F, F, U64, C.POINTER(P)]
    lib.katoann_probe_fit.argtypes = [P, P, U32, P, U32, U32, U32, U32, F, F, U64, C.POINTER(P)]
    lib.katoann_probe_load.argtypes = [C.c_char_p, C.POINTER(P)]
    lib.katoann_probe_save.argtypes = [P, C.c_char_p]
    lib.katoann_probe_free.argtypes = [P]
    lib.katoann_probe_info.argtypes = [P, P, P, P]
    lib.katoann_probe_record.argtypes = [P, P, P, P, P]
    lib.katoann_probe_weights.argtypes = [P, P, P, P, P, P, P, P, P]
    lib.katoann_probe_features.argtypes = [P, P, U32, U32, P]
    lib.katoann_probe_predict.argtypes = [P, P, U32, F, U32, P, P]
    lib.katoann_server_new.argtypes = [P, U32, U32, U64, U32, U32, I32, U32, P, F, D, I32, P, U32,
                                       C.POINTER(P)]
    lib.katoann_server_free.argtypes = [P]
    lib.katoann_server_submit.argtypes = [P, P, U32, C.POINTER(U64)]
    lib.katoann_server_wait.argtypes = [P, U64, P, P, P, P]
    lib.katoann_server_poll.argtypes = [P, U64, P, P, P, P, P]
    lib.katoann_server_drain.argtypes = [P]
    lib.katoann_server_stats.argtypes = [P, P]
    lib.katoann_server_load.argtypes = [P, P, U32, U32, D, U32, P, U32, U64, P]
    lib.katoann_index_autotune.argtypes = [P, P, U32, U32, U32, I32, U32, P, F, P]
    return lib


_lib = _load()


def last_launches() -> int:
    """Kernel launches of this thread's last search (all its batch passes)."""
    return int(_lib.gpu.katoann_gpu_last_launches())


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


_CUDA_STREAM_LEGACY = 0x1  # cudaStreamLegacy


def _stream_arg(stream):
    if stream is None:
        return None
    return C.c_void_p(int(stream) if int(stream) else _CUDA_STREAM_LEGACY)


def _check(rc: int) -> None:
    if rc == 0:
        return
    msg = _lib.katoann_last_error().decode()
    if rc == -1:
        raise ValueError(msg)
    if rc == -3:
        raise RuntimeError(f"logic error: {msg}")
    if rc == -5:
        raise TimeoutError(msg)
    raise RuntimeError(msg)


def set_wait_limit(cycles: int) -> None:
    """Every pipeline wait of the tensor-core ranking pass gives up after this
    many SM cycles (0: the default, about 2 s); a search in which one gives up
    raises TimeoutError. Process-wide."""
    if _lib.gpu.katoann_gpu_set_wait_limit(int(cycles)) != 0:
        raise ValueError(_lib.gpu.katoann_gpu_last_error().decode())


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


def build_partition(data, nlist: int = 2048, train_size: int = 256000, kmeans_iters: int = 12,
                    seed: int = 0, rotation_sample: int = 100000, jacobi_sweeps: int = 8):
    """The partition build() writes, computed on the GPU without writing
    files: (centroids [nlist, dim] float32, assign [n] uint32, rotation
    [dim, dim] float32 or None, head_dims). `data` is a float32 array or a
    CUDA tensor (then the vectors stay on the device)."""
    on_device = hasattr(data, "is_cuda") and data.is_cuda
    keep = data.contiguous() if on_device else np.ascontiguousarray(data, dtype=np.float32)
    if len(keep.shape) != 2:
        raise ValueError("data must be 2-D")
    n, dim = int(keep.shape[0]), int(keep.shape[1])
    ptr = C.c_void_p(keep.data_ptr()) if on_device else _ptr(keep)
    cen = np.zeros((nlist, dim), np.float32)
    assign = np.zeros(n, np.uint32)
    rot = np.zeros((dim, dim), np.float32)
    rotated, head = C.c_uint32(0), C.c_uint32(0)
    _check(_lib.katoann_build_partition(ptr, int(on_device), n, dim, nlist, train_size, kmeans_iters,
                                        seed, rotation_sample, jacobi_sweeps, _ptr(cen), _ptr(assign),
                                        _ptr(rot), C.byref(rotated), C.byref(head)))
    return cen, assign, (rot if rotated.value else None), int(head.value)


def normalize_rows(x: np.ndarray) -> np.ndarray:
    """Unit-length rows, computed as the reference's module does (double sum)."""
    out = np.array(x, dtype=np.float32, order="C", copy=True)
    _lib.katoann_normalize_rows(_ptr(out), out.shape[0], out.shape[1])
    return out


def dist_value(l2: int, step_sq: float) -> float:
    """float(double(l2) * step_sq), by the integer method of the kernels."""
    return float(_lib.katoann_dist_value(int(l2), float(step_sq)))


PHASES = ("rotate+quantize", "coarse product", "coarse select", "probe budget", "inversion",
          "seed bounds", "ranking pass", "survivor merge", "refine")
TIMED_KERNELS = ("rotation", "coarse_tc_kernel", "rank_tc_kernel")  # the phase timer's kernel events


class PhaseTimer:
    """CUDA events at the phase boundaries of every device search pass
    (katoann_gpu_timer_create); read() returns the summed ms per phase."""

    def __init__(self, max_passes: int):
        self.handle = _lib.gpu.katoann_gpu_timer_create(max_passes)
        if not self.handle:
            raise RuntimeError("cannot create the phase timer")

    def read(self) -> tuple[dict, int]:
        ms = np.zeros(len(PHASES), np.float32)
        n = np.zeros(1, np.uint32)
        rc = _lib.gpu.katoann_gpu_timer_read(C.c_void_p(self.handle), _ptr(ms), _ptr(n))
        if rc:
            raise RuntimeError(_lib.gpu.katoann_gpu_last_error().decode())
        return dict(zip(PHASES, map(float, ms))), int(n[0])

    def kernels(self) -> dict:
        """Summed ms and launch count of the single kernels the timer
        brackets, over the passes of the last read()."""
        ms = np.zeros(len(TIMED_KERNELS), np.float32)
        n = np.zeros(len(TIMED_KERNELS), np.uint32)
        _lib.gpu.katoann_gpu_timer_kernels(C.c_void_p(self.handle), _ptr(ms), _ptr(n))
        return {k: (float(a), int(b)) for k, a, b in zip(TIMED_KERNELS, ms, n)}

    def __del__(self):
        h = getattr(self, "handle", None)
        if h:
            _lib.gpu.katoann_gpu_timer_destroy(C.c_void_p(h))
            self.handle = None


class GpuIndexView(C.Structure):
    """The katoann_gpu_index the kernels read (include/katoann_gpu.h)."""
    _fields_ = [("dim", C.c_uint32), ("dc", C.c_uint32), ("nlist", C.c_uint32), ("npts", C.c_uint32),
                ("head_dims", C.c_uint32), ("rotated", C.c_uint32), ("max_list", C.c_uint32),
                ("reserved", C.c_uint32), ("lo", C.c_float), ("pad", C.c_float),
                ("inv_step", C.c_double), ("step_sq", C.c_double),
                ("d_rotation", C.c_void_p), ("d_hi", C.c_void_p), ("d_lo", C.c_void_p),
                ("d_norm", C.c_void_p), ("d_hinorm", C.c_void_p), ("d_headnorm", C.c_void_p),
                ("d_ids", C.c_void_p), ("d_list_off", C.c_void_p), ("d_chi", C.c_void_p),
                ("d_clo", C.c_void_p), ("d_cnorm", C.c_void_p), ("d_chi16", C.c_void_p),
                ("d_clo16", C.c_void_p), ("d_cterm", C.c_void_p),
                ("d_rotation_t", C.c_void_p)]


def device_to_host(ptr: int, nbytes: int, dtype) -> np.ndarray:
    """Copy nbytes of device memory at ptr into a new host array of dtype."""
    buf = np.empty(nbytes, np.uint8)
    if nbytes:
        rc = _lib.gpu.katoann_gpu_copy_to_host(_ptr(buf), C.c_void_p(ptr), nbytes)
        if rc:
            raise RuntimeError(_lib.gpu.katoann_gpu_last_error().decode())
    return buf.view(dtype)


class Index:
    def __init__(self):
        self._h = _lib.katoann_index_new()

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            _lib.katoann_index_free(h)
            self._h = None

    def load(self, prefix: str, precision: str = "sq16", use_amx: bool = True, prefix_dims: int = 0,
             batched_coarse: bool = True, max_batch: int = 4096, code_cache: bool = False) -> None:
        """The reference's Index.load; code_cache=True goes through PREFIX.gpucodes
        (see save_codes)."""
        if precision not in ("sq16", "bf16"):
            raise ValueError("precision is 'sq16' or 'bf16'")
        if code_cache and precision == "sq16" and batched_coarse:
            _check(_lib.katoann_index_load_cached(self._h, prefix.encode(), prefix_dims, max_batch))
            return
        _check(_lib.katoann_index_load(self._h, prefix.encode(), 1 if precision == "bf16" else 0,
                                       int(use_amx), prefix_dims, int(batched_coarse), max_batch))

    def save_codes(self, path: str) -> None:
        """The loaded index as it lives on the device, to one file (the
        device-code cache; no counterpart in the reference)."""
        _check(_lib.katoann_index_save_codes(self._h, path.encode()))

    def load_codes(self, path: str, max_batch: int = 4096) -> None:
        """An index from a file written by save_codes: no float vectors are read
        and nothing is re-coded."""
        _check(_lib.katoann_index_load_codes(self._h, path.encode(), max_batch))

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
               survivors: int = 32, selection: str = "threshold", budget: "ProbeModel | None" = None,
               threshold: float = 0.95, nprobe_per_query=None, return_nprobe: bool = False,
               graph: bool = False):
        """Search all queries together; returns (ids uint32 [nq, k], squared
        L2 distances float32 [nq, k]), nearest first. Queries are normalized
        when the index was built with normalized=True. graph=True replays the
        kernels of each pass as a captured CUDA graph (SearchParams::graph).

        Additions: a per-query nprobe, capped at `nprobe`: given
        (nprobe_per_query, nq values) or chosen by a ProbeModel (`budget`, at
        cumulative probability `threshold`). return_nprobe=True also returns
        every query's nprobe (uint32 [nq])."""
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
        if budget is None and nprobe_per_query is None and not return_nprobe and not graph:
            _check(_lib.katoann_index_search(self._h, _ptr(q), nq, k, nprobe, _RANKING[ranking],
                                             survivors, _SELECTION[selection], _ptr(ids),
                                             _ptr(dists)))
            return ids, dists
        npq = None
        if nprobe_per_query is not None:
            npq = np.ascontiguousarray(nprobe_per_query, dtype=np.uint32)
            if npq.shape != (nq,):
                raise ValueError("nprobe_per_query needs one value per query")
        used = np.zeros(nq, np.uint32)
        _check(_lib.katoann_index_search_budget(
            self._h, _ptr(q), nq, k, nprobe, _RANKING[ranking], survivors, _SELECTION[selection],
            budget._h if budget is not None else None, float(threshold),
            _ptr(npq) if npq is not None else None, _ptr(used), _ptr(ids), _ptr(dists), int(graph)))
        return (ids, dists, used) if return_nprobe else (ids, dists)

    def search_into(self, q_ptr: int, nq: int, ids_ptr: int, dists_ptr: int, k: int = 10,
                    nprobe: int = 64, ranking: str = "prefix", survivors: int = 32,
                    selection: str = "threshold", budget: "ProbeModel | None" = None,
                    threshold: float = 0.95, nprobe_out_ptr: int = 0, graph: bool = False) -> None:
        """search() on raw host pointers (e.g. pinned buffers); no normalisation.
        graph=True replays each pass's kernels as a captured CUDA graph."""
        if budget is None and not nprobe_out_ptr and not graph:
            _check(_lib.katoann_index_search(self._h, C.c_void_p(q_ptr), nq, k, nprobe,
                                             _RANKING[ranking], survivors, _SELECTION[selection],
                                             C.c_void_p(ids_ptr), C.c_void_p(dists_ptr)))
            return
        _check(_lib.katoann_index_search_budget(
            self._h, C.c_void_p(q_ptr), nq, k, nprobe, _RANKING[ranking], survivors,
            _SELECTION[selection], budget._h if budget is not None else None, float(threshold),
            None, C.c_void_p(nprobe_out_ptr) if nprobe_out_ptr else None, C.c_void_p(ids_ptr),
            C.c_void_p(dists_ptr), int(graph)))

    def search_device(self, queries, ids, dists, k: int = 10, nprobe: int = 64,
                      ranking: str = "prefix", survivors: int = 32, selection: str = "threshold",
                      stream: int | None = None, timer: "PhaseTimer | None" = None,
                      budget: "ProbeModel | None" = None, threshold: float = 0.95,
                      nprobe_per_query=None, nprobe_out=None, graph: bool = False) -> None:
        """CUDA tensors in (nq x dim float32) and out (nq x k uint32/int32,
        float32) on `stream` (a cudaStream_t as int, e.g. torch's
        ``Stream.cuda_stream``; 0 is the legacy default stream; None = the
        index's own stream). Asynchronous. nprobe_per_query / nprobe_out are
        CUDA int32 tensors of nq values. graph=True replays a CUDA graph of the
        call, captured the first time these tensors and parameters are seen."""
        nq = int(queries.shape[0])
        tm = C.c_void_p(timer.handle) if timer else None
        if budget is None and nprobe_per_query is None and nprobe_out is None and not graph:
            _check(_lib.katoann_index_search_device(
                self._h, C.c_void_p(queries.data_ptr()), nq, k, nprobe, _RANKING[ranking],
                survivors, _SELECTION[selection], C.c_void_p(ids.data_ptr()),
                C.c_void_p(dists.data_ptr()), _stream_arg(stream), tm))
            return
        _check(_lib.katoann_index_search_device_budget(
            self._h, C.c_void_p(queries.data_ptr()), nq, k, nprobe, _RANKING[ranking], survivors,
            _SELECTION[selection], budget._h if budget is not None else None, float(threshold),
            C.c_void_p(nprobe_per_query.data_ptr()) if nprobe_per_query is not None else None,
            C.c_void_p(nprobe_out.data_ptr()) if nprobe_out is not None else None,
            C.c_void_p(ids.data_ptr()), C.c_void_p(dists.data_ptr()), _stream_arg(stream), tm,
            int(graph)))

    def autotune(self, queries, k: int = 10, nprobe: int = 64, ranking: str = "prefix",
                 survivors: int = 32, budget: "ProbeModel | None" = None,
                 threshold: float = 0.95) -> dict:
        """Times a search of these queries under every candidate setting of the
        ranking pass's knobs (seed rows, CTA split weight, item width) and
        keeps the fastest for the process; results never depend on them."""
        q = np.ascontiguousarray(queries, dtype=np.float32)
        if q.ndim != 2 or q.shape[1] != self.dim:
            raise ValueError("queries must be (n, dim) float32")
        if self.normalized:
            q = normalize_rows(q)
        out = np.zeros(4, np.uint32)
        _check(_lib.katoann_index_autotune(self._h, _ptr(q), q.shape[0], k, nprobe,
                                           _RANKING[ranking], survivors,
                                           budget._h if budget is not None else None,
                                           float(threshold), _ptr(out)))
        return dict(seed_rows=int(out[0]), schedule=int(out[1]), width=int(out[2]),
                    us_per_search=int(out[3]))

    def search_stats(self) -> dict:
        """Diagnostics of the last search (see katoann_gpu_workspace_stats)."""
        s = np.zeros(48, np.uint64)
        _check(_lib.katoann_index_stats(self._h, _ptr(s), 48))
        return dict(coarse_boundary_ties=int(s[0]), survivor_boundary_ties=int(s[1]),
                    ranking_timeouts=int(s[3]), ranking_tiles=int(s[4]),
                    ranking_candidates=int(s[5]), ranking_rescans=int(s[6]),
                    ranking_max_candidates=int(s[7]), ranking_cta_max_cycles=int(s[31]),
                    ranking_role_cycles=dict(zip(
                        ("conv_wait_raw", "conv_wait_a", "conv_total", "mma_wait_b", "mma_wait_acc",
                         "mma_wait_a", "mma_total", "epi_wait_b", "epi_wait_acc", "epi_total",
                         "tma_wait_stage", "tma_total", "stage_wait_b", "stage_total",
                         "mma_issue"), (int(v) for v in s[16:31]))),
                    coarse_role_cycles=dict(zip(
                        ("tma_wait", "tma_total", "mma_wait_acc", "mma_wait_stage", "mma_total",
                         "epi_wait", "epi_total"), (int(v) for v in s[32:39]))),
                    ranking_tiles_by_queries=dict(zip(
                        ("1-2", "3-4", "5-8", "9-16", "17-32", "33-64"), (int(v) for v in s[40:46]))),
                    lists_probed=int(s[46]), probed_rows=int(s[47]))

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

    def view(self) -> GpuIndexView:
        return GpuIndexView.from_address(self.device_view)

    def export_codes(self) -> dict:
        """Host copies of the device-resident index: info (dim, nlist, npts, dc,
        head_dims, rotated), scale (lo, inv_step, step, step_sq), rotation,
        list offsets, ids, code planes (rows x dc) and norms, centroid planes."""
        v = self.view()
        n, dc, L, dim = v.npts, v.dc, v.nlist, v.dim
        h = lambda ptr, nb, dt: device_to_host(ptr, nb, dt)
        return {
            "info": np.array([dim, L, n, dc, v.head_dims, v.rotated], np.uint32),
            "scale": np.array([v.lo, v.inv_step, np.sqrt(v.step_sq), v.step_sq], np.float64),
            "rotation": h(v.d_rotation, dim * dim * 4, np.float32).reshape(dim, dim) if v.rotated else None,
            "list_off": h(v.d_list_off, (L + 1) * 4, np.uint32),
            "ids": h(v.d_ids, n * 4, np.uint32),
            "hi": h(v.d_hi, n * dc, np.uint8).reshape(n, dc),
            "lo": h(v.d_lo, n * dc, np.uint8).reshape(n, dc),
            "norm": h(v.d_norm, n * 8, np.int64), "hinorm": h(v.d_hinorm, n * 8, np.int64),
            "headnorm": h(v.d_headnorm, n * 8, np.int64) if v.head_dims else None,
            "chi": h(v.d_chi, L * dc, np.uint8).reshape(L, dc),
            "clo": h(v.d_clo, L * dc, np.uint8).reshape(L, dc),
            "cnorm": h(v.d_cnorm, L * 8, np.int64),
        }


class ProbeModel:
    """Learned per-query probe budget (include/katoann/probe.h): a
    64 -> 256 -> 256 -> C MLP with bf16 weights over 64 features of a query's
    sorted coarse distances, choosing nprobe from a ladder. Use it as
    ``index.search(q, nprobe=cap, budget=model, threshold=t)``."""

    LADDER = (8, 12, 16, 24, 32, 48, 64, 96, 128, 192, 256, 384, 512)

    def __init__(self, handle):
        self._h = handle

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            _lib.katoann_probe_free(h)
            self._h = None

    @classmethod
    def train(cls, index: Index, queries, ladder=LADDER, depth: int = 256, k: int = 10,
              label_nprobe: int = 0, label_ranking: str = "full", label_survivors: int = 0,
              ranking: str = "prefix", survivors: int = 64, epochs: int = 24, batch: int = 1024,
              lr: float = 1e-3, weight_decay: float = 1e-4, seed: int = 0) -> "ProbeModel":
        """Labels the training queries by searching `index` (the smallest
        ladder value whose fixed-nprobe search recovers as much of the exact
        top-k as any ladder value does; the exact top-k comes from the
        label_ranking search at label_nprobe lists, by default the exact-
        distance one) and trains the model on the device."""
        q = np.ascontiguousarray(queries, dtype=np.float32)
        if q.ndim != 2 or q.shape[1] != index.dim:
            raise ValueError("queries must be (n, dim) float32")
        if index.normalized:
            q = normalize_rows(q)
        lad = np.ascontiguousarray(ladder, dtype=np.uint32)
        h = C.c_void_p()
        _check(_lib.katoann_probe_train(index._h, _ptr(q), q.shape[0], _ptr(lad), lad.size, depth,
                                        k, label_nprobe, _RANKING[label_ranking], label_survivors,
                                        _RANKING[ranking], survivors, epochs, batch, lr,
                                        weight_decay, seed, C.byref(h)))
        return cls(h.value)

    @classmethod
    def fit(cls, z, labels, ladder=LADDER, depth: int = 256, epochs: int = 24, batch: int = 1024,
            lr: float = 1e-3, weight_decay: float = 1e-4, seed: int = 0) -> "ProbeModel":
        """Trains on raw features (n x 64, from features()) and class labels."""
        z = np.ascontiguousarray(z, dtype=np.float32)
        y = np.ascontiguousarray(labels, dtype=np.uint8)
        if z.ndim != 2 or z.shape[1] != 64 or y.shape != (z.shape[0],):
            raise ValueError("features must be (n, 64) with n labels")
        lad = np.ascontiguousarray(ladder, dtype=np.uint32)
        h = C.c_void_p()
        _check(_lib.katoann_probe_fit(_ptr(z), _ptr(y), z.shape[0], _ptr(lad), lad.size, depth,
                                      epochs, batch, lr, weight_decay, seed, C.byref(h)))
        return cls(h.value)

    @classmethod
    def load(cls, path: str) -> "ProbeModel":
        h = C.c_void_p()
        _check(_lib.katoann_probe_load(path.encode(), C.byref(h)))
        return cls(h.value)

    def save(self, path: str) -> None:
        _check(_lib.katoann_probe_save(self._h, path.encode()))

    def _info(self):
        info = np.zeros(2, np.uint32)
        _check(_lib.katoann_probe_info(self._h, _ptr(info), None, None))
        return info

    @property
    def classes(self) -> int:
        return int(self._info()[0])

    @property
    def depth(self) -> int:
        return int(self._info()[1])

    @property
    def ladder(self) -> np.ndarray:
        lad = np.zeros(self.classes, np.uint32)
        _check(_lib.katoann_probe_info(self._h, _ptr(np.zeros(2, np.uint32)), _ptr(lad), None))
        return lad

    @property
    def feature_ranks(self) -> np.ndarray:
        r = np.zeros(64, np.uint32)
        _check(_lib.katoann_probe_info(self._h, _ptr(np.zeros(2, np.uint32)), None, _ptr(r)))
        return r

    @property
    def labels(self) -> np.ndarray:
        n = np.zeros(1, np.uint32)
        _check(_lib.katoann_probe_record(self._h, None, _ptr(n), None, None))
        out = np.zeros(int(n[0]), np.uint8)
        _check(_lib.katoann_probe_record(self._h, _ptr(out), None, None, None))
        return out

    @property
    def loss(self) -> np.ndarray:
        e = np.zeros(1, np.uint32)
        _check(_lib.katoann_probe_record(self._h, None, None, None, _ptr(e)))
        out = np.zeros(int(e[0]), np.float32)
        _check(_lib.katoann_probe_record(self._h, None, None, _ptr(out), None))
        return out

    def weights(self) -> dict:
        """The weights as the device uses them (bf16 as uint16 bit patterns)."""
        c = self.classes
        w = dict(shift=np.zeros(64, np.float32), scale=np.zeros(64, np.float32),
                 w1=np.zeros((64, 256), np.uint16), b1=np.zeros(256, np.float32),
                 w2=np.zeros((256, 256), np.uint16), b2=np.zeros(256, np.float32),
                 w3=np.zeros((256, c), np.uint16), b3=np.zeros(c, np.float32))
        _check(_lib.katoann_probe_weights(self._h, *(_ptr(w[n]) for n in
                                                     ("shift", "scale", "w1", "b1", "w2", "b2",
                                                      "w3", "b3"))))
        return w

    @staticmethod
    def features(index: Index, queries, depth: int = 256) -> np.ndarray:
        """The 64 raw features of each query (n x 64) at `depth`."""
        q = np.ascontiguousarray(queries, dtype=np.float32)
        if index.normalized:
            q = normalize_rows(q)
        z = np.zeros((q.shape[0], 64), np.float32)
        _check(_lib.katoann_probe_features(index._h, _ptr(q), q.shape[0], depth, _ptr(z)))
        return z

    def predict(self, z, threshold: float = 0.95, cap: int = 4096):
        """Class probabilities (n x classes) and budgets (n, capped at cap) of
        raw feature rows."""
        z = np.ascontiguousarray(z, dtype=np.float32)
        n = z.shape[0]
        probs = np.zeros((n, self.classes), np.float32)
        nprobe = np.zeros(n, np.uint32)
        _check(_lib.katoann_probe_predict(self._h, _ptr(z), n, threshold, cap, _ptr(probs),
                                          _ptr(nprobe)))
        return probs, nprobe


class Server:
    """Continuous-batching search server (include/katoann/server.h): requests
    with their own k are batched on arrival, several batches run on the
    device at once within an HBM budget, and every result equals the search
    of that query alone. ``submit`` returns an id; ``wait`` returns
    (ids, dists, nprobe, latency_ms)."""

    def __init__(self, index: Index, max_batch: int = 4096, max_in_flight: int = 3,
                 hbm_budget: int = 0, max_k: int = 128, nprobe: int = 64,
                 ranking: str = "prefix", survivors: int = 32,
                 budget: "ProbeModel | None" = None, threshold: float = 0.95,
                 max_wait_ms: float = 0.0, graphs: bool = True, warm_k=()):
        self._index = index  # the server reads the index's device arrays
        self._budget = budget
        self.dim = index.dim
        self.normalized = index.normalized
        self._k = {}
        h = C.c_void_p()
        warm = np.ascontiguousarray(warm_k, dtype=np.uint32)
        _check(_lib.katoann_server_new(index._h, max_batch, max_in_flight, hbm_budget, max_k,
                                       nprobe, _RANKING[ranking], survivors,
                                       budget._h if budget is not None else None, threshold,
                                       max_wait_ms, int(graphs), _ptr(warm) if warm.size else None,
                                       warm.size, C.byref(h)))
        self._h = h.value

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            _lib.katoann_server_free(h)
            self._h = None

    def submit(self, query, k: int = 10) -> int:
        q = np.ascontiguousarray(query, dtype=np.float32).reshape(1, -1)
        if q.shape[1] != self.dim:
            raise ValueError("query must have dim floats")
        if self.normalized:
            q = normalize_rows(q)
        rid = C.c_uint64()
        _check(_lib.katoann_server_submit(self._h, _ptr(q), k, C.byref(rid)))
        self._k[rid.value] = k
        return rid.value

    def wait(self, rid: int):
        k = self._k.pop(rid)
        ids = np.zeros(k, np.uint32)
        dists = np.zeros(k, np.float32)
        npb = np.zeros(1, np.uint32)
        lat = np.zeros(1, np.float64)
        _check(_lib.katoann_server_wait(self._h, rid, _ptr(ids), _ptr(dists), _ptr(npb),
                                        _ptr(lat)))
        return ids, dists, int(npb[0]), float(lat[0])

    def drain(self) -> None:
        _check(_lib.katoann_server_drain(self._h))

    def load(self, queries, rate: float, requests: int, kmix=(10,), seed: int = 42) -> dict:
        """A Poisson stream of `requests` arrivals at `rate` per second from a
        native client (queries round-robin, k uniform over kmix); latency
        from the scheduled arrival to completion."""
        q = np.ascontiguousarray(queries, dtype=np.float32)
        if q.ndim != 2 or q.shape[1] != self.dim:
            raise ValueError("queries must be (n, dim) float32")
        if self.normalized:
            q = normalize_rows(q)
        ks = np.ascontiguousarray(kmix, dtype=np.uint32)
        r = np.zeros(13, np.float64)
        _check(_lib.katoann_server_load(self._h, _ptr(q), q.shape[0], q.shape[1], float(rate),
                                        requests, _ptr(ks), ks.size, seed, _ptr(r)))
        keys = ("achieved_qps", "p50_ms", "p95_ms", "p99_ms", "max_ms", "batches", "mean_batch",
                "mean_nprobe", "peak_in_flight", "peak_hbm_bytes", "max_lag_ms",
                "max_enqueue_ms", "max_batch_gpu_ms")
        out = dict(zip(keys, map(float, r)))
        for key in ("batches", "peak_in_flight", "peak_hbm_bytes"):
            out[key] = int(out[key])
        return out

    def stats(self) -> dict:
        s = np.zeros(9, np.uint64)
        _check(_lib.katoann_server_stats(self._h, _ptr(s)))
        return dict(requests=int(s[0]), batches=int(s[1]), peak_in_flight=int(s[2]),
                    peak_hbm_bytes=int(s[3]), mean_batch=float(s[4]) / 1000.0,
                    max_enqueue_ms=float(s[5]) / 1000.0, max_batch_gpu_ms=float(s[6]) / 1000.0,
                    graph_batches=int(s[7]), graphs=int(s[8]))
