"""ctypes access to libkatoann_gpu.so for the kernel-level GPU tests."""
from __future__ import annotations

import ctypes as C
import os
import platform

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBDIR = os.path.join(ROOT, "katoann-public_gb300", "katoann", "_lib", platform.machine())


class GpuIndex(C.Structure):
    """Mirror of katoann_gpu_index (include/katoann_gpu.h)."""
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


_gpu = None


def gpu():
    global _gpu
    if _gpu is None:
        _gpu = C.CDLL(os.path.join(LIBDIR, "libkatoann_gpu.so"))
        _gpu.katoann_gpu_last_error.restype = C.c_char_p
        _gpu.katoann_gpu_search_workspace.restype = C.c_size_t
        P, U32, I32, D, S = C.c_void_p, C.c_uint32, C.c_int, C.c_double, C.c_size_t
        _gpu.katoann_gpu_rotate_rows.argtypes = [P, U32, U32, P, P, P]
        _gpu.katoann_gpu_quantize_rows.argtypes = [P, U32, U32, U32, C.c_float, D, U32, P, P, P, P, P, P]
        _gpu.katoann_gpu_sq16_l2.argtypes = [P, P, P, P, P, P, D, U32, U32, U32, P, P]
        _gpu.katoann_gpu_sq16_high_l2.argtypes = [P, P, P, P, D, U32, U32, U32, U32, P, P]
        _gpu.katoann_gpu_coarse.argtypes = [P, P, P, P, U32, U32, P, P, P]
        _gpu.katoann_gpu_search_workspace.argtypes = [P, U32, U32, U32, I32, U32]
        _gpu.katoann_gpu_search.argtypes = [P, P, U32, U32, U32, I32, U32, U32, P, S, P, P, P]
        _gpu.katoann_gpu_dist_values.argtypes = [P, U32, D, P, P]
        _gpu.katoann_gpu_workspace_stats.argtypes = [P, P, U32, P]
    return _gpu


def check(rc):
    if rc != 0:
        raise RuntimeError(f"status {rc}: {gpu().katoann_gpu_last_error().decode()}")


def dptr(t) -> C.c_void_p:
    return C.c_void_p(t.data_ptr())


def view_of(index):
    """The katoann_gpu_index of a katoann.Index (host copy of the struct)."""
    return index.view()


def to_host(ptr: int, nbytes: int, dtype) -> np.ndarray:
    import katoann
    return katoann.device_to_host(ptr, nbytes, dtype)
