"""CPU checks of the drop-in boundary: the libraries load and export every
entry point the headers declare; host-side validation and the exact distance
conversion behave as the reference does. No GPU is touched."""
import ctypes as C
import os
import platform
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBDIR = os.path.join(ROOT, "katoann-public_gb300", "katoann", "_lib", platform.machine())


def _declared(header: str) -> list[str]:
    text = open(os.path.join(ROOT, "include", header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(katoann_[a-z0-9_]+)\s*\(", text)))


@pytest.mark.parametrize("header,lib", [("katoann_gpu.h", "libkatoann_gpu.so"),
                                        ("katoann_c.h", "libkatoann.so")])
def test_library_exports_every_declared_symbol(header, lib):
    path = os.path.join(LIBDIR, lib)
    assert os.path.exists(path), f"{path} missing: run __graft_entry__.build()"
    if lib == "libkatoann.so":
        C.CDLL(os.path.join(LIBDIR, "libkatoann_gpu.so"), mode=C.RTLD_GLOBAL)
    so = C.CDLL(path)
    names = _declared(header)
    assert len(names) >= 8
    missing = [n for n in names if not hasattr(so, n)]
    assert not missing, missing


def test_dist_value_matches_double_path():
    import katoann
    rng = np.random.default_rng(5)
    for step_sq in (1.76061467e-08, 1.0 / (65535.0 * 65535.0), 2.98203776e-09, 0.37):
        l2 = rng.integers(0, 1 << 44, 20000, dtype=np.int64)
        l2[:50] = np.arange(50)
        got = np.array([katoann.dist_value(int(v), step_sq) for v in l2], np.float32)
        want = (l2.astype(np.float64) * step_sq).astype(np.float32)
        assert np.array_equal(got, want)


def test_search_before_load_is_a_logic_error():
    import katoann
    idx = katoann.Index()
    # The module rejects a query width that differs from the index dimension
    # (python/katoann_module.cpp:81-82); an empty-width batch reaches Index::search.
    with pytest.raises(ValueError, match="queries must be"):
        idx.search(np.zeros((1, 4), np.float32))
    with pytest.raises(RuntimeError, match="search before load"):
        idx.search(np.zeros((1, 0), np.float32))


def test_missing_files_raise_runtime_error(tmp_path):
    import katoann
    idx = katoann.Index()
    with pytest.raises(RuntimeError, match="cannot open"):
        idx.load(str(tmp_path / "nothing"))


def test_truncated_invlist_raises(tmp_path):
    import katoann
    prefix = str(tmp_path / "bad")
    np.array([8, 2, 10, 0, 0], np.uint32).tofile(prefix + ".meta")
    np.zeros((2, 8), np.float32).tofile(prefix + ".centroids")
    with open(prefix + ".invlist", "wb") as f:
        np.array([3], np.uint32).tofile(f)
        np.arange(3, dtype=np.uint32).tofile(f)
        np.zeros((3, 8), np.float32).tofile(f)
    with pytest.raises(RuntimeError, match="truncated"):
        katoann.Index().load(prefix)


def test_bad_meta_header_raises(tmp_path):
    import katoann
    prefix = str(tmp_path / "bad")
    np.array([0, 2, 10, 0, 0], np.uint32).tofile(prefix + ".meta")
    with pytest.raises(RuntimeError, match="bad header"):
        katoann.Index().load(prefix)


def test_bf16_precision_and_flat_coarse_are_refused(tmp_path):
    """Both are comparison modes of the reference outside the GPU search path;
    the files are read first, as the reference does (src/index.cpp:777-786)."""
    import katoann
    import synth
    prefix = str(tmp_path / "x")
    synth.materialize(dict(seed=1, n=200, dim=16, ncomp=3, nlist=4, nq=2, rotation="none"), prefix)
    with pytest.raises(ValueError, match="bf16"):
        katoann.Index().load(prefix, precision="bf16")
    with pytest.raises(ValueError, match="coarse"):
        katoann.Index().load(prefix, batched_coarse=False)


def test_candidate_cap_range_is_checked():
    from _gpu import gpu
    lib = gpu()
    assert lib.katoann_gpu_set_candidate_cap(8) == -1
    assert lib.katoann_gpu_set_candidate_cap(1 << 21) == -1
    assert b"candidate buffer" in lib.katoann_gpu_last_error()
    assert lib.katoann_gpu_set_candidate_cap(32768) == 0


def test_seed_rows_range_is_checked():
    from _gpu import gpu
    lib = gpu()
    assert lib.katoann_gpu_set_seed_rows(5000) == -1
    assert b"seed rows" in lib.katoann_gpu_last_error()
    assert lib.katoann_gpu_set_seed_rows(0) == 0
