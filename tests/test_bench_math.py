"""The arithmetic behind bench.py's roofline: the algorithmic work of each
search phase for one launch (pure functions, no GPU)."""
import pytest

import bench

B, L, DC, D, P, S, H = 4096, 16384, 1024, 1024, 72, 64, 256


def test_ranking_pass_counts_each_probed_row_once():
    rows = 8_880_000
    bound, work, unit = bench.phase_work("ranking pass", B, L, DC, D, P, S, H, rows, rows)
    assert (bound, unit) == ("hbm", "GB/s")
    assert work == pytest.approx(rows * H / 1e9)  # h bytes per row: 2.27 GB at the bench's size


def test_coarse_product_is_four_tensor_gemms():
    bound, work, unit = bench.phase_work("coarse product", B, L, DC, D, P, S, H, 0, 0)
    assert (bound, unit) == ("tensor", "TFLOP/s")
    assert work == pytest.approx(8 * B * L * DC / 1e12)  # 550 GFLOP per batch


def test_other_phases():
    assert bench.phase_work("refine", B, L, DC, D, P, S, H, 0, 0)[1] == pytest.approx(
        B * S * (2 * DC + 12) / 1e9)
    assert bench.phase_work("coarse select", B, L, DC, D, P, S, H, 0, 0)[1] == pytest.approx(
        B * L * 4 / 1e9)
    # 2,048 sketched rows of 32 bytes and 3S = 192 rows of 256 bytes per query
    assert bench.phase_work("seed bounds", B, L, DC, D, P, S, H, 0, 0)[1] == pytest.approx(
        B * (2048 * 32 + 3 * S * H) / 1e9)
    assert bench.seed_bytes(B, 128, S, H) == B * 128 * H  # few rows: all in full


def test_traffic_per_tile_is_the_capture():
    # 2,654.7 MB over 96,108 tiles in the 10M x 1024 capture: 27.6 KB per tile
    assert bench.RANK_TC_DRAM_BYTES_PER_TILE == pytest.approx(2654.7e6 / 96108)
    assert 27_000 < bench.RANK_TC_DRAM_BYTES_PER_TILE < 28_000


def test_workloads_and_metric_names():
    """The four workloads the bench runs, and the metric names of their lines."""
    w = bench.WORKLOADS
    assert (w["learned"]["n"], w["learned"]["dim"], w["learned"]["nlist"]) == (10_000_000, 1024, 16384)
    assert (w["small"]["n"], w["small"]["dim"], w["small"]["nlist"], w["small"]["batch"]) == (100_000, 128, 256, 1024)
    assert (w["plain"]["n"], w["plain"]["dim"], w["plain"]["nlist"]) == (1_000_000, 1024, 4096)
    assert (w["wide"]["n"], w["wide"]["dim"], w["wide"]["head"]) == (990_000, 3072, 256)
    # prefix dims are multiples of 64 within the padded dimension (src/index.cpp:695-696)
    assert all(x["head"] % 64 == 0 and x["head"] <= (x["dim"] + 63) // 64 * 64 for x in w.values())
    assert bench.metric_name("learned", 10_000_000, 1024, 4096) == \
        "QPS at recall@10 >= 0.99, 10M x 1024 IVF, learned vs fixed nprobe, batch 4096, 1 GB300"
    assert bench.metric_name("wide", 990_000, 3072, 4096) == \
        "QPS at recall@10 >= 0.99, 990k x 3072 IVF, fixed nprobe, batch 4096, 1 GB300"


def test_fixed_grid_rows_ascend():
    """Both arms sweep the same settings; within a survivors value nprobe
    ascends (the reference arm stops a row at its first point at the target)."""
    g = bench.fixed_grid(16384)
    for s in {x[1] for x in g}:
        row = [p for p, t in g if t == s]
        assert row == sorted(row) and len(row) == len(set(row))
    assert all(p <= 256 for p, _ in bench.fixed_grid(256))


def test_rotation_is_fp32_fma_work():
    bound, work, unit = bench.phase_work("rotate+quantize", B, L, DC, D, P, S, H, 0, 0)
    assert (bound, unit) == ("fp32", "TFMA/s") and work == pytest.approx(B * D * D / 1e12)
    assert bench.FP32_TFMA_NOMINAL == pytest.approx(40.27, abs=0.01)
