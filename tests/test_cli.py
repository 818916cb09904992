"""The katoann command-line tool (tools/katoann.cpp of the reference): the same
commands, flags, JSON lines and exit codes. build, search and load need the
GPU."""
import json
import os
import platform
import subprocess

import numpy as np
import pytest

import oracle
import synth

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CLI = os.path.join(ROOT, "katoann-public_gb300", "katoann", "_lib", platform.machine(), "katoann")


def run(*args, check=True):
    p = subprocess.run([CLI, *args], capture_output=True, text=True, timeout=600)
    if check and p.returncode:
        raise AssertionError(f"katoann {' '.join(args)} -> {p.returncode}\n{p.stderr}")
    return p


def json_lines(text):
    return [json.loads(line) for line in text.splitlines() if line.startswith("{")]


def write_fbin(path, rows):
    rows = np.ascontiguousarray(rows, np.float32)
    with open(path, "wb") as f:
        np.array(rows.shape, np.uint32).tofile(f)
        rows.tofile(f)


def write_gt(path, ids):
    with open(path, "wb") as f:
        np.array(ids.shape, np.uint32).tofile(f)
        np.ascontiguousarray(ids, np.uint32).tofile(f)


def read_out(path):
    with open(path, "rb") as f:
        n, k = np.fromfile(f, np.uint32, 2)
        ids = np.fromfile(f, np.uint32, n * k).reshape(n, k)
        dists = np.fromfile(f, np.float32, n * k).reshape(n, k)
    return ids, dists


def test_usage_and_argument_errors():
    assert run(check=False).returncode == 2
    assert run("nonsense", check=False).returncode == 2
    p = run("search", "--queries", "q.fbin", check=False)
    assert p.returncode == 1 and "katoann: missing --index" in p.stderr
    p = run("search", "stray", check=False)
    assert p.returncode == 1 and "unexpected argument stray" in p.stderr
    p = run("build", "--data", check=False)
    assert p.returncode == 1 and "missing value for --data" in p.stderr
    p = run("search", "--index", "/nonexistent/x", "--queries", "q.fbin", check=False)
    assert p.returncode == 1 and "katoann:" in p.stderr


@pytest.mark.gpu
def test_build_writes_an_index_the_oracle_loads(tmp_path):
    """build partitions on the GPU and writes the reference's file format."""
    xi = synth.mixture_ints(5, 10, 3000, 48, 10)
    data = synth.to_f32(xi)
    write_fbin(tmp_path / "base.fbin", data)
    prefix = str(tmp_path / "idx")
    p = run("build", "--data", str(tmp_path / "base.fbin"), "--out", prefix, "--nlist", "24",
            "--iters", "4", "--seed", "3", "--threads", "4", "--normalize")
    line = json_lines(p.stdout)[-1]
    assert (line["vectors"], line["dim"], line["nlist"]) == (3000, 48, 24) and "build_s" in line
    ref = oracle.OracleIndex(prefix)
    assert (ref.dim, ref.nlist, ref.npts) == (48, 24, 3000)
    assert ref.list_offsets()[-1] == 3000


@pytest.mark.gpu
def test_search_outputs_match_the_oracle(tmp_path):
    spec = dict(seed=31, n=6000, dim=96, ncomp=12, nlist=40, nq=300, rotation="random")
    prefix = str(tmp_path / "x")
    queries, _ = synth.materialize(spec, prefix)
    write_fbin(tmp_path / "q.fbin", queries)
    ref = oracle.OracleIndex(prefix)
    gt, _ = ref.search(queries, k=10, nprobe=40, ranking="full", survivors=10)
    write_gt(tmp_path / "gt.bin", gt)
    with open(tmp_path / "qids.txt", "w") as f:
        f.write(" ".join(str(i) for i in range(0, 300, 2)))
    p = run("search", "--index", prefix, "--queries", str(tmp_path / "q.fbin"), "--gt",
            str(tmp_path / "gt.bin"), "--nprobe", "4,12", "--survivors", "32", "--batch", "64",
            "--repeat", "2", "--query-ids", str(tmp_path / "qids.txt"), "--out",
            str(tmp_path / "res"))
    head, *lines = json_lines(p.stdout)
    assert head["engine"] == "gpu" and head["queries"] == 150 and head["prefix_dims"] == 64
    assert [x["nprobe"] for x in lines] == [4, 12]
    sel = queries[::2]
    for x in lines:
        assert {"qps", "seconds_median", "seconds_min", "seconds_max", "recall"} <= x.keys()
        ids, dists = read_out(str(tmp_path / "res") + f".np{x['nprobe']}.bin")
        rid, rd = ref.search(sel, k=10, nprobe=x["nprobe"], ranking="prefix", survivors=32)
        assert np.array_equal(ids, rid) and np.array_equal(dists, rd)
        hits = sum(len(set(a) & set(b)) for a, b in zip(ids, gt[::2]))
        assert x["recall"] == pytest.approx(hits / ids.size, abs=1e-5)


@pytest.mark.gpu
def test_load_serves_poisson_requests(tmp_path):
    spec = dict(seed=32, n=4000, dim=64, ncomp=8, nlist=32, nq=200, rotation="none")
    prefix = str(tmp_path / "x")
    queries, _ = synth.materialize(spec, prefix)
    write_fbin(tmp_path / "q.fbin", queries)
    p = run("load", "--index", prefix, "--queries", str(tmp_path / "q.fbin"), "--rate", "20000",
            "--requests", "3000", "--nprobe", "8", "--max-batch", "256")
    x = json_lines(p.stdout)[-1]
    assert x["requests"] == 3000 and x["engine"] == "gpu" and x["nprobe"] == 8
    assert 0 < x["p50_ms"] <= x["p95_ms"] <= x["p99_ms"] <= x["max_ms"]
    assert x["batches"] >= 3000 / 256 and 1 <= x["mean_batch"] <= 256


@pytest.mark.gpu
def test_load_serves_mixed_k_with_a_learned_budget(tmp_path):
    import katoann
    spec = dict(seed=33, n=6000, dim=64, ncomp=8, nlist=48, nq=300, rotation="random")
    prefix = str(tmp_path / "x")
    queries, _ = synth.materialize(spec, prefix)
    write_fbin(tmp_path / "q.fbin", queries)
    idx = katoann.Index()
    idx.load(prefix)
    write_fbin(tmp_path / "train.fbin", synth.to_f32(synth.mixture_ints(33, 30, 1500, 64, 8)))
    b = run("budget", "--index", prefix, "--queries", str(tmp_path / "train.fbin"), "--out",
            str(tmp_path / "m.kprb"), "--ladder", "2,4,8,16,32", "--depth", "32",
            "--label-nprobe", "48", "--survivors", "32", "--epochs", "5", "--train-batch", "256")
    info = json_lines(b.stdout)[-1]
    assert info["queries"] == 1500 and info["classes"] == 5 and sum(info["label_histogram"]) == 1500
    model = katoann.ProbeModel.load(str(tmp_path / "m.kprb"))
    assert list(model.ladder) == [2, 4, 8, 16, 32] and model.depth == 32
    p = run("load", "--index", prefix, "--queries", str(tmp_path / "q.fbin"), "--rate", "20000",
            "--requests", "2000", "--nprobe", "32", "--k-mix", "10,100", "--in-flight", "2",
            "--budget", str(tmp_path / "m.kprb"), "--threshold", "0.9")
    x = json_lines(p.stdout)[-1]
    assert x["requests"] == 2000 and x["learned"] is True and x["in_flight"] == 2
    assert 0 < x["p50_ms"] <= x["p99_ms"] and 1 <= x["mean_nprobe"] <= 32
    # where the time went: every batch took device time; the client and the
    # enqueue stay below the slowest request
    assert 0 < x["max_batch_gpu_ms"] <= x["max_ms"] and 0 < x["max_enqueue_ms"]
    assert 0 <= x["max_lag_ms"] <= x["max_ms"]
