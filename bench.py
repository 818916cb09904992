#!/usr/bin/env python3
"""QPS of KatoANN's batched IVF search on GB300 at recall@10 >= 0.99 / 0.999.

Workload: 10,000,000 x 1,024 unit vectors (seeded synthetic stand-in for the
reference's BioASQ-1024-10M: power-law spectrum i^-1.2 in a random orthogonal
basis plus a 10,000-component mixture with Zipf(1.1) weights), nlist 16,384,
batches of 4,096 queries from the same distribution, k = 10, 16-bit codes,
prefix ranking over the leading 256 rotated dimensions. Setup (data, k-means,
PCA rotation, ground truth) runs on the GPU with torch and is not timed; the
index is coded by the library's own load path. A "step" is one search of one
batch of 4,096 queries.

Prints one JSON line (rank 0). `--impl reference` times the reference's CPU
search instead: the oracle restatement (oracle/katoann_oracle.cpp) on the host
cores, since the reference itself only builds on x86-64 with AVX-512/AMX.
"""
from __future__ import annotations

import argparse
import json
import os
import platform
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (os.path.join(ROOT, "katoann-public_gb300"), os.path.join(ROOT, "oracle")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

# The workloads. "learned" (the default line) is the headline: 10M x 1024 with
# skewed lists, learned vs fixed nprobe. The others are the plain method on the
# other quoted shapes: the small CPU-runnable case, 1M x 1024, and 990k x 3072
# (the shape of the reference's OpenAI-3072-1M).
WORKLOADS = {
    "learned": dict(n=10_000_000, dim=1024, nlist=16384, batch=4096, head=256, ncomp=10000,
                    kind="spectral", power=1.2, zipf=1.1, learned=True,
                    data="synthetic: seeded power-law spectrum (i^-1.2) + 10,000-component Zipf(1.1) "
                         "mixture, unit norm; stands in for BioASQ-1024-10M"),
    "small": dict(n=100_000, dim=128, nlist=256, batch=1024, head=64, ncomp=100, kind="mixture",
                  learned=False,
                  data="synthetic: seeded 100-component Gaussian mixture (centres N(0,1), sigma 0.3, "
                       "dimension j scaled by 1/sqrt(j+1)), L2-normalised"),
    "plain": dict(n=1_000_000, dim=1024, nlist=4096, batch=4096, head=128, ncomp=1000,
                  kind="spectral", power=1.2, zipf=None, learned=False,
                  data="synthetic: seeded power-law spectrum (i^-1.2) + 1,000-component mixture, "
                       "unit norm"),
    "wide": dict(n=990_000, dim=3072, nlist=4096, batch=4096, head=256, ncomp=2000,
                 kind="spectral", power=1.0, zipf=None, learned=False,
                 data="synthetic: seeded power-law spectrum (i^-1.0) + 2,000-component mixture, "
                      "unit norm; stands in for OpenAI-3072-1M"),
}


L2_BYTES = 129 << 20  # GB300's L2 (about 129 MB)
# fused multiply-adds per second of the FP32 CUDA cores at the maximum SM clock
# (no measured figure for them; the rotation's roofline says "nominal")
FP32_TFMA_NOMINAL = 152 * 128 * 2.07e9 / 1e12


def size_name(n: int) -> str:
    return f"{n // 1000000}M" if n % 1000000 == 0 else f"{n / 1000:g}k"


def workload_name(n: int, d: int, L: int, B: int, k: int) -> str:
    return f"{size_name(n)} x {d} IVF, nlist {L}, batch {B}, k {k}"


def metric_name(w: str, n: int, d: int, B: int) -> str:
    size = size_name(n)
    path = "learned vs fixed nprobe" if WORKLOADS[w]["learned"] else "fixed nprobe"
    return f"QPS at recall@10 >= 0.99, {size} x {d} IVF, {path}, batch {B}, 1 GB300"


PUBLISHED_QPS = {"learned": (6294.0, "README.md:84, BioASQ-1024-10M on a 28-core Xeon (CPU)"),
                 "wide": (16449.0, "README.md:81, OpenAI-3072-1M on a 28-core Xeon (CPU)")}
LADDER = (8, 12, 16, 24, 32, 48, 64, 96, 128, 192, 256, 384, 512)  # learned nprobe choices
THRESHOLDS = (0.3, 0.5, 0.7, 0.8, 0.82, 0.84, 0.86, 0.88, 0.9, 0.92, 0.94, 0.96, 0.97, 0.98,
              0.985, 0.99, 0.995, 0.999)


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--config", choices=sorted(WORKLOADS), default="learned",
                    help="workload: learned (10M x 1024, the default line), small, plain or wide")
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--n", type=int, default=None)
    ap.add_argument("--dim", type=int, default=None)
    ap.add_argument("--nlist", type=int, default=None)
    ap.add_argument("--ncomp", type=int, default=None)
    ap.add_argument("--batch", type=int, default=None)
    ap.add_argument("--k", type=int, default=10)
    ap.add_argument("--head", type=int, default=None)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--kmeans-iters", type=int, default=6)
    ap.add_argument("--train", type=int, default=262144)
    ap.add_argument("--nprobe", type=int, default=0, help="skip the sweep, use this nprobe")
    ap.add_argument("--survivors", type=int, default=32)
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--ref-seconds", type=float, default=240.0,
                    help="reference arm: time budget of its warm-up and timed steps")
    ap.add_argument("--no-learned", action="store_true", help="skip the learned probe budget")
    ap.add_argument("--train-queries", type=int, default=200000,
                    help="training queries of the probe-budget model")
    ap.add_argument("--label-nprobe", type=int, default=1024,
                    help="lists of the search that gives the training labels' exact top-k")
    ap.add_argument("--label-survivors", type=int, default=256,
                    help="survivors of that search (prefix ranking, exact refinement)")
    ap.add_argument("--no-serving", action="store_true", help="skip the serving measurement")
    ap.add_argument("--no-build", action="store_true",
                    help="skip the timed index build on the device")
    ap.add_argument("--no-autotune", action="store_true",
                    help="keep the default knobs of the ranking pass (profiling runs)")
    ap.add_argument("--probe-epochs", type=int, default=24, help="training epochs of the probe model")
    ap.add_argument("--probe-depth", type=int, default=128,
                    help="coarse ranks the probe model's features read")
    ap.add_argument("--serve-seconds", type=float, default=1.5,
                    help="arrivals per serving run (seconds of the Poisson stream)")
    args = ap.parse_args()
    w = WORKLOADS[args.config]
    for key in ("n", "dim", "nlist", "ncomp", "batch", "head"):
        if getattr(args, key) is None:
            setattr(args, key, w[key])
    if not w["learned"]:
        args.no_learned = True
        args.no_serving = True  # the serving block belongs to the headline index
    return args


def fixed_grid(L: int) -> list[tuple[int, int]]:
    """The fixed (nprobe, survivors) settings both arms sweep, in ascending
    nprobe per survivors value (as fine as the learned path's thresholds)."""
    grid = [(p, s) for s in (32, 64)
            for p in (16, 24, 32, 48, 64, 72, 80, 88, 96, 112, 128, 160, 192, 256) if p <= L]
    grid += [(p, 128) for p in (128, 160, 192, 224, 256, 320, 384, 512) if p <= L]
    return grid


# ----------------------------------------------------------------- ranks
# N GPUs run N replicas: every rank holds the same index (same data seed) and
# searches its own batches of queries. No collective touches the search; the
# job's QPS is all ranks' queries over the slowest rank's time, and every
# rank runs the setting rank 0 chose.

def query_seed(seed: int, rank: int) -> int:
    """The seed of a rank's evaluation queries: rank 0 keeps the single-GPU
    queries, every other rank draws its own."""
    return seed + 1_000_003 * rank


def max_over_ranks(dist, x: float) -> float:
    """The largest x over all ranks (the slowest rank's time); x itself
    without a process group."""
    if dist is None:
        return float(x)
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def from_rank0(dist, i: int) -> int:
    """Rank 0's integer on every rank (i itself without a process group)."""
    if dist is None:
        return int(i)
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([int(i)], dtype=torch.int64, device=dev)
    dist.broadcast(t, src=0)
    return int(t.item())


# ----------------------------------------------------------------- data
def make_data(torch, n, d, ncomp, seed, queries, train_queries=0, qseed=None, dev="cuda",
              kind="spectral", power=1.2, zipf=1.1):
    """Unit vectors of one of two families:
      spectral: mixture centres and per-point noise share an anisotropic
        spectrum (eigenvalue_i ~ i^-power) in a random orthogonal basis;
        component weights follow Zipf(zipf) (skewed lists) or are uniform;
      mixture: centres N(0, 1), per-component sigma 0.3, dimension j scaled
        by 1/sqrt(j + 1), L2-normalised.
    Returns the base, the evaluation queries and (another stream of the same
    distribution) the probe-budget training queries. `seed` fixes the
    distribution, the base and the training queries; `qseed` (default: seed)
    the evaluation queries, so that replicas share an index and differ in
    their queries."""
    g = torch.Generator(device=dev).manual_seed(seed)
    if kind == "mixture":
        centres = torch.randn(ncomp, d, generator=g, device=dev)
        scale = 1.0 / torch.sqrt(torch.arange(d, device=dev, dtype=torch.float32) + 1.0)
        cdf = torch.arange(1, ncomp + 1, device=dev, dtype=torch.float32) / ncomp
    else:
        # random orthogonal basis (QR on the host: torch's linear-algebra
        # library is not needed on the device path)
        A = torch.randn(d, d, generator=g, device=dev).double().cpu().numpy()
        Qn, Rn = np.linalg.qr(A)
        Q = torch.from_numpy(Qn * np.sign(np.diag(Rn))[None, :]).float().to(dev)
        lam = torch.arange(1, d + 1, device=dev, dtype=torch.float32) ** -power
        B = torch.sqrt(lam / lam.sum())[:, None] * Q.T
        centres = torch.randn(ncomp, d, generator=g, device=dev) @ B
        w = (torch.arange(1, ncomp + 1, device=dev, dtype=torch.float64) ** -zipf if zipf
             else torch.ones(ncomp, device=dev, dtype=torch.float64))
        cdf = torch.cumsum(w / w.sum(), 0).float()
    cdf[-1] = 1.0

    def sample(m, gen):
        out = torch.empty(m, d, device=dev)
        for s in range(0, m, 1 << 20):
            e = min(m, s + (1 << 20))
            comp = torch.searchsorted(cdf, torch.rand(e - s, generator=gen, device=dev)).clamp_(max=ncomp - 1)
            if kind == "mixture":
                x = (centres[comp] + 0.3 * torch.randn(e - s, d, generator=gen, device=dev)) * scale
            else:
                x = centres[comp] + 0.5 * (torch.randn(e - s, d, generator=gen, device=dev) @ B)
            out[s:e] = x / x.norm(dim=1, keepdim=True)
        return out

    base = sample(n, g)
    gq = torch.Generator(device=dev).manual_seed((seed if qseed is None else qseed) + 7919)
    q = sample(queries, gq)
    gt_ = torch.Generator(device=dev).manual_seed(seed + 104729)
    tq = sample(train_queries, gt_) if train_queries else None
    return base, q, tq


def assign(torch, x, c, chunk=65536):
    cn = (c * c).sum(1)
    out = torch.empty(x.shape[0], dtype=torch.int64, device=x.device)
    for s in range(0, x.shape[0], chunk):
        e = min(x.shape[0], s + chunk)
        out[s:e] = torch.addmm(cn[None, :], x[s:e], c.T, alpha=-2.0).argmin(1)
    return out


def kmeans(torch, x, L, iters, train, seed):
    g = torch.Generator(device="cuda").manual_seed(seed + 1)
    t = x[torch.randperm(x.shape[0], generator=g, device="cuda")[:train]]
    c = t[torch.randperm(t.shape[0], generator=g, device="cuda")[:L]].clone()
    for _ in range(iters):
        a = assign(torch, t, c)
        sums = torch.zeros_like(c).index_add_(0, a, t)
        cnt = torch.bincount(a, minlength=L)
        nz = cnt > 0
        c[nz] = sums[nz] / cnt[nz, None].float()
    return c


def pca_rotation(torch, x, sample, seed):
    g = torch.Generator(device="cuda").manual_seed(seed + 2)
    s = x[torch.randperm(x.shape[0], generator=g, device="cuda")[:sample]].double()
    s -= s.mean(0, keepdim=True)
    cov = ((s.T @ s) / s.shape[0]).cpu().numpy()
    evals, evecs = np.linalg.eigh(cov)
    order = np.argsort(-evals, kind="stable")
    # row j = axis of the j-th largest variance
    return torch.from_numpy(np.ascontiguousarray(evecs[:, order].T)).float().cuda()


def ground_truth(torch, x, ids, q, k, chunk=262144):
    """Exact float32 top-k by squared L2 (no TF32), ids in the original order."""
    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    bd = torch.full((q.shape[0], k), float("inf"), device="cuda")
    bi = torch.zeros((q.shape[0], k), dtype=torch.int64, device="cuda")
    for s in range(0, x.shape[0], chunk):
        e = min(x.shape[0], s + chunk)
        xc = x[s:e]
        d = torch.addmm((xc * xc).sum(1)[None, :], q, xc.T, alpha=-2.0)
        v, i = torch.topk(d, k, dim=1, largest=False)
        bd, j = torch.topk(torch.cat([bd, v], 1), k, dim=1, largest=False)
        bi = torch.gather(torch.cat([bi, i + s], 1), 1, j)
    torch.backends.cuda.matmul.allow_tf32 = prev
    return ids[bi].cpu().numpy().astype(np.uint32)


def recall(ids: np.ndarray, gt: np.ndarray, k: int) -> float:
    hit = 0
    for a, b in zip(ids, gt):
        hit += len(set(a[:k].tolist()) & set(b[:k].tolist()))
    return hit / (len(gt) * k)


# --------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)),
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------ roofline
SEED_ROWS = 2048  # rows behind each query's seed bound (the library default for survivors <= 128)
# the kernel the phase timer brackets inside each phase it can dominate
PHASE_KERNEL = {"ranking pass": "rank_tc_kernel", "coarse product": "coarse_tc_kernel",
                "rotate+quantize": "rotation"}
SKETCH_BYTES = 32  # head bytes of a row the seed's sketch reads


def seed_bytes(B: int, rows: int, S: int, head: int) -> float:
    """Bytes the seed bounds read: every looked-at row's first SKETCH_BYTES
    head bytes and the 3S rows the sketch picks in full; with at most 3S rows
    every row in full."""
    full = min(rows, 3 * S)
    if rows > full:
        return float(B) * (rows * min(SKETCH_BYTES, head) + full * head)
    return float(B) * rows * head

# DRAM bytes per 128-row tile of the tensor-core ranking kernel: one ncu
# capture (dram__bytes_read.sum + dram__bytes_write.sum, one pass) of this
# 10M x 1024 search at nprobe 72 and 64 survivors moved 2,632.4 + 22.3 MB over
# 96,108 tiles, about 27.6 KB per tile (1.09 x the 256 head bytes of each
# probed row). The traffic of a launch scales with its tiles.
RANK_TC_DRAM_BYTES_PER_TILE = (2632.4e6 + 22.3e6) / 96108


def phase_work(phase: str, B: int, L: int, dc: int, d: int, nprobe: int, S: int, head: int,
               probed_rows: float, probed_lists_rows: float):
    """(bound, algorithmic work per launch, unit) of one pipeline phase.
    Byte products of the exact integer products are counted as the BF16
    tensor-core MACs an exact split-byte product needs (four per code pair and
    dimension for full codes, one for high bytes), two FLOPs each."""
    if phase == "coarse product":
        return "tensor", 2.0 * 4 * B * L * dc / 1e12, "TFLOP/s"
    if phase == "ranking pass":
        # each probed list's head bytes, read once per batch (the row norms are
        # summed from the same bytes; ids are only read for the survivors)
        return "hbm", probed_lists_rows * head / 1e9, "GB/s"
    if phase == "seed bounds":
        # the sketch over the first SEED_ROWS rows of each query's nearest
        # lists, and the rows it picks
        return "hbm", seed_bytes(B, SEED_ROWS, S, head) / 1e9, "GB/s"
    if phase == "refine":
        return "hbm", B * S * (2 * dc + 8 + 4) / 1e9, "GB/s"
    if phase == "rotate+quantize":
        # the rotation's fused multiply-adds in the reference's fixed order
        # (CUDA cores; the quantization is a small epilogue of it)
        return "fp32", B * d * d / 1e12, "TFMA/s"
    if phase == "coarse select":
        return "hbm", B * L * 4 / 1e9, "GB/s"
    if phase == "survivor merge":
        return "hbm", B * nprobe * min(S, 256) * 8 / 1e9, "GB/s"
    return "hbm", B * nprobe * 16 / 1e9, "GB/s"


def measured_peaks() -> dict:
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            p = json.load(f)
        return {"hbm_gbs": p["hbm_gbs"], "bf16_tflops": p["bf16_tflops"], "source": "measured"}
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "source": "fallback"}


# ----------------------------------------------------------------- main
def main():
    args = parse_args()
    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference" and rank != 0:
        return  # rank 0 alone times the CPU reference; it needs no process group
    torch.cuda.set_device(local)
    dist = None
    if world > 1 and args.impl == "ours":
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.backends.cuda.matmul.allow_tf32 = True
    t0 = time.time()
    n, d, L, B, k = args.n, args.dim, args.nlist, args.batch, args.k
    ntrain = 0 if (args.no_learned or args.nprobe or args.impl == "reference") else args.train_queries
    wl = WORKLOADS[args.config]
    base, queries, train_q = make_data(torch, n, d, args.ncomp, args.seed, B, ntrain,
                                       qseed=query_seed(args.seed, rank), kind=wl["kind"],
                                       power=wl.get("power", 1.2), zipf=wl.get("zipf"))
    cen = kmeans(torch, base, L, args.kmeans_iters, min(args.train, n), args.seed)
    rot = pca_rotation(torch, base, min(100000, n), args.seed)
    a = assign(torch, base, cen)
    order = torch.argsort(a, stable=True)
    sizes = torch.bincount(a, minlength=L).cpu().numpy().astype(np.uint32)
    del a
    vectors = base[order]
    del base
    torch.cuda.empty_cache()
    gt = ground_truth(torch, vectors, order, queries, k)
    setup_s = time.time() - t0

    if args.impl == "reference":
        run_reference(args, torch, vectors, order, cen, rot, sizes, queries, gt, setup_s)
        return

    import katoann
    work_stream = torch.cuda.Stream()
    torch.cuda.synchronize()
    torch.cuda.set_stream(work_stream)  # every launch of the timed path on one stream
    idx = katoann.Index()
    t1 = time.time()
    idx.load_arrays(cen, sizes, order.to(torch.int32), vectors, rotation=rot, head_dims=args.head,
                    max_batch=B)
    torch.cuda.synchronize()
    load_s = time.time() - t1
    if args.no_build:
        del vectors  # the index holds its codes; the float vectors are not needed any more
        torch.cuda.empty_cache()
    stream = work_stream.cuda_stream
    ids_d = torch.empty((B, k), dtype=torch.int32, device="cuda")
    dists_d = torch.empty((B, k), dtype=torch.float32, device="cuda")

    np_d = torch.empty(B, dtype=torch.int32, device="cuda")

    def search(cfg, timer=None, nprobe_out=None):
        """One device search of the batch: fixed {nprobe, survivors}, or learned
        {model, threshold, nprobe (the cap), survivors}."""
        idx.search_device(queries, ids_d, dists_d, k=k, nprobe=cfg["nprobe"],
                          survivors=cfg["survivors"], stream=stream, timer=timer,
                          budget=cfg.get("model"), threshold=cfg.get("threshold", 0.95),
                          nprobe_out=nprobe_out)

    def run(cfg, reps=3):
        search(cfg, nprobe_out=np_d if cfg.get("model") else None)
        torch.cuda.synchronize()
        r = recall(ids_d.cpu().numpy().view(np.uint32), gt, k)
        mean_np = float(np_d.float().mean()) if cfg.get("model") else float(cfg["nprobe"])
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            search(cfg)
        e1.record()
        torch.cuda.synchronize()
        return r, e0.elapsed_time(e1) / reps, mean_np

    sweep = []
    grid = [(args.nprobe, args.survivors)] if args.nprobe else fixed_grid(L)
    for p, s in grid:
        r, ms, _ = run(dict(nprobe=p, survivors=s))
        sweep.append({"path": "fixed", "nprobe": p, "survivors": s, "recall": round(r, 5),
                      "ms": round(ms, 3), "qps": round(B / ms * 1e3, 1)})

    # ---- the learned per-query probe budget: train on its own query stream,
    # then sweep the threshold (every query's result is the fixed-nprobe
    # result at its own nprobe; the model only chooses the nprobe)
    models, learned_info = {}, None
    if train_q is not None:
        tq = train_q.cpu().numpy()
        del train_q
        torch.cuda.empty_cache()
        cap = min(LADDER[-1], L)
        ladder = tuple(v for v in LADDER if v <= L)
        lab_p = min(L, args.label_nprobe)
        depth = min(args.probe_depth, L)
        learned_info = {"train_queries": len(tq), "ladder": list(ladder), "depth": depth,
                        "label_search": {"nprobe": lab_p, "ranking": "prefix",
                                         "survivors": args.label_survivors},
                        "models": {}}
        for s_l in (64, 128):
            t_l = time.time()
            m = katoann.ProbeModel.train(idx, tq, ladder=ladder, depth=depth, k=k,
                                         label_nprobe=lab_p, label_ranking="prefix",
                                         label_survivors=args.label_survivors, ranking="prefix",
                                         survivors=s_l, epochs=args.probe_epochs, batch=1024,
                                         seed=args.seed)
            models[s_l] = m
            hist = np.bincount(m.labels, minlength=len(ladder))
            learned_info["models"][s_l] = {"train_s": round(time.time() - t_l, 1),
                                           "loss_first_last": [round(float(m.loss[0]), 4),
                                                               round(float(m.loss[-1]), 4)],
                                           "label_histogram": hist.tolist()}
        # how close the labels' top-k is to the exact-distance search's (a sample)
        t_c = time.time()
        smp = tq[:256]
        ex, _ = idx.search(smp, k=k, nprobe=lab_p, ranking="full", survivors=k)
        lb, _ = idx.search(smp, k=k, nprobe=lab_p, ranking="prefix", survivors=args.label_survivors)
        learned_info["label_check"] = {
            "queries": len(smp), "same_top_k_as_exact_search": float(np.mean(
                [set(a) == set(b) for a, b in zip(ex, lb)])), "seconds": round(time.time() - t_c, 1)}
        del tq
        for s_l, m in models.items():
            for thr in THRESHOLDS:
                r, ms, mnp = run(dict(nprobe=cap, survivors=s_l, model=m, threshold=thr))
                sweep.append({"path": "learned", "survivors": s_l, "threshold": thr, "cap": cap,
                              "mean_nprobe": round(mnp, 2), "recall": round(r, 5),
                              "ms": round(ms, 3), "qps": round(B / ms * 1e3, 1)})

    def best(target, path=None):
        ok = [x for x in sweep if x["recall"] >= target and path in (None, x["path"])]
        return min(ok, key=lambda x: x["ms"]) if ok else None

    def summary(x):
        if x is None:
            return None
        keys = ("nprobe", "survivors") if x["path"] == "fixed" else \
            ("survivors", "threshold", "cap", "mean_nprobe")
        return {"qps": x["qps"], "recall": x["recall"], **{kk: x[kk] for kk in keys}}

    b99, b999 = best(0.99), best(0.999)
    chosen = b99 or max(sweep, key=lambda x: x["recall"])
    chosen = sweep[from_rank0(dist, sweep.index(chosen))]  # the same grid on every rank
    if chosen["path"] == "learned":
        cfg = dict(nprobe=chosen["cap"], survivors=chosen["survivors"],
                   model=models[chosen["survivors"]], threshold=chosen["threshold"])
    else:
        cfg = dict(nprobe=chosen["nprobe"], survivors=chosen["survivors"])
    S = cfg["survivors"]
    fixed99 = best(0.99, "fixed") or max((x for x in sweep if x["path"] == "fixed"),
                                         key=lambda x: x["recall"])

    # ---- the autotuner picks the ranking pass's knobs for this setting
    # (seed rows, CTA split weight, item width; results never depend on them)
    tuned = None
    if not args.no_autotune:
        tuned = idx.autotune(queries.cpu().numpy(), k=k, nprobe=cfg["nprobe"], survivors=S,
                             budget=cfg.get("model"), threshold=cfg.get("threshold", 0.95))
        tuned["ms_before"] = chosen["ms"]

    # ---- timed region: K steps on device-resident queries
    for _ in range(max(3, args.warmup)):
        search(cfg)
    timer = katoann.PhaseTimer(args.steps + 4)
    timer.read()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    code_bytes = n * ((d + 63) // 64 * 64) * 2
    flush = None
    if code_bytes < 2 * L2_BYTES:
        # the index fits in L2: a buffer larger than L2 is written between
        # the timed steps, outside their events
        flush = torch.empty(2 * L2_BYTES, dtype=torch.uint8, device="cuda")
    with ClockSampler(local) as clocks:
        if flush is None:
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(args.steps):
                search(cfg, timer=timer)
            e1.record()
            torch.cuda.synchronize()
            elapsed_ms = e0.elapsed_time(e1)
        else:
            ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
                  for _ in range(args.steps)]
            for a0, a1 in ev:
                flush.zero_()
                a0.record()
                search(cfg, timer=timer)
                a1.record()
            torch.cuda.synchronize()
            elapsed_ms = sum(a0.elapsed_time(a1) for a0, a1 in ev)
    if dist:
        dist.barrier()
    phases, passes = timer.read()
    kernel_ms = timer.kernels()  # the single kernels' events over the same passes
    ms = max_over_ranks(dist, elapsed_ms)
    value = world * B * args.steps / (ms / 1e3)
    search(cfg, nprobe_out=np_d)
    torch.cuda.synchronize()
    search_stats = idx.search_stats()
    launches_per_search = katoann.last_launches()
    per_query_np = np_d.cpu().numpy().astype(np.int64)

    # ---- the same search captured as a CUDA graph and replayed (one launch
    # per step instead of one per kernel)
    def search_graph():
        idx.search_device(queries, ids_d, dists_d, k=k, nprobe=cfg["nprobe"], survivors=S,
                          stream=stream, budget=cfg.get("model"),
                          threshold=cfg.get("threshold", 0.95), graph=True)

    for _ in range(max(3, args.warmup)):
        search_graph()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    g0, g1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    g0.record()
    for _ in range(args.steps):
        search_graph()
    g1.record()
    torch.cuda.synchronize()
    graph_ms = max_over_ranks(dist, g0.elapsed_time(g1) / args.steps)
    graph_recall = recall(ids_d.cpu().numpy().view(np.uint32), gt, k)

    # ---- end to end through the public host API (pinned host buffers)
    qh = torch.empty((B, d), dtype=torch.float32).pin_memory()
    qh.copy_(queries.cpu())
    ih = torch.empty((B, k), dtype=torch.int32).pin_memory()
    dh = torch.empty((B, k), dtype=torch.float32).pin_memory()

    def host_search(graph):
        idx.search_into(qh.data_ptr(), B, ih.data_ptr(), dh.data_ptr(), k=k, nprobe=cfg["nprobe"],
                        survivors=S, budget=cfg.get("model"), threshold=cfg.get("threshold", 0.95),
                        graph=graph)

    # end to end through the host API, each step copying its queries in and
    # its results out: with the kernels replayed as a captured graph (the
    # line's e2e), and launched one by one (e2e_launches)
    e2e_steps = max(10, min(args.steps, 100))
    e2e_runs = {}
    for graph in (False, True):
        for _ in range(3):
            host_search(graph)
        if dist:
            dist.barrier()
        t2 = time.perf_counter()
        for _ in range(e2e_steps):
            host_search(graph)
        e2e_s = max_over_ranks(dist, time.perf_counter() - t2)
        e2e_runs[graph] = (world * B * e2e_steps / e2e_s, recall(ih.numpy().view(np.uint32), gt, k))
    e2e_qps, e2e_recall = e2e_runs[True]

    # ---- the index build on the device: the same base vectors partitioned by
    # the library (katoann.build_partition: k-means++ and Lloyd on a training
    # sample, every vector's list, the PCA rotation), timed, loaded, and
    # searched at the fixed setting; the timed index above comes from the
    # setup's k-means so that both arms search the same index
    build = None
    if not args.no_build:
        build = device_build(args, torch, katoann, vectors, order, queries, gt, fixed99, B, k)
        del vectors
        torch.cuda.empty_cache()

    # ---- serving: Poisson arrivals through the continuous-batching server
    serve = None
    if rank == 0 and world == 1 and not args.no_serving:
        fixed_cfg = {"nprobe": fixed99["nprobe"], "survivors": fixed99["survivors"]}
        l99 = best(0.99, "learned")
        learned_cfg = (dict(nprobe=l99["cap"], survivors=l99["survivors"],
                            model=models[l99["survivors"]], threshold=l99["threshold"])
                       if l99 else None)
        serve = serving(katoann, idx, queries, (1000, 5000, 20000, 100000, 400000), args.serve_seconds,
                        fixed_cfg, learned_cfg)

    # ---- roofline of the dominant phase
    peaks = measured_peaks()
    per_launch = {ph: v / max(passes, 1) for ph, v in phases.items()}
    dom = max(per_launch, key=per_launch.get)
    list_sizes = sizes.astype(np.float64)
    probed = np.zeros(L, bool)
    # lists probed by the batch (for the ranking pass' bytes): from the oracle-free
    # coarse of the library is not exposed, so count via the CPU copy of the centroids
    cq = queries @ (rot.T)
    cc = cen @ (rot.T)
    dd = torch.cdist(cq, cc)
    pmax = int(per_query_np.max())
    top = torch.topk(dd, pmax, dim=1, largest=False).indices.cpu().numpy()
    keep = np.arange(pmax)[None, :] < per_query_np[:, None]  # each query's own nprobe
    probed[np.unique(top[keep])] = True
    p = int(round(float(per_query_np.mean())))
    probed_rows = float(list_sizes[probed].sum())
    rows_source = "float coarse distances on the host (approximate)"
    if search_stats.get("probed_rows"):  # the search's own count of the rows it reads
        probed_rows = float(search_stats["probed_rows"])
        rows_source = "the search's own count"
    skew = {"max_list": int(sizes.max()), "mean_list": round(float(sizes.mean()), 1),
            "p99_list": int(np.percentile(sizes, 99)), "empty_lists": int((sizes == 0).sum()),
            "lists_probed": int(search_stats.get("lists_probed") or probed.sum())}
    bound, work, unit = phase_work(dom, B, L, (d + 63) // 64 * 64, d, p, max(S, k), args.head,
                                   probed_rows, probed_rows)
    # the dominant phase's own kernel, timed by its events on the search stream
    # (the phase adds its preparation, bucketing and the like)
    kname = PHASE_KERNEL.get(dom)
    kms, kn = kernel_ms.get(kname, (0.0, 0))
    launch_ms = kms / kn if kn else per_launch[dom]
    achieved = work / (launch_ms / 1e3)
    peak = {"tensor": peaks["bf16_tflops"], "fp32": FP32_TFMA_NOMINAL}.get(bound, peaks["hbm_gbs"])
    traffic = None
    if dom == "ranking pass" and search_stats.get("ranking_tiles"):
        traffic = round(RANK_TC_DRAM_BYTES_PER_TILE * search_stats["ranking_tiles"] / 1e9, 3)
    roofline = {"kernel": kname if kn else dom, "phase": dom, "bound": bound,
                "achieved": round(achieved, 2), "peak": peak,
                "unit": unit, "frac": round(achieved / peak, 4), "traffic": traffic,
                "traffic_unit": "GB per launch (the 10M capture's bytes per tile x this run's tiles)",
                "algorithmic": round(work, 3), "algorithmic_rows_from": rows_source,
                "peak_source": ("nominal: 152 SMs x 128 FP32 lanes x 2.07 GHz" if bound == "fp32" else
                                peaks["source"] + (" burst bf16" if bound == "tensor" else " copy")),
                "ms_per_launch": round(launch_ms, 4), "launches_timed": kn,
                "phase_ms_per_launch": round(per_launch[dom], 4),
                "phase_frac": round(work / (per_launch[dom] / 1e3) / peak, 4)}

    # ---- CPU baseline (rank 0, N = 1): the oracle on a bounded sample, and a
    # full-size parity check of the same queries
    cpu = None
    parity = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu, parity = cpu_baseline(args, torch, idx, queries, fixed99, cfg, k)

    clk = clocks.summary()
    pub = PUBLISHED_QPS.get(args.config) if (n, d) == (wl["n"], wl["dim"]) else None
    out = {
        "metric": metric_name(args.config, n, d, B),
        "value": round(value, 1), "unit": "queries/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 4), "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": round(value / pub[0], 2) if pub else None,
        "baseline_published": ({"value": pub[0], "unit": "queries/s", "source": pub[1]} if pub else None),
        "dtype": "u8",
        "data": wl["data"],
        "config": {"workload": workload_name(n, d, L, B, k),
                   "nprobe_path": chosen["path"],
                   **{kk: v for kk, v in summary(chosen).items() if kk not in ("qps", "recall")},
                   "prefix_dims": args.head,
                   "ranking": "prefix",
                   "l2_policy": (f"inputs larger than L2 (index codes {code_bytes / 1e9:.1f} GB per pass)"
                                 if flush is None else
                                 f"L2 flushed between steps (a {2 * L2_BYTES >> 20} MiB write outside "
                                 f"the timed events; index codes {code_bytes / 1e6:.0f} MB)")},
        "recall": chosen["recall"],
        "qps_at_recall_0.999": (round(b999["qps"], 1) if b999 else None),
        "setting_at_recall_0.999": ({"path": b999["path"], **summary(b999)} if b999 else None),
        "learned_vs_fixed": {
            "recall_0.99": {"fixed": summary(best(0.99, "fixed")),
                            "learned": summary(best(0.99, "learned"))},
            "recall_0.999": {"fixed": summary(best(0.999, "fixed")),
                             "learned": summary(best(0.999, "learned"))}},
        "autotune": tuned,
        "index_build": build,
        "probe_model": learned_info,
        "serving": serve,
        "sweep": sweep,
        "phases_ms_per_step": {k2: round(v, 4) for k2, v in per_launch.items()},
        "kernels_ms_per_launch": {k2: round(a / b, 4) for k2, (a, b) in kernel_ms.items() if b},
        "roofline": roofline,
        "graph_replay": {"ms_per_step": round(graph_ms, 4),
                         "qps": round(world * B / graph_ms * 1e3, 1),
                         "recall": round(graph_recall, 5),
                         "api": "katoann.Index.search_device(graph=True)"},
        "e2e": {"value": round(e2e_qps, 1), "unit": "queries/s", "recall": round(e2e_recall, 5),
                "h2d_bytes_per_step": B * d * 4, "d2h_bytes_per_step": B * k * 8,
                "api": "katoann.Index.search_into(graph=True) (pinned host buffers)",
                "launched_one_by_one": {"value": round(e2e_runs[False][0], 1),
                                        "recall": round(e2e_runs[False][1], 5)}},
        "gpu_launches": launches_per_search * args.steps,
        "clocks": clk,
        "cpu_baseline": cpu,
        "parity_full_size": parity,
        "lists": skew,
        "search_stats": search_stats,
        "setup_s": round(setup_s, 1), "load_s": round(load_s, 1),
        "host": platform.machine(),
    }
    if rank == 0:
        print(json.dumps(out))
    if dist:
        dist.destroy_process_group()


def device_build(args, torch, katoann, vectors, order, queries, gt, fixed, B, k):
    """katoann.build_partition on the device-resident base vectors, then the
    index of that partition and its recall at the fixed setting."""
    L = args.nlist
    torch.cuda.synchronize()
    t0 = time.time()
    cen, assign, rot, head = katoann.build_partition(
        vectors, nlist=L, train_size=min(args.train, vectors.shape[0]), kmeans_iters=args.kmeans_iters,
        seed=args.seed + 1, rotation_sample=100000)
    build_s = time.time() - t0
    a = torch.from_numpy(assign.astype(np.int64)).cuda()
    pos = torch.argsort(a, stable=True)  # lists in ascending id order
    del a
    sizes = np.bincount(assign, minlength=L).astype(np.uint32)
    idx = katoann.Index()
    t1 = time.time()
    moved = vectors[pos]
    # device vectors: every array goes in as a CUDA tensor
    idx.load_arrays(torch.from_numpy(cen).cuda(), sizes, order[pos].to(torch.int32), moved,
                    rotation=None if rot is None else torch.from_numpy(rot).cuda(),
                    head_dims=args.head, max_batch=B)
    torch.cuda.synchronize()
    load_s = time.time() - t1
    del moved
    torch.cuda.empty_cache()
    ids, _ = idx.search(queries.cpu().numpy(), k=k, nprobe=fixed["nprobe"], survivors=fixed["survivors"])
    del idx
    return {"seconds": round(build_s, 1), "load_s": round(load_s, 1), "nlist": L,
            "train": min(args.train, vectors.shape[0]), "kmeans_iters": args.kmeans_iters,
            "empty_lists": int((sizes == 0).sum()), "max_list": int(sizes.max()),
            "rotated": rot is not None, "head_dims": head,
            "recall_at_fixed_setting": round(recall(ids, gt, k), 5),
            "setting": {"nprobe": fixed["nprobe"], "survivors": fixed["survivors"]},
            "api": "katoann.build_partition (device data, no files)"}


def serving(katoann, idx, queries, rates, seconds, fixed, learned, seed=0):
    """Poisson arrivals at each rate, k drawn from {10, 100} per request, served
    by katoann.Server (continuous batching, 3 batches in flight, each a replay
    of a captured search graph) from the library's native client; latency
    from the scheduled arrival to completion. `fixed` / `learned` are the search settings (learned: model,
    threshold, cap)."""
    out = []
    q = queries.cpu().numpy()
    for name, cfg in (("fixed", fixed), ("learned", learned)):
        if cfg is None:
            continue
        server = katoann.Server(idx, max_batch=4096, max_in_flight=3, max_k=100,
                                nprobe=cfg["nprobe"], survivors=cfg["survivors"],
                                budget=cfg.get("model"), threshold=cfg.get("threshold", 0.95),
                                warm_k=(10, 100))
        for _ in range(2):  # warm-up: a full batch of each k
            for r in [server.submit(q[i], k) for k in (10, 100) for i in range(len(q))]:
                server.wait(r)
        for rate in rates:
            n = max(2000, int(rate * seconds))
            r = server.load(q, rate, n, kmix=(10, 100), seed=seed + int(rate))
            st = server.stats()
            out.append({"nprobe_path": name, "rate": rate, "requests": n,
                        **{key: (round(v, 3) if isinstance(v, float) else v)
                           for key, v in r.items()},
                        "graph_batches": st["graph_batches"], "graphs": st["graphs"],
                        "batches_so_far": st["batches"]})
        del server
    return out


def _time_oracle(o, qs, k, p, S, budget_s):
    """Queries per second of the oracle on a sample sized to the time budget."""
    t = time.perf_counter()
    o.search(qs[:16], k=k, nprobe=p, survivors=S)
    per_q = (time.perf_counter() - t) / 16
    m = int(min(len(qs), max(16, budget_s / max(per_q, 1e-6))))
    t = time.perf_counter()
    ids, dists = o.search(qs[:m], k=k, nprobe=p, survivors=S)
    dt = time.perf_counter() - t
    return m / dt, m, dt, ids, dists


def cpu_baseline(args, torch, idx, queries, fixed, cfg, k):
    """The oracle (the reference's algorithm, all host cores) on a bounded
    sample of the batch at the fixed setting that reaches the recall target,
    and a bit-exactness check of the timed path on the same sample: fixed, or
    learned (then every query against the oracle at its own nprobe)."""
    import oracle
    codes = idx.export_codes()
    o = oracle.OracleIndex(None, codes=codes)
    del codes
    cores = os.cpu_count() or 1
    oracle.set_threads(cores)
    q = queries.cpu().numpy()
    p, S = fixed["nprobe"], fixed["survivors"]
    qps, m, dt, oids, odists = _time_oracle(o, q, k, p, S, args.cpu_seconds)
    cpu = {"value": round(qps, 1), "unit": "queries/s", "cores": cores, "kind": "port",
           "sample": f"{m} of the {len(q)} batch queries, same index, fixed nprobe {p}, "
                     f"survivors {S}, {dt:.1f} s", "isa": platform.machine()}
    if cfg.get("model") is None and cfg["nprobe"] == p and cfg["survivors"] == S:
        gids, gd = idx.search(q[:m], k=k, nprobe=p, survivors=S)
        exact = bool(np.array_equal(gids, oids) and np.array_equal(gd, odists))
        return cpu, {"queries": m, "path": "fixed", "bit_exact_vs_oracle": exact}
    gids, gd, used = idx.search(q[:m], k=k, nprobe=cfg["nprobe"], survivors=cfg["survivors"],
                                budget=cfg.get("model"), threshold=cfg.get("threshold", 0.95),
                                return_nprobe=True)
    exact = True
    for v in np.unique(used):
        sel = np.nonzero(used == v)[0]
        rid, rd = o.search(q[:m][sel], k=k, nprobe=int(v), survivors=cfg["survivors"])
        exact &= bool(np.array_equal(gids[sel], rid) and np.array_equal(gd[sel], rd))
    return cpu, {"queries": m, "path": "learned (each query at its own nprobe)",
                 "bit_exact_vs_oracle": exact}


def run_reference(args, torch, vectors, order, cen, rot, sizes, queries, gt, setup_s):
    """The reference's CPU search on the host cores: the oracle restatement
    (oracle/katoann_oracle.cpp; the reference's own sources build only on
    x86-64 with AVX-512/AMX), loaded from the same float vectors as the GPU
    arm and coded by the oracle itself, handed over in pieces from the
    device. No library of this repository is loaded in this process.

    Its setting follows the reference's protocol (scripts/plot.py:37-50): a
    fixed nprobe x survivors sweep over the whole batch, and the fastest point
    at recall@10 >= 0.99. A row of the sweep stops at its first point that
    reaches the target (a larger nprobe at the same survivors only costs
    more). A step is one search of the whole 4,096-query batch, unless
    (warm-up + steps) whole batches would exceed --ref-seconds; then each step
    searches the largest sample of the batch that fits."""
    import oracle
    k, B = args.k, args.batch
    cores = os.cpu_count() or 1
    oracle.set_threads(cores)
    t0 = time.time()
    meta = dict(centroids=cen.cpu().numpy(), list_sizes=sizes,
                ids=order.cpu().numpy().astype(np.uint32), rotation=rot.cpu().numpy(),
                head_dims=args.head)
    chunk = 1 << 18
    pieces = ((s0, vectors[s0:s0 + chunk].cpu().numpy()) for s0 in range(0, vectors.shape[0], chunk))
    o = oracle.OracleIndex(None, arrays=meta, pieces=pieces)
    load_s = time.time() - t0
    q = queries.cpu().numpy()

    # ---- the sweep (whole batch per point)
    t1 = time.time()
    target = 0.99
    sweep = []
    grid = [(args.nprobe, args.survivors)] if args.nprobe else fixed_grid(args.nlist)
    done_s = set()
    for p, S in grid:
        if S in done_s:
            continue
        t = time.perf_counter()
        ids, _ = o.search(q, k=k, nprobe=p, survivors=S)
        dt = time.perf_counter() - t
        r = recall(ids, gt, k)
        sweep.append({"nprobe": p, "survivors": S, "recall": round(r, 5), "seconds": round(dt, 3),
                      "qps": round(len(q) / dt, 1)})
        if r >= target:
            done_s.add(S)
    ok = [x for x in sweep if x["recall"] >= target]
    pick = min(ok, key=lambda x: x["seconds"]) if ok else max(sweep, key=lambda x: x["recall"])
    p, S = pick["nprobe"], pick["survivors"]
    sweep_s = time.time() - t1

    # ---- timed steps at that setting
    per_batch = pick["seconds"]
    m = len(q)
    if per_batch * (args.steps + args.warmup) > args.ref_seconds:
        m = max(16, int(len(q) * args.ref_seconds / (per_batch * (args.steps + args.warmup))))
    for i in range(args.warmup):
        o.search(q[:m], k=k, nprobe=p, survivors=S)
    tot_t = 0.0
    for i in range(args.steps):
        s0 = (i * m) % max(1, len(q) - m + 1)
        t = time.perf_counter()
        o.search(q[s0:s0 + m], k=k, nprobe=p, survivors=S)
        tot_t += time.perf_counter() - t
    value = m * args.steps / tot_t
    sample = (f"the whole {len(q)}-query batch per step" if m == len(q) else
              f"{m} of the {len(q)} batch queries per step (whole batches would exceed "
              f"{args.ref_seconds:.0f} s)")
    out = {"impl": "reference", "metric": metric_name(args.config, args.n, args.dim, B),
           "value": round(value, 1), "unit": "queries/s",
           "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": round(tot_t / args.steps * 1e3, 3), "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "u8",
           "data": WORKLOADS[args.config]["data"] + " (the same seeded workload as the GPU arm)",
           "config": {"workload": workload_name(args.n, args.dim, args.nlist, B, k),
                      "nprobe_path": "fixed",
                      "nprobe": p, "survivors": S, "prefix_dims": args.head,
                      "setting_rule": "fastest fixed setting at recall@10 >= 0.99 over the sweep"},
           "recall": pick["recall"],
           "sweep": sweep,
           "cpu_baseline": {"value": round(value, 1), "unit": "queries/s", "cores": cores, "kind": "port",
                            "sample": sample, "isa": platform.machine()},
           "e2e": {"value": round(value, 1), "unit": "queries/s", "h2d_bytes_per_step": 0,
                   "d2h_bytes_per_step": 0},
           "setup_s": round(setup_s, 1), "oracle_coding_s": round(load_s, 1),
           "sweep_s": round(sweep_s, 1),
           "index_coding": "the oracle, from the float vectors (no repository library loaded)"}
    print(json.dumps(out))


if __name__ == "__main__":
    main()
