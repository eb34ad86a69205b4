"""Benchmark of the NCVis fit_transform hot path on GB300.

Headline workload: fit_transform of N=1,024,000 x D=100 float32 unit vectors
from a 128-component von Mises-Fisher mixture (kappa=50, Dirichlet(1)
weights, seed 42), cosine distance, n_neighbors=15, d=2, 50 epochs, 20 init
epochs, the reference's default noise plan and a/b (spread 1, min_dist 0.4).

One step = one full fit_transform (preprocess, kNN, symmetrize, init, SGD)
on inputs already resident in HBM (X is 410 MB, larger than the 129 MB L2, so
no explicit flush is needed between steps).  `e2e` times the same call
through the C ABI with pinned host buffers (the H2D copy of X and the D2H
copy of Y inside the timed region).  With --gpus N > 1 (one rank per GPU
under torchrun) every rank embeds its own replica: the path shards only in
its kNN stage, so replicas are what scale here.

--impl reference times the reference's algorithm after its kNN on the host
cores (the oracle port in oracle/, all threads) at the full workload, every
step timed, nothing extrapolated; the reference's kNN (HNSW) is absent and
its input table is made before the timed region (see `config.knn` and
`cpu_baseline.sample` in its line).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_FULL, D_FULL, K_NN, D_EMB, EPOCHS, INIT_EPOCHS = 1_024_000, 100, 15, 2, 50, 20
ONE_THREAD_N = 32_768  # points of the one-thread CPU figure
RECALL_QUERIES = 10_000  # recall@15 sample against FP64 exact search
# DRAM bytes (read + write) of one full-size BF16 kNN-selection launch, from a
# one-pass ncu capture (dram__bytes_read.sum + dram__bytes_write.sum).
KNN_TRAFFIC_BYTES = 250.94e9


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--knn", choices=["fp32", "bf16", "ivf"], default="bf16",
                   help="exact FP32, exact BF16 tensor-core selection + FP32 rerank (default), or "
                        "the approximate inverted-file search (default cells and probes)")
    p.add_argument("--sgd", choices=["hogwild", "hogwild_unstaged"], default="hogwild",
                   help="optimizer noise: staged in shared-memory windows (default) or read "
                        "from the whole embedding")
    p.add_argument("--n", type=int, default=N_FULL, help="points (default: the full workload)")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-recall", action="store_true")
    p.add_argument("--workload", choices=["fit", "nce", "batched"], default="fit",
                   help="fit: the headline fit_transform; nce: the differentiable loss at "
                        "N=200,000; batched: 256 independent embeddings in one run")
    p.add_argument("--no-quality", action="store_true",
                   help="skip the quality comparison against the plain FP32 path")
    p.add_argument("--no-extras", action="store_true",
                   help="skip the other configurations (131,072 x 100 kNN, NCE loss, batched)")
    return p.parse_args()


def workload(n):
    from ncvis_gb300.synthetic import vmf_mixture
    X, _ = vmf_mixture(n, D_FULL, n_comp=128, kappa=50.0, seed=42)
    return X


def config(n, knn):
    return {
        "workload": f"fit_transform N={n} D={D_FULL} vMF mixture (128 comps, kappa=50), cosine, "
                    f"n_neighbors={K_NN}, d={D_EMB}, {EPOCHS} epochs, {INIT_EPOCHS} init epochs",
        "knn": {"fp32": "exact FP32", "bf16": "BF16 tcgen05 + exact FP32 rerank",
                "ivf": "approximate: inverted file (k-means cells) on BF16 tcgen05 + exact FP32 "
                       "rerank"}[knn],
        "noise_plan": "reference default (sum 262)",
        "l2": "inputs larger than L2 (X 410 MB)",
        "parallelism": "replicas (one independent embedding per GPU)",
    }


# ------------------------------------------------------------------ clocks

class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    def __init__(self, path, index):
        self.path, self.index, self.proc = path, index, None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.fh, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            self.proc.wait()
            self.fh.close()

    def summary(self):
        if not self.proc or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append((float(parts[1]), float(parts[2]), parts[5:9]))
            except ValueError:
                continue
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        seen = sorted({n for _, _, flags in rows for n, f in zip(names, flags) if f == "Active"})
        return {"sm_mhz": statistics.median(r[0] for r in rows), "sm_max_mhz": max(r[1] for r in rows),
                "reasons": seen, "samples": len(rows)}


# --------------------------------------------------------- distributed glue

def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def max_over_ranks(value: float, device=None) -> float:
    """Maximum of `value` over all ranks (identity without a process group)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return value
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(device=None):
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized():
        if device is not None and str(device).startswith("cuda"):
            dist.barrier(device_ids=[device.index])
        else:
            dist.barrier()


# ------------------------------------------------------- CPU (reference) arm

def reference_table(Xp, k=K_NN, log=print):
    """The CPU arm's input kNN table, made before its timed region.  The
    reference builds it with hnswlib (src/ncvis.cpp:72-153), whose source is
    absent, so this is an exact search with the reference's row contract (the
    k + 1 nearest by 1 - <x, y> on the preprocessed rows, the nearest dropped,
    descending order) in FP32 GEMMs by torch: on the GPU where there is one (a
    host brute force at 1,024,000 points takes far longer than the arm's run
    on these cores), else on the host.  Returns (inds int64, dists f32,
    seconds, where)."""
    import torch
    dev = "cuda" if torch.cuda.is_available() else "cpu"
    t0 = time.perf_counter()
    X = torch.from_numpy(Xp).to(dev)
    N = X.shape[0]
    inds = np.empty((N, k), np.int64)
    dists = np.empty((N, k), np.float32)
    block = 4096 if dev == "cuda" else 1024
    for s in range(0, N, block):
        d = 1.0 - X[s:s + block] @ X.T
        v, i = torch.topk(d, k + 1, dim=1, largest=False, sorted=True)
        inds[s:s + block] = i[:, 1:].flip(1).cpu().numpy()
        dists[s:s + block] = v[:, 1:].flip(1).cpu().numpy()
        del d
    del X
    if dev == "cuda":
        torch.cuda.synchronize()
        torch.cuda.empty_cache()
    t = time.perf_counter() - t0
    log(f"reference input table: {N} points in {t:.1f}s ({dev})")
    return inds, dists, t, dev


def cpu_pipeline(inds, dists, threads, steps, warmup, log=print):
    """The reference's algorithm after its kNN (the oracle port, compiled
    C++, `threads` host threads): per step symmetrize + build_edges +
    init_embedding + optimize on the given table (src/knntable.cpp:24-99,
    src/ncvis.cpp:155-352), timed with the host clock.  Returns the mean
    step time of the timed steps, the edge count, the per-stage times of the
    last step and its symmetrized CSR (row_ptr, cols, vals; the same for any
    thread count)."""
    from oracle import oracle as O
    from ncvis_gb300.api import default_noise_plan, find_ab_params
    a, b = find_ab_params(1.0, 0.4)
    plan = default_noise_plan(EPOCHS).astype(np.uint64)
    N = inds.shape[0]
    times, stages, csr, E = [], {}, None, 0
    for s in range(warmup + steps):
        t0 = time.perf_counter()
        rp, cols, vals = O.symmetrize(inds, dists, n_threads=threads)
        src = O.edges_from_csr(rp)
        t1 = time.perf_counter()
        Y = O.init_embedding(N, D_EMB, src, cols, 42, INIT_EPOCHS, np.float32(1 / K_NN), threads)
        t2 = time.perf_counter()
        O.optimize(Y, 0.0, src, cols, 42, plan, a, b, n_threads=threads)
        t3 = time.perf_counter()
        if s >= warmup:
            times.append(t3 - t0)
        stages = {"symmetrize_build_edges_s": t1 - t0, "init_s": t2 - t1, "optimize_s": t3 - t2}
        E = int(src.size)
        csr = (rp, cols, vals)
        log(f"cpu step {s}: {t3 - t0:.2f}s (N={N}, E={E}, {threads} threads)")
    return statistics.mean(times), E, stages, csr


def run_reference(args):
    """The reference arm: the reference's algorithm after its kNN
    (symmetrize, build_edges, init, optimize; the oracle port, compiled C++)
    at the full workload on all host cores, every step timed, nothing
    extrapolated.  Its kNN (HNSW) is unavailable; the input table is made
    before the timed region.  Rank 0 alone runs it."""
    world, rank, _ = dist_env()
    if rank != 0:
        return 0
    from oracle import oracle as O
    threads = os.cpu_count() or 1
    log = lambda m: print(m, file=sys.stderr)  # noqa: E731
    n = args.n
    Xp = O.preprocess(workload(n), 2)
    inds, dists, t_table, where = reference_table(Xp, log=log)
    del Xp
    per_step, E, st, _ = cpu_pipeline(inds, dists, threads, args.steps, args.warmup, log=log)
    cfg = config(n, args.knn)
    cfg["knn"] = (f"not in the timed region: the reference's HNSW is unavailable (hnswlib "
                  f"absent); its input table came from an exact FP32 search (torch GEMMs on the "
                  f"{'GPU' if where == 'cuda' else 'host'}, {t_table:.1f}s) made before it")
    sample = (f"all {n} points, every step timed (no extrapolation): symmetrize + build_edges + "
              f"init_embedding + optimize (E={E}); the kNN is excluded")
    line = {
        "impl": "reference", "metric": "fit_transform_seconds", "value": per_step, "unit": "s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": per_step * 1000.0, "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded vMF mixture)",
        "config": cfg,
        "cpu_baseline": {"value": per_step, "unit": "s", "cores": threads, "kind": "port",
                         "sample": sample, "stages_last_step": st},
        "e2e": {"value": per_step, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def cpu_baseline_and_parity(inds, dists, log):
    """The GPU arm's cpu_baseline leg and its parity checks, after the timed
    region.

    * cpu_baseline: one full-size step of the reference's algorithm after the
      kNN (the oracle port) on all host cores, on the engine's own kNN table
      of this workload; and the same port on one thread at 32,768 points of
      the same generator (measured there, not scaled).
    * parity: the same table through the GPU symmetrization against that
      step's CSR (src/knntable.cpp:24-99 and build_edges,
      src/ncvis.cpp:155-173), bit for bit (row_ptr, columns in order,
      distance bits, sources); then init_embedding on that graph
      (src/ncvis.cpp:184-273) within 1e-5 * max(1, max|Y|): with the
      statistics summed in the reference's one-thread FP32 order against the
      oracle's one-thread init, and the default (FP64 statistics) against the
      oracle with its sums in double; the default's gap to the reference
      (the FP32 sums' drift at this size) is reported beside them."""
    from ncvis_gb300 import stages
    from oracle import oracle as O
    ti, td = inds.cpu().numpy().astype(np.int64), dists.cpu().numpy()
    threads = os.cpu_count() or 1
    per_step, E, st, (orp, ocols, ovals) = cpu_pipeline(ti, td, threads, 1, 0, log=log)
    Xs = O.preprocess(workload(ONE_THREAD_N), 2)
    si, sd, _, _ = reference_table(Xs, log=log)
    one, E1, _, _ = cpu_pipeline(si, sd, 1, 1, 0, log=log)
    baseline = {
        "value": per_step, "unit": "s", "cores": threads, "kind": "port",
        "sample": (f"one step of the full {ti.shape[0]}-point workload: symmetrize + build_edges + "
                   f"init_embedding + optimize (E={E}) on the engine's kNN table; the reference's "
                   f"HNSW kNN is unavailable and excluded"),
        "stages": st,
        "one_thread": {"value": one, "unit": "s", "cores": 1, "n": ONE_THREAD_N, "E": E1,
                       "sample": f"{ONE_THREAD_N} points of the same generator, measured there"},
    }
    t0 = time.perf_counter()
    rp, cols, vals, src = stages.symmetrize(inds, dists)
    osrc = O.edges_from_csr(orp)
    same = bool(np.array_equal(rp.cpu().numpy(), orp)
                and np.array_equal(cols.cpu().numpy().astype(np.int64), ocols)
                and np.array_equal(vals.cpu().numpy().view(np.uint32), ovals.view(np.uint32))
                and np.array_equal(src.cpu().numpy().astype(np.int64), osrc))
    N = orp.size - 1
    alpha = np.float32(1 / K_NN)
    Ys = stages.init_embedding(rp, cols, D_EMB, 42, INIT_EPOCHS, alpha,
                               sequential_stats=True).cpu().numpy()
    Yd = stages.init_embedding(rp, cols, D_EMB, 42, INIT_EPOCHS, alpha).cpu().numpy()
    Yo = O.init_embedding(N, D_EMB, osrc, ocols, 42, INIT_EPOCHS, alpha, 1)
    Yo64 = O.init_embedding(N, D_EMB, osrc, ocols, 42, INIT_EPOCHS, alpha, 1, stats64=True)
    e_seq = float(np.abs(Ys - Yo).max())
    e_def = float(np.abs(Yd - Yo64).max())
    tol = 1e-5 * max(1.0, float(np.abs(Yo).max()))
    log(f"parity checks: {time.perf_counter() - t0:.1f}s")
    parity = {"table": "the engine's kNN table of this workload (its fit's kNN path)",
              "csr_bit_exact": same, "E": int(orp[-1]),
              "rows_over_64_items": int((np.diff(orp) > 64).sum()),
              "init_tol": tol,
              "init_sequential_stats_vs_reference": e_seq,
              "init_default_vs_double_sums": e_def,
              "init_within_tol": bool(e_seq <= tol and e_def <= tol),
              "init_default_vs_reference": float(np.abs(Yd - Yo).max()),
              "reference_vs_double_sums": float(np.abs(Yo - Yo64).max())}
    return baseline, parity


# ------------------------------------------------------------------ GPU arm

def recall_at_15(Xd, inds, n_queries=RECALL_QUERIES, seed=0):
    """recall@15 of the engine's kNN table against FP64 exact search for a
    query subsample, same row contract (k+1 nearest by (distance, index),
    nearest dropped).  The FP64 distances are computed on the GPU with torch
    (a plain FP64 GEMM, after the timed region): 10,000 queries against
    1,024,000 points are 2e12 FLOP, minutes on the host."""
    import torch
    N = Xd.shape[0]
    n_queries = min(n_queries, N)
    rng = np.random.default_rng(seed)
    q = np.sort(rng.choice(N, n_queries, replace=False))
    X64 = Xd.double()
    X64 /= X64.norm(dim=1, keepdim=True)
    block = max(64, min(512, int(2e9 // (8 * N))))
    hits = 0
    for s in range(0, n_queries, block):
        qs = q[s:s + block]
        dist = 1.0 - X64[torch.as_tensor(qs, device=Xd.device)] @ X64.T
        vals, idx = torch.topk(dist, K_NN + 2, dim=1, largest=False)
        vals, idx = vals.cpu().numpy(), idx.cpu().numpy()
        order = np.lexsort((idx, vals), axis=-1)[:, :K_NN + 1]
        exact = np.take_along_axis(idx, order, 1)[:, 1:]
        found = np.asarray(inds[qs], dtype=np.int64)
        hits += int((found[:, :, None] == exact[:, None, :]).sum())
        del dist
    del X64
    return hits / (n_queries * K_NN)


def update_ceiling(rows, rate, positive_pairs, opt_ms):
    """The GPU's rate for the optimizer's per-sample traffic (a random row
    gather plus a random row reduction over an L2-resident array of `rows`
    2-float rows), measured live; the SGD's pair-update rate as a fraction of
    it; and the floor it sets for the positive samples alone (every positive
    sample is such a random gather + reduction; staged noise samples are
    served from shared memory)."""
    import ctypes as C
    from ncvis_gb300 import _lib
    g, u = C.c_double(0), C.c_double(0)
    rc = _lib.lib().ncvis_measure_update_rate(rows, D_EMB, C.byref(g), C.byref(u), None)
    if rc != 0:
        return {"update_ceiling_error": _lib.lib().ncvis_get_last_error().decode()}
    floor_ms = positive_pairs / u.value * 1e3
    return {"gather_ceiling_per_s": g.value, "update_ceiling_per_s": u.value,
            "frac_of_update_ceiling": rate / u.value, "positive_floor_ms": floor_ms,
            "frac_of_positive_floor": floor_ms / opt_ms}


def small_config(dev):
    """The reference's own CPU-runnable case, whole fit_transform on both sides:
    10,000 x 64 float32 points of a 10-component Gaussian mixture (centres
    ~ N(0, 25 I), sigma 1, equal weights, seed 42) at the reference's defaults
    (squared L2, k=15, d=2, 50 epochs, 20 init epochs, default noise plan and
    a/b).  GPU: the plain FP32 path (the drop-in), median of 5 device-timed
    fits.  CPU: the oracle (the reference's algorithm restated; brute-force
    kNN where the reference uses HNSW) on all host threads, median of 3."""
    import torch
    import ncvis_gb300 as ncvis
    from ncvis_gb300.api import default_noise_plan, find_ab_params
    from ncvis_gb300.synthetic import gaussian_mixture
    from oracle import oracle as O
    X, _ = gaussian_mixture(10_000, 64, 10, 5.0, 1.0, seed=42)
    Xd = torch.from_numpy(X).to(dev)
    vis = ncvis.NCVis(random_seed=42)
    for _ in range(2):
        vis.fit_transform(Xd)
    gpu = []
    for _ in range(5):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        vis.fit_transform(Xd)
        b.record()
        torch.cuda.synchronize()
        gpu.append(a.elapsed_time(b) / 1000.0)
    av, bv = find_ab_params(1.0, 0.4)
    plan = default_noise_plan(EPOCHS).astype(np.uint64)
    threads = os.cpu_count() or 1
    cpu = []
    for _ in range(3):
        t = time.perf_counter()
        O.fit_transform(X, 2, K_NN, 42, EPOCHS, INIT_EPOCHS, av, bv, 1.0, 1.0, plan, 0, threads)
        cpu.append(time.perf_counter() - t)
    g, c = statistics.median(gpu), statistics.median(cpu)
    return {"workload": "fit_transform 10,000 x 64 Gaussian mixture, reference defaults "
                        "(squared L2, k=15, d=2, 50 epochs)",
            "gpu_plain_fp32_s": g, "cpu_reference_algorithm_s": c, "cpu_threads": threads,
            "cpu_knn": "brute force (the reference's HNSW is unavailable)",
            "speedup": c / g}


def run_ours(args):
    import torch
    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)
    import ncvis_gb300 as ncvis
    from ncvis_gb300 import _lib, stages

    n = args.n
    X = workload(n)
    Xd = torch.from_numpy(X).to(dev)
    vis = ncvis.NCVis(d=D_EMB, n_neighbors=K_NN, n_epochs=EPOCHS, n_init_epochs=INIT_EPOCHS,
                      random_seed=42, distance="cosine", knn_precision=args.knn,
                      sgd_mode=args.sgd)
    for _ in range(args.warmup):
        vis.fit_transform(Xd)
    torch.cuda.synchronize()

    L = _lib.lib()
    stage_list = []
    clocks_path = os.environ.get("NCVIS_CLOCKS_CSV", f"/tmp/ncvis_clocks_rank{rank}_{os.getpid()}.csv")
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier(dev)
    torch.cuda.synchronize()
    launches0 = L.ncvis_kernel_launch_count()
    with ClockSampler(clocks_path, local) as clk:
        start.record()
        for _ in range(args.steps):
            vis.fit_transform(Xd)
            stage_list.append(vis.stage_times())
        stop.record()
        torch.cuda.synchronize()
    launches = L.ncvis_kernel_launch_count() - launches0
    barrier(dev)
    step_s = start.elapsed_time(stop) / 1000.0 / args.steps
    step_s = max_over_ranks(step_s, dev)

    # e2e through the C ABI with pinned host buffers.
    Xh = torch.from_numpy(X).pin_memory()
    Yh = torch.empty((n, D_EMB), dtype=torch.float32).pin_memory()
    import ctypes as C
    L.ncvis_fit_transform(vis._h, Xh.data_ptr(), n, D_FULL, Yh.data_ptr())  # warm host path
    e2e_times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        rc = L.ncvis_fit_transform(vis._h, Xh.data_ptr(), n, D_FULL, Yh.data_ptr())
        e2e_times.append(time.perf_counter() - t0)
        _lib.check(rc, vis._h)
    e2e_s = max_over_ranks(statistics.mean(e2e_times), dev)

    if rank != 0:
        return 0

    knn_ms = statistics.mean(s["knn_ms"] for s in stage_list)
    opt_ms = statistics.mean(s["optimize_ms"] for s in stage_list)
    E = int(stage_list[-1]["n_edges"])
    plan = vis.noise_plan.astype(np.int64)
    pair_updates = E * int((plan + 1).sum())
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except OSError:
        pass
    flops = 2.0 * n * n * D_FULL
    if args.knn in ("bf16", "ivf"):
        peak = peaks.get("bf16_tflops_sustained", 1700.0)
        roof = {"bound": "tensor", "unit": "TFLOP/s",
                "peak_source": "bf16_tflops_sustained of measured" if peaks else "fallback"}
    else:
        # No measured FP32-SIMT peak exists; nominal FFMA rate.
        peak = 152 * 128 * 2 * 2.07e9 / 1e12
        roof = {"bound": "fp32_simt", "unit": "TFLOP/s",
                "peak_source": "nominal FP32 FFMA (152 SMs x 128 lanes x 2 flop x 2.07 GHz)"}
    # The selection kernel's own time: the kNN stage minus the k-means cell
    # ordering that precedes the sweep (CUDA events on the engine's stream).
    order_ms = statistics.mean(s["knn_order_ms"] for s in stage_list)
    sweep_ms = knn_ms - order_ms
    achieved = flops / (sweep_ms / 1000.0) / 1e12
    roof.update({"kernel": "knn candidate selection (knn_select_tc)", "achieved": achieved,
                 "peak": peak, "frac": achieved / peak,
                 "traffic": KNN_TRAFFIC_BYTES if (n == N_FULL and args.knn == "bf16") else None,
                 "traffic_unit": "DRAM bytes per launch (ncu)",
                 "kernel_ms": sweep_ms, "cell_ordering_ms": order_ms,
                 "frac_of_knn_stage": flops / (knn_ms / 1000.0) / 1e12 / peak,
                 "algorithmic": f"2*N^2*D = {flops:.3e} FLOP per launch (D=100 unpadded)"})
    if args.knn == "ivf":
        # The inverted file computes a data-dependent fraction of the N^2 pairs:
        # the exact search's FLOP count does not describe it.
        roof.update({"achieved": None, "frac": None,
                     "algorithmic": "data-dependent (probed cells); see recall_at_15"})
    log = lambda m: print(m, file=sys.stderr)  # noqa: E731

    # The engine's kNN table of this workload (the fit's own kNN path).
    if args.knn == "ivf":
        inds, dists = stages.knn_ivf(Xd, K_NN, 2)
    else:
        inds, dists = stages.knn(Xd, K_NN, 2, precision=1 if args.knn == "bf16" else 0)
    recall = None
    if not args.no_recall:
        recall = recall_at_15(Xd, inds.cpu().numpy())

    quality = None
    if not args.no_quality:
        # Embedding quality at k=15 of this path and of the plain FP32 path
        # (one extra fit): kNN preservation and trustworthiness on all points
        # (exact kNN of X and of Y, and every neighbour's rank, on the GPU),
        # and trustworthiness of a 10,000-point sample by FP64 brute force.
        from ncvis_gb300 import quality as Qm
        Y_ours = vis.fit_transform(Xd)
        plain = ncvis.NCVis(d=D_EMB, n_neighbors=K_NN, n_epochs=EPOCHS, n_init_epochs=INIT_EPOCHS,
                            random_seed=42, distance="cosine", knn_precision="fp32",
                            sgd_mode="hogwild_unstaged")
        plain.fit_transform(Xd)  # warm-up (arena, kernels)
        torch.cuda.synchronize()
        t_plain = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t_plain[0].record()
        Y_plain = plain.fit_transform(Xd)
        t_plain[1].record()
        torch.cuda.synchronize()
        plain_s = t_plain[0].elapsed_time(t_plain[1]) / 1000.0
        plain_stages = plain.stage_times()
        # X's table: the one measured above against FP64 (recall_at_15).
        x_inds = inds
        sub = np.sort(np.random.default_rng(1).choice(n, min(n, 10000), replace=False))
        Xs = X[sub] / np.linalg.norm(X[sub], axis=1, keepdims=True)
        quality = {
            "k": K_NN,
            "plain_fp32_path_fit_s": plain_s,
            "plain_fp32_path_knn_ms": plain_stages["knn_ms"],
            "speedup_vs_plain_fp32_path": plain_s / step_s,
            "knn_preservation_full": {
                "this_path": Qm.knn_preservation_device(Xd, Y_ours, K_NN, 2, x_inds=x_inds),
                "plain_fp32_path": Qm.knn_preservation_device(Xd, Y_plain, K_NN, 2, x_inds=x_inds)},
            "trustworthiness_full": {
                "this_path": Qm.trustworthiness_device(Xd, Y_ours, K_NN, distance=2),
                "plain_fp32_path": Qm.trustworthiness_device(Xd, Y_plain, K_NN, distance=2)},
            "trustworthiness_sample10k": {
                "this_path": Qm.trustworthiness(Xs, Y_ours[sub].cpu().numpy(), K_NN),
                "plain_fp32_path": Qm.trustworthiness(Xs, Y_plain[sub].cpu().numpy(), K_NN)},
        }

    cpu = parity = small = None
    if not args.no_cpu_baseline and world == 1:
        cpu, parity = cpu_baseline_and_parity(inds, dists, log)
        small = small_config(dev)
    del inds, dists
    extras = None if (args.no_extras or world > 1) else run_extras(args, dev, log)

    line = {
        "metric": "fit_transform_seconds", "value": step_s, "unit": "s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_s * 1000.0,
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32" if args.knn == "fp32" else "bf16+f32",
        "data": "synthetic (seeded vMF mixture, no dataset)", "config": config(n, args.knn),
        "e2e": {"value": e2e_s, "unit": "s", "h2d_bytes_per_step": n * D_FULL * 4,
                "d2h_bytes_per_step": n * D_EMB * 4},
        "roofline": roof,
        "sgd": {"pair_updates_per_s": pair_updates / (opt_ms / 1000.0),
                "edge_epochs_per_s": E * EPOCHS / (opt_ms / 1000.0), "optimize_ms": opt_ms,
                **update_ceiling(n, pair_updates / (opt_ms / 1000.0), E * EPOCHS, opt_ms),
                "noise": ("staged in shared-memory windows" if args.sgd == "hogwild"
                          else "each sample read from the whole embedding"),
                "E": E},
        "recall_at_15": recall,
        "recall_queries": None if recall is None else min(RECALL_QUERIES, n),
        "quality": quality,
        "parity": parity,
        "stage_ms": {k: statistics.mean(s[k] for s in stage_list) for k in
                     ("preprocess_ms", "knn_ms", "knn_order_ms", "rerank_ms", "symmetrize_ms",
                      "init_ms", "optimize_ms")},
        "cpu_baseline": cpu,
        "small_config": small,
        "extras": extras,
        "clocks": clk.summary(),
        "gpu_launches": int(launches),
    }
    print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


def nce_figures(dev, steps, warmup):
    """Forward + backward of the NCE loss (torch.autograd.Function over the
    engine's kernels) over the symmetrized 15-NN graph of a 200,000-point,
    64-D, 10-component Gaussian mixture, Y ~ N(0, 1e-4 I), Q = 1, 5 noise
    samples per edge, batches of 2^20 edges; one step = one pass over all
    edges.  Throughput in (positive + noise) samples per second, at d = 2
    and d = 16."""
    import torch
    from ncvis_gb300 import nce, stages
    from ncvis_gb300.synthetic import gaussian_mixture
    X, _ = gaussian_mixture(200_000, 64, 10, 5.0, 1.0, seed=42)
    inds, dists = stages.knn(torch.from_numpy(X).to(dev), 15, 0)
    _, cols, _, src = stages.symmetrize(inds, dists)
    E = src.shape[0]
    batch = 1 << 20
    lines = []
    for d in (2, 16):
        g = torch.Generator(device=dev).manual_seed(0)
        Y = (1e-2 * torch.randn((200_000, d), device=dev, generator=g)).requires_grad_(True)
        Q = torch.tensor(1.0, device=dev, requires_grad=True)

        def step(it):
            for b0 in range(0, E, batch):
                loss = nce.nce_loss(Y, Q, src[b0:b0 + batch], cols[b0:b0 + batch], n_noise=5,
                                    seed=it, edge_offset=b0)
                loss.backward()
        for it in range(warmup):
            step(it)
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for it in range(steps):
            step(100 + it)
        b.record()
        torch.cuda.synchronize()
        ms = a.elapsed_time(b) / steps
        samples = E * 6
        lines.append({"d": d, "ms_per_pass": ms, "samples_per_s": samples / (ms / 1e3),
                      "edges": int(E), "batches": (E + batch - 1) // batch})
    return lines


def run_nce(args):
    lines = nce_figures(torch_device(), args.steps, args.warmup)
    print(json.dumps({"metric": "nce_fwd_bwd_samples_per_s", "value": lines[0]["samples_per_s"],
                      "unit": "samples/s", "higher_is_better": True, "n_gpus": 1,
                      "steps": args.steps, "warmup": args.warmup, "dtype": "f32",
                      "data": "synthetic (seeded Gaussian mixture)",
                      "config": {"workload": "NCE loss fwd+bwd, N=200000 D=64 GMM 15-NN graph, "
                                             "5 noise samples, batches of 2^20 edges"},
                      "per_dim": lines}), flush=True)
    return 0


def batched_figures(dev, steps, warmup, knn="bf16", compare=True):
    """256 independent embeddings (N log-uniform in [500, 50000], D=64
    Gaussian mixtures with 4-20 components, per-problem seeds, k=15, d=2,
    50 epochs) in one run, against looping the single-problem path (the
    plain drop-in: exact FP32 kNN, one fit each); pair updates per second
    over the whole job, and each problem's trustworthiness at k=15 in the
    batched run against its single fit."""
    import torch
    import ncvis_gb300 as ncvis
    from ncvis_gb300 import quality as Qm
    from ncvis_gb300.synthetic import gaussian_mixture
    rng = np.random.default_rng(42)
    sizes = np.exp(rng.uniform(np.log(500), np.log(50000), 256)).astype(int)
    Xs = [torch.from_numpy(gaussian_mixture(int(n), 64, int(rng.integers(4, 21)), 5.0, 1.0,
                                            seed=42 + p)[0]).to(dev) for p, n in enumerate(sizes)]
    seeds = list(range(42, 42 + len(Xs)))
    vis = ncvis.NCVis(random_seed=42, knn_precision=knn)
    for _ in range(warmup):
        vis.fit_transform_batched(Xs, seeds=seeds)
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(steps):
        Ys = vis.fit_transform_batched(Xs, seeds=seeds)
    b.record()
    torch.cuda.synchronize()
    wall = a.elapsed_time(b) / 1000.0 / steps
    st = vis.stage_times()
    plan_sum = int((vis.noise_plan.astype(np.int64) + 1).sum())
    updates = st["n_edges"] * plan_sum
    out = {"wall_s": wall, "pair_updates_per_s": updates / wall, "stage_ms": st,
           "total_N": int(sizes.sum()), "problems": len(Xs)}
    if compare:
        singles = [ncvis.NCVis(random_seed=42 + p) for p in range(len(Xs))]
        for p, x in enumerate(Xs[:4]):
            singles[p].fit_transform(x)  # warm-up
        torch.cuda.synchronize()
        a.record()
        Y1 = [singles[p].fit_transform(x) for p, x in enumerate(Xs)]
        b.record()
        torch.cuda.synchronize()
        loop = a.elapsed_time(b) / 1000.0
        dt = np.array([Qm.trustworthiness_device(x, yb, 15, distance=0)
                       - Qm.trustworthiness_device(x, y1, 15, distance=0)
                       for x, yb, y1 in zip(Xs, Ys, Y1)])
        out.update({"loop_of_single_fits_s": loop, "speedup_vs_loop": loop / wall,
                    "loop_pair_updates_per_s": updates / loop,
                    "trustworthiness_vs_single_fit": {
                        "max_abs_diff": float(np.abs(dt).max()),
                        "mean_diff": float(dt.mean()),
                        "within_0.01": int((np.abs(dt) <= 0.01).sum())}})
    return out


def run_batched(args):
    r = batched_figures(torch_device(), args.steps, args.warmup, knn=args.knn)
    print(json.dumps({"metric": "batched_pair_updates_per_s", "value": r["pair_updates_per_s"],
                      "unit": "pair-updates/s", "higher_is_better": True, "n_gpus": 1,
                      "steps": args.steps, "warmup": args.warmup, "dtype": "f32",
                      "data": "synthetic (seeded Gaussian mixtures)",
                      "config": {"workload": "256 embeddings, N log-uniform [500, 50000], D=64, "
                                             "k=15, d=2, 50 epochs", "total_N": r["total_N"],
                                 "knn": ("BF16 tcgen05 + exact FP32 rerank (batched problems "
                                         "run the exact search in every BF16 mode)"
                                         if args.knn != "fp32" else "exact FP32"),
                                 "loop": "plain per-problem path (exact FP32 kNN), one fit each"},
                      **r}), flush=True)
    return 0


def knn_131072_figures(dev):
    """131,072 x 100 unit vectors of a 32-component vMF mixture (kappa 50),
    cosine, k = 15: the BF16 + rerank kNN inside one fit_transform (stage
    times of the selection, its cell ordering and the rerank) and recall@15
    of the engine's table against FP64 exact search over all 131,072 rows."""
    import torch
    import ncvis_gb300 as ncvis
    from ncvis_gb300 import stages
    from ncvis_gb300.synthetic import vmf_mixture
    X, _ = vmf_mixture(131_072, 100, n_comp=32, kappa=50.0, seed=42)
    Xd = torch.from_numpy(X).to(dev)
    vis = ncvis.NCVis(distance="cosine", knn_precision="bf16", random_seed=42)
    vis.fit_transform(Xd)
    st = []
    for _ in range(3):
        vis.fit_transform(Xd)
        st.append(vis.stage_times())
    inds, _ = stages.knn(Xd, K_NN, 2, precision=1)
    recall = recall_at_15(Xd, inds.cpu().numpy(), n_queries=131_072)
    knn_ms = statistics.mean(s["knn_ms"] for s in st)
    order_ms = statistics.mean(s["knn_order_ms"] for s in st)
    flops = 2.0 * 131_072 ** 2 * 100
    return {"workload": "131,072 x 100 vMF (32 comps, kappa 50), cosine, k=15, BF16 + rerank",
            "knn_ms": knn_ms, "cell_ordering_ms": order_ms, "selection_ms": knn_ms - order_ms,
            "selection_tflops": flops / ((knn_ms - order_ms) / 1e3) / 1e12,
            "rerank_ms": statistics.mean(s["rerank_ms"] for s in st),
            "fit_transform_ms": statistics.mean(s["total_ms"] for s in st),
            "recall_at_15_all_rows": recall}


def run_extras(args, dev, log):
    """The other benchmark configurations, after the headline's timed region
    (the headline value is unchanged by them)."""
    out = {}
    t0 = time.perf_counter()
    out["knn_131072x100"] = knn_131072_figures(dev)
    log(f"extras: 131,072 x 100 kNN {time.perf_counter() - t0:.1f}s")
    t0 = time.perf_counter()
    out["nce_200000"] = {"workload": "NCE loss fwd+bwd, N=200000 D=64 GMM 15-NN graph, 5 noise "
                                     "samples, batches of 2^20 edges",
                         "per_dim": nce_figures(dev, 3, 2)}
    log(f"extras: NCE {time.perf_counter() - t0:.1f}s")
    t0 = time.perf_counter()
    out["batched_256"] = {"workload": "256 embeddings, N log-uniform [500, 50000], D=64, k=15, "
                                      "d=2, 50 epochs; BF16 + rerank kNN, staged-noise SGD",
                          **batched_figures(dev, 3, 2)}
    log(f"extras: batched {time.perf_counter() - t0:.1f}s")
    return out


def torch_device():
    import torch
    return torch.device("cuda", 0)


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "nce":
        return run_nce(args)
    if args.workload == "batched":
        return run_batched(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
