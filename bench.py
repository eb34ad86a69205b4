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

--impl reference times the reference's algorithm on the host cores (the
oracle port in oracle/, all threads) on a bounded sample of the same
workload and extrapolates it to the full size; see `sample` in its line.
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
SAMPLE_N = 65_536  # CPU-baseline sample of the same generator
SAMPLE_N_ONE_THREAD = 16_384  # its one-thread sample
RECALL_QUERIES = 10_000  # recall@15 sample against FP64 exact search
# DRAM bytes (read + write) of one full-size BF16 kNN-selection launch, from the
# ncu capture in profiles/knn_select_tc_1024000x100_dram.md.
KNN_TRAFFIC_BYTES = 9.60e9


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

def cpu_sample_pipeline(threads, steps, warmup, log=print, n_sample=SAMPLE_N, knn_threads=0):
    """The reference's algorithm (oracle port, `threads` host threads) on an
    n_sample-point sample of the workload: kNN once (brute force, reported,
    not in the value), then per step symmetrize + build_edges + init +
    optimize, extrapolated linearly to N_FULL (all four are O(E)).  The
    untimed kNN runs on knn_threads threads (default: `threads`)."""
    from oracle import oracle as O
    from ncvis_gb300.api import default_noise_plan, find_ab_params
    X = workload(n_sample)
    a, b = find_ab_params(1.0, 0.4)
    plan = default_noise_plan(EPOCHS).astype(np.uint64)
    t = time.perf_counter()
    Xp = O.preprocess(X, 2)
    knn_threads = knn_threads or threads
    inds, dists = O.knn(Xp, 2, K_NN, use_f64=False, n_threads=knn_threads)
    t_knn = time.perf_counter() - t
    times = []
    for s in range(warmup + steps):
        t0 = time.perf_counter()
        rp, cols, _ = O.symmetrize(inds, dists, n_threads=threads)
        src = O.edges_from_csr(rp)
        Y = O.init_embedding(n_sample, D_EMB, src, cols, 42, INIT_EPOCHS, np.float32(1 / K_NN),
                             threads)
        O.optimize(Y, 0.0, src, cols, 42, plan, a, b, n_threads=threads)
        dt = time.perf_counter() - t0
        if s >= warmup:
            times.append(dt)
        log(f"cpu step {s}: {dt:.2f}s (E={src.size})")
    per_step = statistics.median(times)
    scale = N_FULL / n_sample
    return {
        "value": per_step * scale,
        "unit": "s",
        "cores": threads,
        "kind": "port",
        "sample": (f"{n_sample} points of the same vMF generator; symmetrize+build_edges+init+"
                   f"optimize timed ({per_step:.2f}s median of {len(times)}) and scaled by "
                   f"N_full/N_sample={scale:.2f} (O(E) stages); the reference's HNSW kNN is "
                   f"unavailable (hnswlib absent) and excluded, so this is a lower bound of its "
                   f"fit_transform time; brute-force FP32 kNN of the sample took {t_knn:.2f}s "
                   f"on {knn_threads} threads"),
        "sample_step_s": per_step,
        "knn_bruteforce_sample_s": t_knn,
        "edges_sample": int(src.size),
    }


def run_reference(args):
    world, rank, _ = dist_env()
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    res = cpu_sample_pipeline(threads, args.steps, args.warmup, log=lambda m: print(m, file=sys.stderr))
    line = {
        "impl": "reference", "metric": "fit_transform_seconds", "value": res["value"], "unit": "s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": res["value"] * 1000.0, "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded vMF mixture)",
        "config": config(N_FULL, args.knn),
        "cpu_baseline": {k: res[k] for k in ("value", "unit", "cores", "kind", "sample")},
        "e2e": {"value": res["value"], "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


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
    achieved = flops / (knn_ms / 1000.0) / 1e12
    roof.update({"kernel": "knn candidate selection", "achieved": achieved, "peak": peak,
                 "frac": achieved / peak,
                 "traffic": KNN_TRAFFIC_BYTES if (n == N_FULL and args.knn == "bf16") else None,
                 "traffic_unit": "DRAM bytes per launch (ncu)",
                 "algorithmic": f"2*N^2*D = {flops:.3e} FLOP per launch (D=100 unpadded)"})
    if args.knn == "ivf":
        # The inverted file computes a data-dependent fraction of the N^2 pairs:
        # the exact search's FLOP count does not describe it.
        roof.update({"achieved": None, "frac": None,
                     "algorithmic": "data-dependent (probed cells); see recall_at_15"})
    sgd_bytes = E * (EPOCHS * 4 + 16 * D_EMB * int((plan + 1).sum()))
    sgd_gbs = sgd_bytes / (opt_ms / 1000.0) / 1e9
    hbm = peaks.get("hbm_gbs", 6800.0)

    recall = None
    inds = None
    if not args.no_recall:
        if args.knn == "ivf":
            inds, _ = stages.knn_ivf(Xd, K_NN, 2)
        else:
            inds, _ = stages.knn(Xd, K_NN, 2, precision=1 if args.knn == "bf16" else 0)
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
        # X's table: the one measured above against FP64 (recall_at_15), else exact FP32.
        x_inds = inds if inds is not None else stages.knn(Xd, K_NN, 2, precision=0)[0]
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

    cpu = None
    small = None
    if not args.no_cpu_baseline and world == 1:
        cpu_full = cpu_sample_pipeline(os.cpu_count() or 1, 1, 0, log=lambda m: print(m, file=sys.stderr))
        cpu = {k: cpu_full[k] for k in ("value", "unit", "cores", "kind", "sample")}
        # The same port on one thread (a smaller sample keeps it near 10 s).
        one = cpu_sample_pipeline(1, 1, 0, log=lambda m: print(m, file=sys.stderr),
                                  n_sample=SAMPLE_N_ONE_THREAD, knn_threads=os.cpu_count() or 1)
        cpu["one_thread"] = {k: one[k] for k in ("value", "unit", "cores", "sample")}
        small = small_config(dev)

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
                "algorithmic_GBps": sgd_gbs, "hbm_peak_GBps": hbm, "frac_of_hbm": sgd_gbs / hbm,
                **update_ceiling(n, pair_updates / (opt_ms / 1000.0), E * EPOCHS, opt_ms),
                "noise": ("staged in shared-memory windows" if args.sgd == "hogwild"
                          else "each sample read from the whole embedding"),
                "E": E},
        "recall_at_15": recall,
        "recall_queries": None if recall is None else min(RECALL_QUERIES, n),
        "quality": quality,
        "stage_ms": {k: statistics.mean(s[k] for s in stage_list) for k in
                     ("preprocess_ms", "knn_ms", "rerank_ms", "symmetrize_ms", "init_ms",
                      "optimize_ms")},
        "cpu_baseline": cpu,
        "small_config": small,
        "clocks": clk.summary(),
        "gpu_launches": int(launches),
    }
    print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


def run_nce(args):
    """Forward + backward of the NCE loss (torch.autograd.Function over the
    engine's kernels) over the symmetrized 15-NN graph of a 200,000-point,
    64-D, 10-component Gaussian mixture, Y ~ N(0, 1e-4 I), Q = 1, 5 noise
    samples per edge, batches of 2^20 edges; one step = one pass over all
    edges.  Throughput in (positive + noise) samples per second."""
    import torch
    import ncvis_gb300 as ncvis
    from ncvis_gb300 import nce, stages
    from ncvis_gb300.synthetic import gaussian_mixture
    dev = torch.device("cuda", 0)
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
        for it in range(args.warmup):
            step(it)
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for it in range(args.steps):
            step(100 + it)
        b.record()
        torch.cuda.synchronize()
        ms = a.elapsed_time(b) / args.steps
        samples = E * 6
        lines.append({"d": d, "ms_per_pass": ms, "samples_per_s": samples / (ms / 1e3),
                      "edges": int(E), "batches": (E + batch - 1) // batch})
    print(json.dumps({"metric": "nce_fwd_bwd_samples_per_s", "value": lines[0]["samples_per_s"],
                      "unit": "samples/s", "higher_is_better": True, "n_gpus": 1,
                      "steps": args.steps, "warmup": args.warmup, "dtype": "f32",
                      "data": "synthetic (seeded Gaussian mixture)",
                      "config": {"workload": "NCE loss fwd+bwd, N=200000 D=64 GMM 15-NN graph, "
                                             "5 noise samples, batches of 2^20 edges"},
                      "per_dim": lines}), flush=True)
    return 0


def run_batched(args):
    """256 independent embeddings (N log-uniform in [500, 50000], D=64
    Gaussian mixtures with 4-20 components, per-problem seeds, k=15, d=2,
    50 epochs) in one run, against looping the single-problem path; pair
    updates per second over the whole job."""
    import torch
    import ncvis_gb300 as ncvis
    from ncvis_gb300.synthetic import gaussian_mixture
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(42)
    sizes = np.exp(rng.uniform(np.log(500), np.log(50000), 256)).astype(int)
    Xs = [torch.from_numpy(gaussian_mixture(int(n), 64, int(rng.integers(4, 21)), 5.0, 1.0,
                                            seed=42 + p)[0]).to(dev) for p, n in enumerate(sizes)]
    seeds = list(range(42, 42 + len(Xs)))
    vis = ncvis.NCVis(random_seed=42, knn_precision=args.knn)
    for _ in range(args.warmup):
        vis.fit_transform_batched(Xs, seeds=seeds)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        vis.fit_transform_batched(Xs, seeds=seeds)
    torch.cuda.synchronize()
    wall = (time.perf_counter() - t0) / args.steps
    st = vis.stage_times()
    plan_sum = int((vis.noise_plan.astype(np.int64) + 1).sum())
    updates = st["n_edges"] * plan_sum
    t0 = time.perf_counter()
    for p, x in enumerate(Xs):
        ncvis.NCVis(random_seed=42 + p).fit_transform(x)
    torch.cuda.synchronize()
    loop = time.perf_counter() - t0
    print(json.dumps({"metric": "batched_pair_updates_per_s", "value": updates / wall,
                      "unit": "pair-updates/s", "higher_is_better": True, "n_gpus": 1,
                      "steps": args.steps, "warmup": args.warmup, "dtype": "f32",
                      "data": "synthetic (seeded Gaussian mixtures)",
                      "config": {"workload": "256 embeddings, N log-uniform [500, 50000], D=64, "
                                             "k=15, d=2, 50 epochs", "total_N": int(sizes.sum()),
                                 "knn": ("BF16 tcgen05 + exact FP32 rerank (batched problems "
                                         "run the exact search in every BF16 mode)"
                                         if args.knn != "fp32" else "exact FP32"),
                                 "loop": "plain per-problem path (exact FP32 kNN), one fit each"},
                      "wall_s": wall, "stage_ms": st, "loop_of_single_fits_s": loop,
                      "loop_pair_updates_per_s": updates / loop, "speedup_vs_loop": loop / wall}),
          flush=True)
    return 0


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
