#!/usr/bin/env python
"""Benchmark of the batched coherent sky scan on GB300.

Workload (one "step"): the batched sky loop of 4,096 synthetic clusters of
one segment -- pixel counts log-uniform in [20, 3000], network SNR uniform
in [8, 40], independent sky directions -- over the full HEALPix order-7 sky
(196,608 directions) with L1/H1/V1 geometry, 41 delay samples (K = 20),
float32 amplitudes.  One step = the DPF regulator and the sky scan of every
cluster (pycwb/modules/likelihoodWP/likelihood.py:310-325 for each), as one
persistent launch replayed from a CUDA graph.

Reported (one JSON line on rank 0):
  value       cluster-sky evaluations/s with inputs resident in HBM
  e2e         the same through the public API (BatchedSkyLoop.run) with the
              cluster data in pinned host memory: H2D of every step's inputs
              and D2H of the per-cluster results inside the timed region
  plain       the same kernel launched once per cluster on the same data
  roofline    FP32 work of the sky-loop kernel against the measured FP32
              FMA peak of the device
  cpu_baseline  the CPU oracle (a restatement of the reference's loops,
              OpenMP over the sky) on a bounded sample, all host cores
  skystat, stage, ...  the stage around the loop: the statistics at every
              maximum and the sky probability (device-timed), and the whole
              likelihood stage through its drop-in likelihood_wrapper on
              host cluster objects (host wall time)

--impl reference times the reference's CPU implementation (the oracle port;
the reference's own compiled code needs numba/ROOT, absent here) on the
same metric.  Under torchrun each rank evaluates its own 4,096 clusters
(weak scaling; no collective on the data path).
"""

from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

METRIC = "cluster-sky evals/s at HEALPix-7, 3 ifo: batched vs plain GPU at 1e-4 rel err"
UNIT = "cluster-sky evals/s"
IFOS = ("L1", "H1", "V1")
K_TD = 20


def scan_ops(n_ifo: int) -> int:
    """FP32 ops of the scan per (direction, pixel): 77I+108 flops + 8 sqrt +
    12 div (FMA = 2 flops, sqrt/div = 1 op), counted from sky_stat.py:37-410
    and sky_scan.py:97-179."""
    return 77 * n_ifo + 108 + 8 + 12


def reg_ops(n_ifo: int) -> int:
    """FP32 ops of the DPF regulator per (direction, pixel): 23I+18 flops +
    3 sqrt + 4 div, counted from dpf.py:343-453."""
    return 23 * n_ifo + 18 + 3 + 4


def ops_per_pair(n_ifo: int) -> int:
    """The reference's FP32 ops per (direction, pixel): scan + regulator."""
    return scan_ops(n_ifo) + reg_ops(n_ifo)


# --------------------------------------------------------------------------
# helpers
# --------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []
        self._t = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self._t = threading.Thread(target=self._read, daemon=True)
        self._t.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, power, reasons = [], [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
                power.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": float(max(smax)) if smax else None,
                "power_w_median": float(np.median(power)) if power else None,
                "samples": len(sm), "reasons": sorted(reasons)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch
        import torch.distributed as dist
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        dist.init_process_group(backend=backend)
        pg = dist
    return world, rank, local, pg


def barrier(pg):
    if pg is not None:
        pg.barrier()


def max_over_ranks(pg, value: float, device) -> float:
    if pg is None:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64, device=device)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def sky_tables_np(order: int):
    from pycwb_gb300 import sky
    ml, FP, FX = sky.compute_sky_delay_and_patterns(list(IFOS), IFOS[0], 512.0, K_TD,
                                                    healpix_order=order)
    return ml, FP.T.astype(np.float32).copy(), FX.T.astype(np.float32).copy()


def workload_config(args, sizes, n_sky):
    """The workload both arms run, the same dict in both JSON lines."""
    return {"workload": (f"batched sky loop (regulator + scan), {args.clusters} clusters, "
                         f"pixels log-uniform[20,3000], SNR U[8,40], HEALPix {args.order} "
                         f"({n_sky} directions), L1/H1/V1, 41 delays, float32"),
            "clusters": int(args.clusters), "total_pix": int(np.sum(sizes)), "n_sky": int(n_sky),
            "healpix_order": int(args.order), "n_ifo": 3, "n_delay": 2 * K_TD + 1,
            "seed": int(args.seed),
            "l2": "inputs larger than L2: 2.4 GB td amplitudes + 35 GB maps per step"}


N_CPU_SAMPLE = 32

# Per-warp pixel iterations the regulator runs, as a fraction of the full
# sum over (direction, pixel) pairs, counted in a diagnostic build on 1,024
# clusters of this workload (its early decisions stop the rest).
REG_ITER_FRACTION = 0.458


def sampled_clusters(seed, sizes, ml, FP_t, FX_t):
    """The clusters both arms time on the CPU: a size-stratified sample of the
    workload, each generated on the host from its own seed (seed, c), so the
    reference arm and the GPU arm's batch hold identical data for them."""
    from pycwb_gb300.autotune import sample_indices
    from pycwb_gb300.synthetic import make_cluster
    out = {}
    for c in sample_indices(sizes, N_CPU_SAMPLE):
        rng = np.random.default_rng([int(seed), int(c)])
        td00, td90, rms, _ = make_cluster(rng, ml, FP_t, FX_t, int(sizes[c]), K_TD,
                                          float(rng.uniform(8, 40)))
        out[int(c)] = (td00, td90, rms)
    return out


# --------------------------------------------------------------------------
# CPU baseline (the oracle: the reference's loops restated in C, OpenMP)
# --------------------------------------------------------------------------
def cpu_sample(batch, ml, FP_t, FX_t, reg, n_clusters=32, n_dirs=2048, seed=7, threads=0):
    """Oracle regulator + scan of n_clusters size-stratified clusters, each on
    n_dirs random directions.  Returns (seconds, pairs, evals)."""
    from oracle import oracle
    from pycwb_gb300.autotune import sample_indices

    oracle.build()
    rng = np.random.default_rng(seed)
    n_sky = ml.shape[1]
    idx = sample_indices(batch.sizes, n_clusters)
    REG0 = np.float32(reg["delta_regulator"] * math.sqrt(2))
    pairs = evals = 0
    t0 = time.perf_counter()
    for c in idx:
        td00, td90, rms = batch.cluster_views(int(c))
        valid = np.sort(rng.choice(n_sky, n_dirs, replace=False)).astype(np.int64)
        reg1 = oracle.calculate_dpf(FP_t, FX_t, rms, n_sky, 3, reg["gamma_regulator"],
                                    reg["network_energy_threshold"], valid, n_threads=threads)
        REG = np.array([REG0, reg1, 0.0], np.float32)
        oracle.scan_sky_for_best_fit(3, rms.shape[0], n_sky, FP_t, FX_t, rms, td00, td90, ml, REG,
                                     reg["netCC"], reg["delta_regulator"],
                                     reg["network_energy_threshold"], valid, n_threads=threads)
        pairs += rms.shape[0] * n_dirs
        evals += n_dirs
    return time.perf_counter() - t0, pairs, evals, idx


def parity_sample(res, batch, ml, FP_t, FX_t, reg, order, n_dirs=2000, seed=11):
    """The oracle against the GPU's own results on three clusters of the timed
    batch (the smallest, the median and the largest), outside the timed region.

    Per cluster: REG[1] over the whole sky must equal the oracle's; the 11 maps
    at n_dirs random directions plus the 25 directions nearest the GPU's
    maximum are compared under the parity tolerance (1e-4 relative, floor
    1e-3 of the map's largest value, plus twice the reference's own float32
    error against float64); the oracle's maximum over that sample must be the
    GPU's (or tie within 1e-5)."""
    from oracle import oracle
    from pycwb_gb300 import sky

    oracle.build()
    t0 = time.perf_counter()
    rng = np.random.default_rng(seed)
    n_sky = ml.shape[1]
    phi, lat = sky.build_sky_directions(n_sky, healpix_order=order)
    xyz = np.stack([np.cos(lat) * np.cos(phi), np.cos(lat) * np.sin(phi), np.sin(lat)], axis=1)
    srt = np.argsort(batch.sizes, kind="stable")
    picks = [int(srt[0]), int(srt[srt.size // 2]), int(srt[-1])]
    full = np.arange(n_sky, dtype=np.int64)
    REG0 = np.float32(reg["delta_regulator"] * math.sqrt(2))
    rows = []
    for c in picks:
        td00, td90, rms = batch.cluster_views(c)
        reg1 = oracle.calculate_dpf(FP_t, FX_t, rms, n_sky, 3, reg["gamma_regulator"],
                                    reg["network_energy_threshold"], full)
        lg = int(res.l_max[c])
        near = np.argsort(-(xyz @ xyz[lg]), kind="stable")[:25]
        sub = np.unique(np.concatenate([rng.choice(n_sky, n_dirs, replace=False), near]))
        sub = sub.astype(np.int64)
        REG = np.array([REG0, reg1, 0.0], np.float32)
        args = (3, rms.shape[0], n_sky, FP_t, FX_t, rms, td00, td90, ml)
        tail = (reg["netCC"], reg["delta_regulator"], reg["network_energy_threshold"], sub)
        ref = oracle.scan_sky_for_best_fit(*args, REG, *tail)
        f64 = oracle.scan_sky_for_best_fit(*args, REG.astype(np.float64), *tail, precision="f64")
        maps = res.maps[c][:, torch_index(sub, res.maps.device)].cpu().numpy().astype(np.float64)
        worst = 0.0
        for k in range(11):
            a, b, d = maps[k], ref[k + 1][sub].astype(np.float64), f64[k + 1][sub]
            ok = ~(np.isnan(a) | np.isnan(b))
            if not ok.any():
                continue
            den = np.maximum(np.abs(b[ok]), 1e-3 * max(np.max(np.abs(b[ok])), 1e-30))
            diff = np.maximum(np.abs(a[ok] - b[ok]) - 2.0 * np.nan_to_num(np.abs(b[ok] - d[ok])), 0)
            worst = max(worst, float(np.max(diff / den)))
        lr = int(ref[0])
        tie = lr != lg and abs(float(ref[7][lr]) - float(ref[7][lg])) <= 1e-5 * abs(float(ref[7][lr]))
        rows.append({"cluster": c, "pixels": int(rms.shape[0]),
                     "regulator_equal": bool(np.float32(res.regulator[c]) == np.float32(reg1)),
                     "l_max_equal": lr == lg, "near_tie": bool(tie),
                     "max_rel_err": worst, "directions": int(sub.size)})
    return {"clusters": rows,
            "all_pass": all(r["regulator_equal"] and (r["l_max_equal"] or r["near_tie"])
                            and r["max_rel_err"] <= 1e-4 for r in rows),
            "seconds": round(time.perf_counter() - t0, 1),
            "rule": "REG[1] equal over the whole sky; maps within 1e-4 relative (floor 1e-3 of "
                    "the map's max, plus 2x the reference's float32 error vs float64) at "
                    f"{n_dirs} random directions + the 25 nearest the GPU maximum; oracle "
                    "maximum over that sample = GPU maximum or a tie within 1e-5"}


def torch_index(idx, device):
    import torch
    return torch.from_numpy(np.asarray(idx, np.int64)).to(device)


def cpu_rate(batch, ml, FP_t, FX_t, reg, target_s=12.0):
    """Cluster-sky evals/s of the oracle on all host cores, normalised to the
    workload's mean cluster size (evals/s = pairs/s / mean pixels)."""
    cores = os.cpu_count() or 1
    dt, pairs, _, _ = cpu_sample(batch, ml, FP_t, FX_t, reg, n_clusters=8, n_dirs=256)
    rate = pairs / dt
    n_dirs = int(min(ml.shape[1], max(256, target_s * rate / (32 * float(batch.sizes.mean())))))
    dt, pairs, evals, idx = cpu_sample(batch, ml, FP_t, FX_t, reg, n_clusters=32, n_dirs=n_dirs)
    pair_rate = pairs / dt
    value = pair_rate / float(batch.sizes.mean())
    sample = (f"oracle float32 (regulator + scan) on {len(idx)} size-stratified clusters of the "
              f"workload x {n_dirs} random directions each, {pairs:.3e} direction-pixel pairs in "
              f"{dt:.1f} s; evals/s = pairs/s / mean cluster size {batch.sizes.mean():.1f}")
    return {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample,
            "seconds": dt}


# --------------------------------------------------------------------------
def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=("ours", "reference"), default="ours")
    ap.add_argument("--clusters", type=int, default=4096)
    ap.add_argument("--order", type=int, default=7)
    ap.add_argument("--seed", type=int, default=20240914)
    ap.add_argument("--fast-math", type=int, default=1,
                    help="1: the scan's refined division and approximate square root "
                         "(default); 0: IEEE rounding of every division and square root")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-parity", action="store_true",
                    help="skip the oracle comparison on three clusters of the timed batch")
    ap.add_argument("--no-tune", action="store_true", help="default launch shape")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-skystat", action="store_true",
                    help="skip the statistics-at-the-maximum field")
    ap.add_argument("--no-td", action="store_true")
    ap.add_argument("--no-subnet", action="store_true",
                    help="skip the sub-network-cut sky loop field")
    ap.add_argument("--no-ieee", action="store_true",
                    help="skip timing the IEEE-rounding variant of the scan")
    ap.add_argument("--no-pipeline", action="store_true",
                    help="skip the 4-detector HEALPix-8 lag pipeline field")
    ap.add_argument("--pipeline-clusters", type=int, default=1024)
    ap.add_argument("--no-stage", action="store_true",
                    help="skip the likelihood-stage drop-in field")
    ap.add_argument("--stage-clusters", type=int, default=256)
    ap.add_argument("--profile-subnet", action="store_true",
                    help="with --profile: the sub-network-cut sky loop field only")
    ap.add_argument("--profile-td", action="store_true",
                    help="with --profile: one td-vector build of 1e6 pixels instead")
    ap.add_argument("--profile-pipeline", action="store_true",
                    help="with --profile: the lag pipeline field only")
    ap.add_argument("--no-wdm", action="store_true",
                    help="skip the WDM transform (strain -> padded planes) field")
    ap.add_argument("--profile-wdm", action="store_true",
                    help="with --profile: the WDM transform field only")
    ap.add_argument("--profile-regulator", action="store_true",
                    help="with --profile: one regulator-only launch instead")
    ap.add_argument("--profile-plain", action="store_true",
                    help="with --profile: one plain pgw_sky_loop call per size of PLAIN_SIZES")
    ap.add_argument("--profile", action="store_true",
                    help="one eager launch of the batched loop and exit (for ncu)")
    args = ap.parse_args()

    world, rank, local, pg = dist_setup()
    from pycwb_gb300.synthetic import log_uniform_sizes, regulators

    reg = regulators(len(IFOS))
    n_sky_expected = 12 * 4 ** args.order

    if args.impl == "reference":
        if rank != 0:
            return
        ml, FP_t, FX_t = sky_tables_np(args.order)
        rng = np.random.default_rng(args.seed)
        sizes = log_uniform_sizes(rng, args.clusters, 20, 3000)
        from pycwb_gb300.likelihoodWP.batched import ClusterBatch
        # the reference arm needs host data of only the sampled clusters, the
        # same clusters the GPU arm's batch holds at those positions
        views = sampled_clusters(args.seed, sizes, ml, FP_t, FX_t)
        batch = ClusterBatch.__new__(ClusterBatch)
        batch.sizes = sizes
        batch.cluster_views = lambda c: views[int(c)]
        cores = os.cpu_count() or 1
        vals, secs = [], []
        for step in range(args.warmup + args.steps):
            dt, pairs, evals, idx = cpu_sample(batch, ml, FP_t, FX_t, reg,
                                               n_clusters=N_CPU_SAMPLE, n_dirs=256, seed=step)
            if step >= args.warmup:
                vals.append(pairs / dt / float(sizes.mean()))
                secs.append(dt)
        v = float(np.median(vals))
        n_sky = ml.shape[1]
        line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": float(np.median(secs)) * 1e3, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "impl": "reference",
                "config": workload_config(args, sizes, n_sky),
                "step": (f"one step = the oracle's regulator + scan of {N_CPU_SAMPLE} "
                         "size-stratified clusters of the workload (identical to the GPU arm's "
                         "clusters at those positions) on 256 random directions each; value = "
                         "direction-pixel pairs per second / the workload's mean cluster size"),
                "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                                 "sample": "oracle float32 (a restatement of the reference's "
                                           "dpf.py/sky_stat.py/sky_scan.py loops; the reference's "
                                           "own numba code cannot be installed offline), OpenMP "
                                           f"on {cores} threads, {N_CPU_SAMPLE} size-stratified "
                                           "clusters x 256 random directions per step, "
                                           "normalised by the workload's mean cluster size"},
                "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return

    import torch

    from pycwb_gb300 import _lib
    from pycwb_gb300.autotune import autotune
    from pycwb_gb300.likelihoodWP.batched import BatchedSkyLoop, ClusterBatch, SkyTables
    from pycwb_gb300.synthetic import make_batch_device

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    _lib.build()
    L = _lib.load()
    if args.profile and args.profile_td:
        print(json.dumps({"profile": "td build", **time_td_build(dev)}))
        return
    if args.profile and args.profile_pipeline:
        print(json.dumps({"profile": "lag pipeline",
                          **time_pipeline(dev, args.seed, args.pipeline_clusters)}))
        return
    if args.profile and args.profile_wdm:
        print(json.dumps({"profile": "wdm transform", **time_wdm(dev, reps=1)}))
        return
    if args.profile and args.profile_subnet:
        print(json.dumps({"profile": "sub-network sky loop", **time_subnet(dev, args.seed, reps=1)}))
        return

    ml, FP_t, FX_t = sky_tables_np(args.order)
    n_sky = ml.shape[1]
    assert n_sky == n_sky_expected
    tables = SkyTables.from_arrays(FP_t, FX_t, ml, None, **{k: reg[k] for k in (
        "network_energy_threshold", "gamma_regulator", "delta_regulator", "netCC")})
    if args.profile and args.profile_plain:
        time_plain_sizes(L, tables, ml, FP_t, FX_t, dev, args.seed, reps=0)
        print(json.dumps({"profile": "one plain call per size", "sizes": PLAIN_SIZES}))
        return

    rng = np.random.default_rng(args.seed + 1000 * rank)
    sizes = log_uniform_sizes(rng, args.clusters, 20, 3000)
    batch = ClusterBatch(len(IFOS), 2 * K_TD + 1, sizes)
    t_gen = time.perf_counter()
    td00, td90, rms, l_true, snr = make_batch_device(args.seed + 1000 * rank, sizes, ml, FP_t,
                                                     FX_t, K_TD, device=dev)
    batch.td00.copy_(td00)
    batch.td90.copy_(td90)
    batch.rms.copy_(rms)
    del td00, td90, rms
    torch.cuda.synchronize()
    # the clusters the CPU baselines time: identical data in both arms
    for c, v in sampled_clusters(args.seed + 1000 * rank, sizes, ml, FP_t, FX_t).items():
        batch.set_cluster(c, *v)
    t_gen = time.perf_counter() - t_gen

    shape = None if args.no_tune else autotune(tables, batch, fast_math=bool(args.fast_math))
    if shape is None:
        shape = _lib.TileShape(0, 0, 0, 0, 0, 1 if args.fast_math else -1)
    loop = BatchedSkyLoop(tables, batch, shape=shape)
    loop.upload()
    loop.stream.synchronize()

    if args.profile and args.profile_regulator:
        with torch.cuda.stream(loop.stream):
            reg_buf = torch.empty(args.clusters, dtype=torch.float64, device=dev)
        loop.launch_regulators(reg_buf)
        loop.stream.synchronize()
        print(json.dumps({"profile": "one regulator-only launch", "clusters": args.clusters}))
        return
    if args.profile:
        loop.launch()
        loop.stream.synchronize()
        print(json.dumps({"profile": "one launch", "clusters": args.clusters}))
        return

    total_pix = batch.total_pix
    n_valid = n_sky
    work_evals = args.clusters * n_valid            # cluster-sky evaluations per step
    work_pairs = total_pix * n_valid
    ops = ops_per_pair(len(IFOS)) * work_pairs

    # ---- device-resident timed region ------------------------------------
    loop.capture()
    for _ in range(args.warmup):
        loop.replay()
    loop.stream.synchronize()
    barrier(pg)
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    torch.cuda.nvtx.range_push("timed")   # ncu --nvtx --nvtx-include timed/ selects these
    evs[0].record(loop.stream)
    for k in range(args.steps):
        loop.replay()
        evs[k + 1].record(loop.stream)
    loop.stream.synchronize()
    torch.cuda.nvtx.range_pop()
    torch.cuda.synchronize()
    clk = clocks.stop()
    barrier(pg)
    step_ms = [evs[k].elapsed_time(evs[k + 1]) for k in range(args.steps)]
    total_ms = evs[0].elapsed_time(evs[-1])
    total_ms = max_over_ranks(pg, total_ms, dev)
    ms_per_step = total_ms / args.steps
    value = world * work_evals / (ms_per_step * 1e-3)
    loop.download()
    loop.stream.synchronize()
    res = loop.results()

    # ---- FP32 roofline ---------------------------------------------------
    # Work the kernel has to do: the regulator over every (direction, pixel)
    # pair, the scan over the pairs above the energy threshold (a pair below
    # it adds exactly zero; the reference evaluates it anyway).
    active = int(res.active_pairs.sum())
    useful_ops = reg_ops(3) * work_pairs + scan_ops(3) * active
    peak = ctypes_peak(L)
    kernel_ms = float(np.median(step_ms))
    achieved = useful_ops / (kernel_ms * 1e-3) / 1e12
    traffic = traffic_from_profile(args.clusters, total_pix)

    # ---- the regulator alone (pgw_calculate_dpf_batched), same device data --
    with torch.cuda.stream(loop.stream):
        reg_buf = torch.empty(args.clusters, dtype=torch.float64, device=dev)
    loop.launch_regulators(reg_buf)
    r0 = torch.cuda.Event(enable_timing=True)
    r1 = torch.cuda.Event(enable_timing=True)
    r0.record(loop.stream)
    loop.launch_regulators(reg_buf)
    r1.record(loop.stream)
    r1.synchronize()
    reg_only_ms = r0.elapsed_time(r1)
    assert np.array_equal(reg_buf.cpu().numpy(), res.regulator)

    # ---- the same launch with approximate division / square root ----------
    # ---- the same launch with IEEE rounding of every division and sqrt ----
    ieee = None
    if not args.no_ieee and args.fast_math:
        ishape = (_lib.TileShape(0, 0, 0, 0, 0, -1) if args.no_tune
                  else autotune(tables, batch, fast_math=False))
        loop.shape = ishape
        loop.launch()
        f0 = torch.cuda.Event(enable_timing=True)
        f1 = torch.cuda.Event(enable_timing=True)
        f0.record(loop.stream)
        for _ in range(args.steps):
            loop.launch()
        f1.record(loop.stream)
        f1.synchronize()
        loop.shape = shape
        ims = f0.elapsed_time(f1) / args.steps
        ieee = {"ms_per_step": ims, "value": world * work_evals / (ims * 1e-3),
                "launch_shape": dict(zip(("threads", "lanes_per_sky", "chunk_pix", "stages",
                                          "min_blocks", "fast_math"), ishape.key())),
                "note": "the scan with IEEE rounding of every division and square root; the "
                        "headline uses the refined division (within one ulp) and approximate "
                        "square root; both pass the 1e-4 parity tests"}

    # ---- end to end through the public API ------------------------------
    e2e = None
    if not args.no_e2e:
        loop.run()  # warm
        barrier(pg)
        # every step copies its inputs from pinned host memory and reads its
        # results back; run_many overlaps step k+1's copy with step k's
        # launch, so only the first copy is exposed (counted in the time)
        n_e2e = max(2, min(args.steps, 3))
        t0 = time.perf_counter()
        for r in loop.run_many([batch] * n_e2e):
            pass
        dt = (time.perf_counter() - t0) / n_e2e
        dt = max_over_ranks(pg, dt, dev)
        t1 = time.perf_counter()
        loop.run(upload=True, download=True)
        dt_one = max_over_ranks(pg, time.perf_counter() - t1, dev)
        e2e = {"value": world * work_evals / dt, "unit": UNIT,
               "h2d_bytes_per_step": batch.h2d_bytes, "d2h_bytes_per_step": loop.d2h_bytes,
               "ms_per_step": dt * 1e3, "steps": n_e2e, "api": "BatchedSkyLoop.run_many",
               "run_ms": dt_one * 1e3,
               "run_note": "one BatchedSkyLoop.run (copy, launch, read-back in sequence)"}

    # ---- plain: one launch per cluster on the same device data ------------
    plain = None
    if not args.no_plain:
        plain = time_plain(L, loop, tables, batch, shape, dev)
        plain["us_per_call_by_size"] = time_plain_sizes(L, tables, ml, FP_t, FX_t, dev, args.seed)
        plain["value"] = world * work_evals / (plain["ms"] * 1e-3)
        plain["roofline_frac"] = (useful_ops / (plain["ms"] * 1e-3) / 1e12 / peak) if peak else None

    parity = None
    if rank == 0 and not args.no_parity:
        parity = parity_sample(res, batch, ml, FP_t, FX_t, reg, args.order)

    skystat = (time_skystat(loop, res, batch, dev, args.seed + 3)
               if not args.no_skystat else None)
    adjoint = time_adjoint(loop, res, batch, args.order, dev) if not args.no_adjoint else None
    td_build = time_td_build(dev) if not args.no_td else None
    wdm_field = time_wdm(dev) if not args.no_wdm else None
    found, l_max = res.found.copy(), res.l_max.copy()
    res.maps = None                  # release the 4096-cluster buffers first
    del loop, res
    torch.cuda.empty_cache()
    pipeline = (time_pipeline(dev, args.seed + 1000 * rank, args.pipeline_clusters)
                if not args.no_pipeline else None)
    subnet = time_subnet(dev, args.seed + 7 + 1000 * rank) if not args.no_subnet else None
    stage = (time_stage(ml, FP_t, FX_t, args.order, args.seed + 11 + 1000 * rank,
                        args.stage_clusters) if not args.no_stage else None)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu = cpu_rate(batch, ml, FP_t, FX_t, reg)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic",
            "config": workload_config(args, sizes, n_sky),
            "launch_shape": dict(zip(("threads", "lanes_per_sky", "chunk_pix", "stages",
                                      "min_blocks", "fast_math"), shape.key())),
            "generation_s": round(t_gen, 2),
            "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                         "frac": achieved / peak if peak else None, "traffic": traffic,
                         "ops_per_launch": useful_ops,
                         "ops_note": (f"regulator {reg_ops(3)} ops x {work_pairs:.4e} pairs + scan "
                                      f"{scan_ops(3)} ops x {active:.4e} pairs above E_thr "
                                      f"({active / work_pairs:.3%} of pairs)"),
                         "reference_ops_per_launch": ops,
                         "reference_equivalent_tflops": ops / (kernel_ms * 1e-3) / 1e12,
                         "frac_regulator_as_executed": (
                             (REG_ITER_FRACTION * reg_ops(3) * work_pairs + scan_ops(3) * active)
                             / (kernel_ms * 1e-3) / 1e12 / peak) if peak else None,
                         "frac_regulator_as_executed_note": (
                             f"the regulator credited only for the {REG_ITER_FRACTION:.1%} of its "
                             "per-warp pixel iterations that run (its early pass/fail "
                             "decisions stop the rest; fraction counted on 1,024 clusters of this "
                             "workload in a diagnostic build)"),
                         "kernel_ms": kernel_ms,
                         "peak_source": "measured: pgw_fp32_fma_peak (register FMA chains, "
                                        "2 flops per FMA) in this run"},
            "cpu_baseline": cpu,
            "e2e": e2e,
            "gpu_launches": 2 * args.steps,  # set-up (prepare_kernel), sky loop
            "clocks": clk,
            "plain": plain,
            "batched_vs_plain": (plain["ms"] / ms_per_step) if plain else None,
            "regulator_only_ms": reg_only_ms,
            "ieee_variant": ieee,
            "adjoint": adjoint,
            "skystat": skystat,
            "td_build": td_build,
            "wdm": wdm_field,
            "pipeline": pipeline,
            "subnet": subnet,
            "stage": stage,
            "parity_sample": parity,
            "selected": {"found": int(found.sum()),
                         "l_max_equals_injected": int(np.sum(l_max == l_true))},
            "step_ms": step_ms,
        }
        print(json.dumps(line), flush=True)


def ctypes_peak(L):
    import ctypes
    import torch
    out = ctypes.c_double(0.0)
    ms = ctypes.c_double(0.0)
    rc = L.pgw_fp32_fma_peak(20000, ctypes.byref(out), ctypes.byref(ms),
                             torch.cuda.current_stream().cuda_stream)
    return out.value if rc == 0 else None


def fp64_peak(L):
    """Measured float64 multiply + add rate (G ops/s) of this GPU."""
    import ctypes
    import torch
    out = ctypes.c_double(0.0)
    ms = ctypes.c_double(0.0)
    rc = L.pgw_fp64_mul_add_peak(400, ctypes.byref(out), ctypes.byref(ms),
                                 torch.cuda.current_stream().cuda_stream)
    return out.value if rc == 0 else None


def td_ops(taps: int) -> int:
    """float64 multiplies + adds of one (pixel, delay) td pair at an interior
    layer: two amplitudes, each three FIRs of `taps` products and sums plus
    nine to combine them with the phase factors (td_vector_kernels.py:40-131)."""
    return 2 * (6 * taps + 9)


def td_roofline(L, pairs: int, taps: int, ms: float):
    peak = fp64_peak(L)
    achieved = pairs * td_ops(taps) / (ms * 1e-3) / 1e9
    return {"bound": "fp64", "achieved": achieved, "peak": peak, "unit": "G ops/s",
            "frac": achieved / peak if peak else None, "ops_per_pair": td_ops(taps),
            "peak_source": "measured: pgw_fp64_mul_add_peak (separately rounded multiply and "
                           "add chains) in this run"}


def traffic_from_profile(n_clusters, total_pix):
    """DRAM bytes per launch scaled from the committed ncu capture, or None.

    The capture's traffic is compulsory: the output maps (per cluster) and
    the td amplitudes (per pixel); it is scaled by those two counts."""
    path = os.path.join(REPO, "profiles", "sky_loop_traffic.json")
    try:
        with open(path) as f:
            p = json.load(f)
        return (float(p["write_bytes_per_cluster"]) * n_clusters +
                float(p["read_bytes_per_pixel"]) * total_pix)
    except (OSError, ValueError, KeyError):
        return None


def time_adjoint(loop, res, batch, order, dev):
    """Off-grid refinement of up to 256 clusters of 200-2000 pixels (10 ascent
    steps each, one launch) from their grid maxima; timed with CUDA events."""
    import torch
    from pycwb_gb300.adjoint import GradInputs, detector_geometry, grid_angles, refine

    sel = np.flatnonzero((batch.sizes >= 200) & (batch.sizes <= 2000) & res.found)[:256]
    if sel.size == 0:
        return None
    inp = GradInputs.from_loop(loop, detector_geometry(IFOS, IFOS[0], 512.0), res.regulator)
    theta, phi = grid_angles(loop.t.n_sky, order)
    args = (inp, res.l_max[sel], theta, phi, res.sky_stat_max[sel])
    refine(*args, n_steps=10, healpix_order=order, clusters=sel)  # warm-up
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(loop.stream)
    r = refine(*args, n_steps=10, healpix_order=order, clusters=sel)
    e1.record(loop.stream)
    e1.synchronize()
    gain = (r.statistic - r.start_statistic) / np.maximum(np.abs(r.start_statistic), 1e-30)
    return {"clusters": int(sel.size), "steps": 10, "ms": e0.elapsed_time(e1),
            "improved": int(r.improved.sum()),
            "median_relative_gain": float(np.median(gain[r.improved])) if r.improved.any() else 0.0,
            "median_shift_rad": float(np.median(r.distance[r.improved])) if r.improved.any() else 0.0,
            "evaluations": int(sel.size) * 11,
            "note": "statistic and (theta, phi) gradient at continuous directions, "
                    "grid maximum kept where refinement does not beat it"}


def time_td_build(dev, n_pix=1_000_000, M=64, nc=20, K=20):
    """td-amplitude vectors (pgw_batch_get_td_vecs) of n_pix random pixels of one
    (M+1)-layer plane, K = 20, TD filters of 2*nc+1 taps; CUDA-event timed."""
    import torch
    from pycwb_gb300.utils.td_vector_kernels import batch_get_td_vecs

    rng = np.random.default_rng(1)
    n_time = 4096
    rows = n_time + 2 * nc
    p00 = torch.zeros((rows, M + 1), dtype=torch.float32, device=dev)
    p90 = torch.zeros_like(p00)
    p00[nc:nc + n_time] = torch.randn((n_time, M + 1), device=dev)
    p90[nc:nc + n_time] = torch.randn((n_time, M + 1), device=dev)
    T0 = torch.randn((2 * M + 1, 2 * nc + 1), dtype=torch.float64, device=dev)
    Tx = torch.randn((2 * M + 1, 2 * nc + 1), dtype=torch.float64, device=dev)
    idx = torch.from_numpy(rng.integers(0, n_time * (M + 1), n_pix).astype(np.int32)).to(dev)
    from pycwb_gb300 import _device as dv
    batch_get_td_vecs(idx, p00, p90, T0, Tx, M, nc, K, M, return_device=True)  # warm-up
    torch.cuda.synchronize()
    s = dv.stream()                  # the stream the library launches on
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(s)
    batch_get_td_vecs(idx, p00, p90, T0, Tx, M, nc, K, M, return_device=True)
    e1.record(s)
    e1.synchronize()
    ms = e0.elapsed_time(e1)
    from pycwb_gb300 import _lib
    return {"pixels": n_pix, "layers": M, "K": K, "taps": 2 * nc + 1, "ms": ms,
            "pixels_per_s": n_pix / (ms * 1e-3),
            "roofline": td_roofline(_lib.load(), n_pix * (2 * K + 1), 2 * nc + 1, ms),
            "note": "float64 accumulation, bit-identical to the reference"}


WDM_LAYERS = (16, 32, 64, 128, 256, 512)


def wdm_instructions(M: int, n_filter: int, n_time: int) -> int:
    """float64 instructions of one transform (an FMA counted once): per time
    slice the fold's 2M * 2k + 1 FMAs (the 2 * 2kM + 1 filter taps, k = (n_filter
    - 1) / 2M) and 8 per butterfly of the radix-2 FFT of length 2M (M log2(2M)
    butterflies: a complex multiply as 2 multiplies + 2 FMAs, then 4 adds)."""
    M2 = 2 * M
    kf = (n_filter - 1) // M2
    return n_time * (M2 * 2 * kf + 1 + 8 * M * int(round(math.log2(M2))))


def time_wdm(dev, n_ifo=4, duration=600.0, rate=512.0, nc=12, L=4, beta=4, prec=10, reps=3):
    """T2: every detector's strain to the padded float32 WDM planes of every
    level (16-512 layers), as the reference's per-segment td-inputs cache
    (td_vector_batch.py:35-144); CUDA-event timed on the launching stream.
    Basis and TD filters are designed on the host once per level (timed
    apart); the oracle's numpy transform of one detector is the CPU line."""
    import torch
    from pycwb_gb300 import _lib, wdm
    from oracle import wdm_oracle

    t0 = time.perf_counter()
    bases = [wdm.WDM(M, M, beta, prec) for M in WDM_LAYERS]
    for b in bases:
        b.set_td_filter(nc, L)
    host_ms = (time.perf_counter() - t0) * 1e3
    n = int(duration * rate)
    rng = np.random.default_rng(3)
    strains = [torch.from_numpy(rng.standard_normal(n)).to(dev) for _ in range(n_ifo)]
    s = torch.cuda.current_stream(dev)

    def run():
        return [[b.td_inputs(x, stream=s) for x in strains] for b in bases]

    run()
    torch.cuda.synchronize()
    ms = []
    for _ in range(reps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(s)
        out = run()
        e1.record(s)
        e1.synchronize()
        ms.append(e0.elapsed_time(e1))
    t = float(np.median(ms))
    instr = n_ifo * sum(wdm_instructions(b.M, b.m_H, wdm.t2w_n_time(n, b.M)) for b in bases)
    nbytes = n_ifo * sum(8 * n + 2 * 4 * (wdm.t2w_n_time(n, b.M) + 2 * nc) * (b.M + 1)
                         for b in bases)
    peak = fp64_peak(_lib.load())
    achieved = instr / (t * 1e-3) / 1e9
    c0 = time.perf_counter()
    for b in bases:
        wdm_oracle.t2w(strains[0].cpu().numpy(), b.M, b.filter)
    cpu_ms = (time.perf_counter() - c0) * 1e3 * n_ifo
    del out
    return {"workload": f"{n_ifo} detectors x {duration:.0f} s at {rate:.0f} Hz, "
                        f"{WDM_LAYERS[0]}-{WDM_LAYERS[-1]} layers ({len(WDM_LAYERS)} levels), "
                        f"beta {beta}, precision {prec}, TD filters {2 * nc + 1} taps, upTDF {L}",
            "transforms": n_ifo * len(bases), "ms": t, "launches": n_ifo * len(bases),
            "samples_per_s": n_ifo * len(bases) * n / (t * 1e-3),
            "host_design_ms": host_ms, "bytes": nbytes,
            "achieved_gbs": nbytes / (t * 1e-3) / 1e9,
            "roofline": {"bound": "fp64", "achieved": achieved, "peak": peak, "unit": "G ops/s",
                         "frac": achieved / peak if peak else None, "instructions": instr,
                         "peak_source": "measured: pgw_fp64_mul_add_peak in this run; "
                                        "float64 instructions, an FMA counted once"},
            "cpu_oracle_ms": cpu_ms, "cpu_cores": 1,
            "cpu_note": "oracle numpy transform (fold + numpy.fft.rfft) of one detector's "
                        "levels, times the detector count",
            "note": "writes the zero-padded float32 planes the td build reads "
                    "(t2w + prepare_td_inputs in one kernel)"}


PIPE_IFOS = ["L1", "H1", "V1", "K1"]
PIPE_RATE = 2048.0     # TD rate: 4096 Hz data, levelR 3 (512 Hz analysis), upTDF 4
PIPE_K = 67            # max(TDSize 12 * upTDF 4, int(max_delay 0.0325 s * 2048) + 1)
PIPE_ORDER = 8


def time_pipeline(dev, seed, n_clusters=1024, steps=2):
    """One lag of the 4-detector network end to end on the device: td build of
    every cluster from its WDM resolution's planes (16-512 layers), batched
    regulator + scan over HEALPix 8, refinement of every sky maximum."""
    import torch

    from pycwb_gb300 import _lib, sky
    from pycwb_gb300.adjoint import detector_geometry
    from pycwb_gb300.likelihoodWP.batched import SkyTables
    from pycwb_gb300.likelihoodWP.lag_pipeline import LagPipeline
    from pycwb_gb300.synthetic import make_strain_lag, regulators

    t_set = time.perf_counter()
    ml, FP, FX = sky.compute_sky_delay_and_patterns(PIPE_IFOS, "L1", PIPE_RATE, PIPE_K,
                                                    healpix_order=PIPE_ORDER)
    FP_t, FX_t = FP.T.astype(np.float32).copy(), FX.T.astype(np.float32).copy()
    reg = regulators(len(PIPE_IFOS))
    tables = SkyTables.from_arrays(FP_t, FX_t, ml, None, **{k: reg[k] for k in (
        "network_energy_threshold", "gamma_regulator", "delta_regulator", "netCC")})
    layers = (16, 32, 64, 128, 256, 512)
    planes, level, pixels, rms, l_true, info = make_strain_lag(
        seed, PIPE_IFOS, ml, FP_t, FX_t, PIPE_RATE, layers=layers, duration=600.0, rate=512.0,
        n_inj=200, n_clusters=n_clusters, device=dev)
    pipe = LagPipeline(tables, planes, level, pixels, rms, PIPE_K,
                       geometry=detector_geometry(PIPE_IFOS, "L1", PIPE_RATE),
                       healpix_order=PIPE_ORDER)
    t_set = time.perf_counter() - t_set
    pipe.run(refine=True)                       # warm-up (phase tables, kernels)
    torch.cuda.synchronize()
    walls, stages = [], []
    for _ in range(steps):
        t0 = time.perf_counter()
        out = pipe.run(refine=True, timed=True)
        walls.append(time.perf_counter() - t0)
        stages.append(out.stage_ms)
    wall = float(np.median(walls))
    st = {k: float(np.median([x[k] for x in stages])) for k in stages[0]}
    n_sky = tables.n_sky
    r = out.refined
    inj = np.flatnonzero(l_true >= 0)
    phi, lat = sky.build_sky_directions(n_sky, PIPE_ORDER)
    vec = np.stack([np.cos(lat) * np.cos(phi), np.cos(lat) * np.sin(phi), np.sin(lat)], 1)
    ang = np.degrees(np.arccos(np.clip(np.einsum(
        "ij,ij->i", vec[out.scan.l_max[inj]], vec[l_true[inj]]), -1.0, 1.0)))
    return {
        "workload": (f"one lag: L1/H1/V1/K1, 600 s of white noise at 512 Hz with 200 "
                     f"sine-Gaussian / Gaussian-pulse injections (SNR 8-40), WDM at "
                     f"{layers[0]}-{layers[-1]} layers on the device, {n_clusters} clusters "
                     f"P~logU[50,5000] (200 around injections), td build (K={PIPE_K}, "
                     f"{2 * PIPE_K + 1} delays, 25-tap filters, upTDF 4) -> batched scan over "
                     f"HEALPix {PIPE_ORDER} ({n_sky} directions) -> refinement of every sky "
                     "maximum"),
        "t2w_ms_per_segment": info["t2w_ms"],
        "injections_located_within_2deg": int(np.sum(ang <= 2.0)),
        "injection_median_angle_deg": float(np.median(ang)),
        "injection_median_angle_deg_snr_above_20": float(np.median(
            ang[info["snr"][inj] > 20.0])) if np.any(info["snr"][inj] > 20.0) else None,
        "clusters": n_clusters, "total_pix": pipe.total_pix, "n_sky": n_sky,
        "steps": steps, "ms_per_lag": wall * 1e3, **st,
        "cluster_sky_evals_per_s": n_clusters * n_sky / (wall),
        "scan_cluster_sky_evals_per_s": n_clusters * n_sky / (st["sky_loop_ms"] * 1e-3),
        "td_roofline": td_roofline(_lib.load(), pipe.total_pix * len(PIPE_IFOS) * (2 * PIPE_K + 1),
                                   25, st["td_build_ms"]),
        "h2d_bytes_per_lag": pipe.h2d_bytes, "found": int(out.scan.found.sum()),
        "refined": int(r.improved.sum()) if r is not None else 0,
        "setup_s": round(t_set, 2),
        "note": "wall clock per lag through LagPipeline.run (td amplitudes never leave "
                "the device; rms in, per-cluster results out)",
    }


def time_subnet(dev, seed, n_clusters=1024, n_loud=200, order=4, reps=3):
    """Sub-network-cut sky loop (sub_net_cut.py:404-517) for a lag's
    superclusters: n_clusters clusters of their n_loud loudest pixels
    (LOUD = 200, utils.py:705-711) over the HEALPix-4 grid (MIN_SKYRES_HEALPIX
    = 4), L1/H1/V1, K = 20, Acore 1.7, subcut 0.33; one launch of
    pgw_subnet_sky_batched, device-resident inputs, CUDA-event timed; the
    float32 oracle (one core) on 4 of the clusters for the CPU figure."""
    import torch

    from pycwb_gb300 import _device as dv
    from pycwb_gb300 import _lib, sky
    from pycwb_gb300.likelihoodWP.batched import ClusterBatch
    from pycwb_gb300.synthetic import make_batch_device, subnet_constants

    ml, FP, FX = sky.compute_sky_delay_and_patterns(IFOS, "L1", 512.0, K_TD, healpix_order=order)
    FP_t, FX_t = FP.T.astype(np.float32).copy(), FX.T.astype(np.float32).copy()
    n_sky = ml.shape[1]
    c = subnet_constants(len(IFOS), acore=1.7, subcut=0.33)
    sizes = np.full(n_clusters, n_loud, np.int64)
    b = ClusterBatch(len(IFOS), 2 * K_TD + 1, sizes)
    td00, td90, rms, _, _ = make_batch_device(seed, sizes, ml, FP_t, FX_t, K_TD, device=dev)
    b.td00.copy_(td00)
    b.td90.copy_(td90)
    b.rms.copy_(rms)
    s = dv.stream()
    L = _lib.load()
    FPd, FXd = torch.from_numpy(FP_t).to(dev), torch.from_numpy(FX_t).to(dev)
    mld = torch.from_numpy(ml.astype(np.int32)).to(dev)
    pix_off = torch.from_numpy(b.pix_offsets).to(dev)
    td_off = torch.from_numpy(b.td_offsets).to(dev)
    out = torch.empty((n_clusters, 48), dtype=torch.uint8, device=dev)
    torch.cuda.synchronize()   # the generator wrote the device inputs

    def launch():
        rc = L.pgw_subnet_sky_batched(len(IFOS), n_clusters, pix_off.data_ptr(), td_off.data_ptr(),
                                      b.total_pix, n_sky, FPd.data_ptr(), FXd.data_ptr(),
                                      rms.data_ptr(), td00.data_ptr(), td90.data_ptr(),
                                      2 * K_TD + 1, mld.data_ptr(),
                                      float(np.float32(c["network_energy_threshold"])),
                                      c["e2or"], c["subcut"], out.data_ptr(), s.cuda_stream)
        if rc:
            raise RuntimeError(L.pgw_last_error().decode())
    launch()
    s.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(s)
    for _ in range(reps):
        launch()
    e1.record(s)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / reps
    evals = n_clusters * n_sky
    from oracle import oracle as orc   # the CPU baseline (test infrastructure)
    t0 = time.perf_counter()
    n_cpu = 4
    for k in range(n_cpu):
        a_, b_ = int(b.td_offsets[k]), int(b.td_offsets[k + 1])
        shp = (2 * K_TD + 1, len(IFOS), n_loud)
        p0, p1 = int(b.pix_offsets[k]), int(b.pix_offsets[k + 1])
        orc.optimze_sky_loc_from_td(len(IFOS), n_loud, n_sky, FP_t, FX_t, b.rms[p0:p1].numpy(),
                                    b.td00[a_:b_].numpy().reshape(shp),
                                    b.td90[a_:b_].numpy().reshape(shp), ml,
                                    c["network_energy_threshold"], c["e2or"], c["subcut"])
    cpu_s = time.perf_counter() - t0
    res = out.cpu().numpy().view(np.dtype([("key", "<u8"), ("l_max", "<i8"), ("f", "<f4", 5),
                                           ("Vm", "<i4"), ("status", "<i4"), ("r", "<i4")]))
    return {"workload": f"{n_clusters} clusters x {n_loud} loudest pixels, HEALPix {order} "
                        f"({n_sky} directions), L1/H1/V1, K={K_TD}, Acore 1.7, subcut 0.33",
            "ms": ms, "cluster_sky_evals_per_s": evals / (ms * 1e-3),
            "cpu_oracle_evals_per_s": n_cpu * n_sky / cpu_s, "cpu_cores": 1,
            "cpu_sample": f"{n_cpu} clusters, float32 oracle, one thread",
            "selected": int((res["key"].reshape(-1) != 0).sum())}


def synthetic_xtalk_rows(rng, sizes, n_nbr=4, scale=0.05):
    """Packed xtalk overlaps for a batch (the overlap catalog is not
    available): every pixel overlaps itself with (1, 0, 0, 1) and n_nbr
    random pixels of its cluster with N(0, scale) coefficients; rows (n, 8)
    float32 with cluster-local neighbour indices, lookup (total_pix, 2)."""
    sizes = np.asarray(sizes, np.int64)
    total = int(sizes.sum())
    per = n_nbr + 1
    owner_size = np.repeat(sizes, sizes)
    rows = np.zeros((total, per, 8), np.float32)
    local = np.concatenate([np.arange(P) for P in sizes]) if total else np.zeros(0, np.int64)
    rows[:, 0, 0] = local
    rows[:, 0, 4] = 1.0
    rows[:, 0, 7] = 1.0
    nb = (rng.random((total, n_nbr)) * owner_size[:, None]).astype(np.int64)
    rows[:, 1:, 0] = nb
    rows[:, 1:, 4:8] = rng.normal(0.0, scale, (total, n_nbr, 4))
    lookup = np.stack([np.arange(total) * per, np.arange(total) * per + per], axis=1)
    return rows.reshape(-1, 8), lookup.astype(np.int64)


def time_skystat(loop, res, batch, dev, seed, reps=3):
    """The reference caller's per-cluster consumers of the sky maps, on the
    device, CUDA-event timed: the statistics at the sky maximum
    (pgw_skystat_batched, sky_statistics.py:94-262) of every cluster of the
    timed batch in one launch (synthetic xtalk overlaps), and the sky
    probability of every cluster with sky_stat_max > 0 in one launch."""
    import ctypes
    import torch
    from pycwb_gb300 import _lib
    from pycwb_gb300.likelihoodWP.sky_statistics import SKYSTAT_DTYPE

    L = _lib.load()
    t, b = loop.t, batch
    n = b.n_clusters
    xt_h, lk_h = synthetic_xtalk_rows(np.random.default_rng(seed), b.sizes)
    s = loop.stream
    with torch.cuda.stream(s):
        xt = torch.from_numpy(xt_h).to(dev)
        lk = torch.from_numpy(lk_h).to(dev)
        l = torch.from_numpy(np.ascontiguousarray(res.l_max, np.int64)).to(dev)
        regs = loop.regs.to(torch.float32)
        ws = torch.empty(int(L.pgw_skystat_workspace_bytes(b.n_ifo, b.total_pix)),
                         dtype=torch.uint8, device=dev)
        out = torch.empty((n, SKYSTAT_DTYPE.itemsize), dtype=torch.uint8, device=dev)
    P = lambda x: ctypes.c_void_p(x.data_ptr())

    def launch():
        rc = L.pgw_skystat_batched(b.n_ifo, n, P(loop.pix_off), P(loop.td_off), b.total_pix,
                                   t.n_sky, P(t.FP), P(t.FX), P(loop.rms), P(loop.td00),
                                   P(loop.td90), b.n_delay, P(t.ml), P(l), P(regs),
                                   float(t.REG0), float(t.network_energy_threshold), P(xt),
                                   int(xt.shape[0]), P(lk), 0, P(ws), ws.numel(), P(out),
                                   ctypes.c_void_p(s.cuda_stream))
        if rc:
            raise RuntimeError(L.pgw_last_error().decode())
    launch()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(s)
    for _ in range(reps):
        launch()
    e1.record(s)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / reps
    rec = np.frombuffer(out.cpu().numpy().tobytes(), dtype=SKYSTAT_DTYPE)
    # the sky probability (softmax of nSkyStat) of every cluster the
    # reference's caller computes it for: those with sky_stat_max > 0
    # (likelihood.py:328-342)
    keep = np.flatnonzero(res.found & (res.sky_stat_max > 0)).astype(np.int32)
    n_p = int(keep.size)
    with torch.cuda.stream(s):
        sel = torch.from_numpy(keep).to(dev)
        prob = torch.empty((n_p, t.n_sky), dtype=torch.float32, device=dev)
        summ = torch.empty((n_p, 4), dtype=torch.float64, device=dev)

    def prob_launch():
        rc = L.pgw_sky_probability(n_p, t.n_sky, loop.stats.data_ptr(), int(loop.stats.stride(0)),
                                   sel.data_ptr(), prob.data_ptr(), summ.data_ptr(),
                                   ctypes.c_void_p(s.cuda_stream))
        if rc:
            raise RuntimeError(L.pgw_last_error().decode())
    prob_launch()
    e0.record(s)
    prob_launch()
    e1.record(s)
    e1.synchronize()
    prob_ms = e0.elapsed_time(e1)
    return {"workload": f"{n} clusters of the timed batch at their sky maxima, "
                        f"{b.total_pix} pixels, 5 synthetic xtalk rows per pixel",
            "ms": ms, "us_per_cluster": ms * 1e3 / n, "clusters_per_s": n / (ms * 1e-3),
            "status_ok": int((rec["status"] == 0).sum()),
            "probability_ms": prob_ms, "probability_maps": n_p,
            "probability_note": "pgw_sky_probability: softmax of nSkyStat (float32-accurate "
                                "exponentials, compensated sum, float64 across the block) and "
                                "the 50 % / 90 % direction counts (binade histogram, bisection "
                                "in shared memory) of every cluster with sky_stat_max > 0, one "
                                "launch"}


def time_plain(L, loop, tables, batch, shape, dev):
    """The same clusters, one pgw_sky_loop launch each (device-resident)."""
    import ctypes
    import torch

    n_sky = tables.n_sky
    s = loop.stream
    with torch.cuda.stream(s):
        ws = torch.empty(L.pgw_workspace_bytes(batch.n_ifo, batch.n_delay, int(batch.sizes.max()), 1),
                         dtype=torch.uint8, device=dev)
        st = torch.empty((11, n_sky), dtype=torch.float32, device=dev)
        res = torch.empty((batch.n_clusters, 32), dtype=torch.uint8, device=dev)
        regs = torch.empty(batch.n_clusters, dtype=torch.float64, device=dev)
    ptrs = []
    for c in range(batch.n_clusters):
        a, b = int(batch.td_offsets[c]), int(batch.pix_offsets[c])
        ptrs.append((int(batch.sizes[c]), loop.td00.data_ptr() + 4 * a, loop.td90.data_ptr() + 4 * a,
                     loop.rms.data_ptr() + 4 * batch.n_ifo * b))
    shp = None   # the default one-cluster shape, as sky_loop / scan_sky_for_best_fit use it

    def one(c):
        P, t0, t9, rm = ptrs[c]
        rc = L.pgw_sky_loop(batch.n_ifo, P, n_sky, tables.FP.data_ptr(), tables.FX.data_ptr(), rm,
                            t0, t9, batch.n_delay, tables.ml.data_ptr(), tables.REG0,
                            tables.gamma_regulator, tables.netCC, tables.network_energy_threshold,
                            tables.valid.data_ptr(), tables.valid.numel(), tables.order.data_ptr(),
                            tables.reg_order.data_ptr(), st.data_ptr(),
                            res.data_ptr() + 32 * c, regs.data_ptr() + 8 * c, shp, ws.data_ptr(),
                            ws.numel(), s.cuda_stream)
        if rc:
            raise RuntimeError(L.pgw_last_error().decode())

    for c in range(min(64, batch.n_clusters)):  # warm-up
        one(c)
    s.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(s)
    for c in range(batch.n_clusters):
        one(c)
    e1.record(s)
    e1.synchronize()
    ms = e0.elapsed_time(e1)
    return {"ms": ms, "launches": batch.n_clusters * 2,  # set-up, sky loop
            "note": "same kernel, one pgw_sky_loop per cluster with the default one-cluster "
                    "launch shape, device-resident, 1 timed pass"}


class _StagePixels:
    """A cluster's pixel arrays as the reference's stage reads them:
    noise_rms (nIFO, P) and td_amp_dense() (P, nIFO, 2 (2K + 1))."""

    def __init__(self, rms, td00, td90):
        self.noise_rms = (1.0 / rms.astype(np.float64)).T
        self._td = np.concatenate([np.transpose(td00, (2, 1, 0)), np.transpose(td90, (2, 1, 0))],
                                  axis=2)

    def __len__(self):
        return self.noise_rms.shape[1]

    def td_amp_dense(self):
        return self._td


class _StageXTalk:
    """Synthetic packed xtalk overlaps per cluster (get_xtalk_pixels)."""

    def __init__(self):
        self.by_id = {}

    def get_xtalk_pixels(self, pixels, check=True):
        rows, lookup = self.by_id[id(pixels)]
        return lookup, rows


def time_stage(ml, FP_t, FX_t, order, seed, n_clusters, reps=2):
    """The whole likelihood stage through its drop-in
    (pycwb_gb300.likelihoodWP.likelihood.likelihood_wrapper, the reference's
    likelihood.py:58-135 signature) on host cluster objects: per-cluster
    input extraction on the host, one batched regulator + scan launch, the
    statistics at every maximum and the threshold cut, the sky probability
    and the read-back of the accepted clusters' 11 maps, probabilities and
    per-pixel statistics.  Host wall time per call after one warm-up call;
    pixel counts log-uniform in [20, 3000], SNR U[8, 40]."""
    from types import SimpleNamespace

    from pycwb_gb300.likelihoodWP.likelihood import likelihood_wrapper
    from pycwb_gb300.likelihoodWP.likelihood_setup import prepare_likelihood_inputs
    from pycwb_gb300.synthetic import log_uniform_sizes, make_cluster

    cfg = SimpleNamespace(nIFO=len(IFOS), Acore=math.sqrt(2.0), gamma=0.5, delta=0.5,
                          netRHO=3.5, netCC=0.5, healpix=order, precision=0, nRES=1)
    setup = prepare_likelihood_inputs(cfg, None, len(IFOS), ml=ml, FP=FP_t.T, FX=FX_t.T)
    rng = np.random.default_rng(seed)
    sizes = log_uniform_sizes(rng, n_clusters, 20, 3000)
    xtalk = _StageXTalk()
    clusters = []
    for P in sizes:
        td00, td90, rms, _ = make_cluster(rng, ml, FP_t, FX_t, int(P), K_TD,
                                          float(rng.uniform(8.0, 40.0)))
        pix = _StagePixels(rms, td00, td90)
        xtalk.by_id[id(pix)] = synthetic_xtalk_rows(rng, [int(P)])
        clusters.append(SimpleNamespace(pixel_arrays=pix, cluster_status=0, cluster_time=5.0,
                                        cluster_freq=200.0))
    lag = SimpleNamespace(clusters=clusters)

    def call():
        for cl in clusters:
            cl.cluster_status = 0
            cl.cluster_meta = SimpleNamespace(l_max=None, theta=None, phi=None, c_time=0.0,
                                              c_freq=0.0)
        return likelihood_wrapper(cfg, [lag], None, None, xtalk=xtalk, setup=setup)

    call()
    secs, accepted = [], 0
    for _ in range(reps):
        t0 = time.perf_counter()
        out = call()
        secs.append(time.perf_counter() - t0)
        accepted = len(out[0])
    t = float(np.median(secs))
    n_sky = int(ml.shape[1])
    return {"workload": f"{n_clusters} clusters, pixels log-uniform[20,3000], SNR U[8,40], "
                        f"HEALPix {order}, {len(IFOS)} detectors, synthetic xtalk "
                        "(5 rows per pixel)",
            "api": "likelihood_wrapper (likelihood.py:58-135 signature)",
            "pixels": int(sizes.sum()), "accepted": accepted, "s_per_call": t,
            "clusters_per_s": n_clusters / t, "cluster_sky_evals_per_s": n_clusters * n_sky / t,
            "d2h_bytes": accepted * (11 + 1) * 4 * n_sky,
            "note": "host wall time of the drop-in call: input extraction per cluster, "
                    "the GPU stage, and the accepted clusters' maps and per-pixel arrays "
                    "read back"}


PLAIN_SIZES = (20, 100, 300, 1000, 3000)


def time_plain_sizes(L, tables, ml, FP_t, FX_t, dev, seed, reps=50):
    """One cluster of each size in PLAIN_SIZES (SNR 20), pgw_sky_loop over the
    whole sky with device-resident inputs: microseconds per call, CUDA events
    over `reps` calls after 5 warm-up calls.  reps = 0: one call per size,
    untimed (the form an ncu capture runs)."""
    import torch

    from pycwb_gb300.synthetic import make_cluster

    rng = np.random.default_rng(seed + 77)
    n_sky = tables.n_sky
    s = torch.cuda.Stream(device=dev)
    with torch.cuda.stream(s):
        st = torch.empty((11, n_sky), dtype=torch.float32, device=dev)
        res = torch.empty(32, dtype=torch.uint8, device=dev)
        regs = torch.empty(1, dtype=torch.float64, device=dev)
    out = {}
    for P in PLAIN_SIZES:
        td00, td90, rms, _ = make_cluster(rng, ml, FP_t, FX_t, P, K_TD, 20.0)
        with torch.cuda.stream(s):
            d0 = torch.from_numpy(td00).to(dev)
            d9 = torch.from_numpy(td90).to(dev)
            rm = torch.from_numpy(rms).to(dev)
            ws = torch.empty(int(L.pgw_workspace_bytes(len(IFOS), 2 * K_TD + 1, P, 1)),
                             dtype=torch.uint8, device=dev)

        def one():
            rc = L.pgw_sky_loop(len(IFOS), P, n_sky, tables.FP.data_ptr(), tables.FX.data_ptr(),
                                rm.data_ptr(), d0.data_ptr(), d9.data_ptr(), 2 * K_TD + 1,
                                tables.ml.data_ptr(), tables.REG0, tables.gamma_regulator,
                                tables.netCC, tables.network_energy_threshold,
                                tables.valid.data_ptr(), tables.valid.numel(),
                                tables.order.data_ptr(), tables.reg_order.data_ptr(),
                                st.data_ptr(), res.data_ptr(), regs.data_ptr(), None,
                                ws.data_ptr(), ws.numel(), s.cuda_stream)
            if rc:
                raise RuntimeError(L.pgw_last_error().decode())

        if reps == 0:
            one()
            s.synchronize()
            continue
        for _ in range(5):
            one()
        s.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(s)
        for _ in range(reps):
            one()
        e1.record(s)
        e1.synchronize()
        out[str(P)] = round(e0.elapsed_time(e1) * 1e3 / reps, 1)
    return out


if __name__ == "__main__":
    main()
