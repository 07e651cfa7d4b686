#!/usr/bin/env python3
"""Benchmark: DEAC generations/s summed over runs on GB300, batched
split-precision engine against the plain FP64 engine on the same runs.

Workload (the batching form, 1024 independent runs in one batch): seeds
1-1024; from each run's seed its genome size M in {1024, 4096, 16384} on
[0, 64], population P in {8, 32, 64}, temperature T in {0.5, 1.35, 3.0} and
model in {standard, hyperbolic, normalization}; two-sided (bfull), N_tau =
128 on [0, beta], the single-run data recipe at its temperature (0.7 N(5,1) +
0.3 N(20,3), sigma = 1e-4 F, noise from the seed; deac_gb300.data
.config3_runs), stop fitness 1.0.  Both engines draw from counter streams
(the batched forms' compact draw layout, deac_batch_set_streams), so the
split engine's every decision equals the plain engine's and the line
records whether every run ended with identical chi^2, best member and
spectrum.

A step is G = 16 generations of every run (one captured graph block).
Launch shapes: the engine's autotuner (deac_batch_autotune) runs once on a
batch of the same runs set up for it alone; the timed batches (and the e2e
batch) take its choice from the per-process cache, so they run no extra
generation and split and plain stay generation for generation alike.
Timing: W untimed warm-up steps, then K steps, each bracketed by CUDA events
on the batch stream; the working set (18 GB) is far larger than L2, so no
flush is needed between steps; the K steps sit between a barrier + device
synchronize on both sides; value is the max over ranks.  With --gpus N
(torchrun), each rank runs its own 1024 seeds (weak scaling, no data-path
collective).

Secondary keys: `config4_full_size`, the batched split-precision form at
full size (4096 runs of M = 16384 on [0, 1024], P = 64, N_tau = 512, 270 GB;
the plain engine on 256 of the same runs, whose chi^2, best member and
spectrum must match); the single-run production scale (8 runs of
N_tau = 128, M = 4096, P = 8, --normalize, reference streams) over an early
window and over a long window of 100,000 generations, where the exact FP64
passes of a converging population weigh more.  `gpu_launches` counts the
engine's kernel launches in the timed steps (its per-generation count, from
the engine, times the generations).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl engine|reference]

--impl reference times the reference's own CPU implementation of the path
(the CPU-order oracle, a restatement of the reference's CPU code path, since
the reference sources are not on the GPU host) on the host cores, one
process per run, on a sample of the same runs.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

REPO = Path(__file__).resolve().parent
for p in (REPO / "deac-cpp_gb300", REPO / "tests"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))

METRIC = "generations/s summed over runs: batched split-precision vs plain FP64, same χ²"
UNIT = "generations/s"
RUNS_PER_GPU = 1024
NT = 128
GENS_PER_STEP = 16
WORKLOAD = ("deac batching form: 1024 ragged runs in one batch (seeds 1-1024; M in {1024, 4096, 16384} on [0,64], "
            "P in {8, 32, 64}, T in {0.5, 1.35, 3.0}, model in {standard, hyperbolic, normalization}, each drawn "
            "from the seed; two-sided bfull, N_tau=128), counter streams; split-precision engine, plain FP64 "
            "engine on the same runs beside it")
DATA = ("synthetic (benchmark recipe per run: 0.7 N(5,1) + 0.3 N(20,3) at the run's temperature, sigma = 1e-4 F, "
        "numpy default_rng(seed))")
# DRAM bytes per unit of the two main kernels, from one ncu capture each of
# the first 64 runs (295.3 MB read + 757.6 MB written over 36.85 M genes;
# 1.2986 GB + 17.5 MB over 4.716 G products)
SLICE_DRAM_BYTES_PER_GENE = (295.264e6 + 757.633e6) / 36847616
CONTRACT_DRAM_BYTES_PER_PRODUCT = (1.298555e9 + 17.477632e6) / 4716494848
# the single-run production scale, for the secondary keys
P1, M1, OMEGA1, T1 = 8, 4096, 512.0, 1.35
LONG_WINDOW = 100_000


def run_specs(rank, n_runs=RUNS_PER_GPU):
    """(config, tau, isf, err, frequency) of the workload's runs on `rank`."""
    import deac_gb300
    from deac_gb300.data import config3_runs

    out = []
    for r in config3_runs(n_runs, first_seed=rank * RUNS_PER_GPU + 1):
        cfg = deac_gb300.make_config(model=r["model"], temperature=r["temperature"], spectra_type="bfull",
                                     population_size=r["population_size"], number_of_generations=1_600_000,
                                     stop_minimum_fitness=1.0, seed=r["seed"])
        out.append((cfg, r["tau"], r["isf"], r["err"], r["frequency"]))
    return out


def config1_specs(rank):
    import deac_gb300
    from deac_gb300.data import config1_data, uniform_grid

    freq = uniform_grid(M1, OMEGA1)
    out = []
    for k in range(8):
        seed = rank * 8 + k + 1
        cfg = deac_gb300.make_config(temperature=T1, spectra_type="bfull", population_size=P1,
                                     number_of_generations=1_600_000, normalize=True, stop_minimum_fitness=1.0,
                                     seed=seed)
        tau, isf, err = config1_data(seed, T1)
        out.append((cfg, tau, isf, err, freq))
    return out


class ClockSampler:
    """nvidia-smi clocks and throttle reasons every 200 ms during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
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

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("nccl")
    return world, rank, local


def barrier_max(value, world, device):
    if world == 1:
        return value
    import torch
    import torch.distributed as dist
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world, device):
    if world > 1:
        import torch
        import torch.distributed as dist
        dist.barrier(device_ids=[device])
    import torch
    torch.cuda.synchronize()


# ------------------------------------------------------------------ CPU side

def _cpu_worker(args):
    """Run `index` of the workload on `rank` for `gens` generations with the
    CPU-order oracle (the reference's CPU code path); returns (generations
    executed, seconds)."""
    rank, index, gens = args
    sys.path.insert(0, str(REPO / "tests"))
    sys.path.insert(0, str(REPO / "deac-cpp_gb300"))
    from deac_testlib import CPU_ORDER, Oracle
    cfg, tau, isf, err, freq = run_specs(rank, index + 1)[index]
    cfg.number_of_generations = gens + 1
    cfg.stop_minimum_fitness = -1.0
    t0 = time.perf_counter()
    r = Oracle().run(cfg, tau, isf, err, freq, order=CPU_ORDER)
    return r["executed"], time.perf_counter() - t0


def ensure_oracle():
    subprocess.run(["make", "-s", "-C", str(REPO / "oracle"), "all"], check=True)


CPU_SAMPLE_RUNS = 16      # the workload's first 16 runs (its mix of M, P, T and models)
CPU_SAMPLE_GENERATIONS = 2


def cpu_sample(rank, pool_size, gens=CPU_SAMPLE_GENERATIONS, rounds=1):
    """Generations/s of the reference's CPU path on the workload's first
    CPU_SAMPLE_RUNS runs, one process per run on `pool_size` host cores."""
    import multiprocessing as mp
    ensure_oracle()
    ctx = mp.get_context("spawn")
    with ctx.Pool(pool_size) as pool:
        t0 = time.perf_counter()
        total = 0
        for _ in range(rounds):
            res = pool.map(_cpu_worker, [(rank, k, gens) for k in range(CPU_SAMPLE_RUNS)])
            total += sum(g for g, _ in res)
        dt = time.perf_counter() - t0
    return total, dt


def cpu_baseline(rank):
    """Bounded sample of the reference CPU path on the workload (all host cores)."""
    cores = min(CPU_SAMPLE_RUNS, os.cpu_count() or 1)
    total, dt = cpu_sample(rank, cores)
    return {"value": total / dt, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"the workload's first {CPU_SAMPLE_RUNS} runs x {CPU_SAMPLE_GENERATIONS} generations, one "
                      f"process per run on {cores} host cores (CPU-order oracle = the reference's CPU code path, "
                      f"including its set-up), {dt:.1f} s"}


def reference_arm(args, world, rank):
    if rank != 0:
        return
    cores = min(CPU_SAMPLE_RUNS, os.cpu_count() or 1)
    for _ in range(args.warmup):
        cpu_sample(0, cores)
    total, dt = cpu_sample(0, cores, rounds=args.steps)
    value = total / dt
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3 / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": DATA,
        "config": {"workload": WORKLOAD + " (reference CPU path on a sample of the runs)", "runs": CPU_SAMPLE_RUNS,
                   "generations_per_run_per_step": CPU_SAMPLE_GENERATIONS, "processes": cores},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"the workload's first {CPU_SAMPLE_RUNS} runs x {CPU_SAMPLE_GENERATIONS} "
                                   f"generations per step, one process per run (CPU-order oracle: the reference's "
                                   f"CPU code path restated; the reference sources are not present on the GPU host)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- GPU side

KEPT_DIGIT_PAIRS = 28   # digit pairs a+b <= 6 of seven 7-bit digits
KERNEL_NAMES = {0: "trial_slice_kernel", 1: "contract_kernel (exact pass)", 2: "norm_kernel",
                3: "split_contract_kernel", 4: "split_combine_kernel+split_select_kernel"}


def workload_sizes(configs):
    rows = sum(c.population_size for c, *_ in configs)
    genes = sum(c.population_size * 2 * len(f) for c, _, _, _, f in configs)  # S = 2 (two-sided)
    # sum over runs of rows x N_tau x M x S: the contraction's products
    products = sum(c.population_size * len(t) * len(f) * 2 for c, t, _, _, f in configs)
    return rows, genes, products


def kernel_roofline(kind, launch_s, peaks, configs):
    """Algorithmic work per launch of kernel kind `kind` and the rate it
    reached, against the measured peak of what bounds it."""
    rows, genes, products = workload_sizes(configs)
    if kind == 0:
        # counter streams (trial slices): every parent gene in once (the
        # donors are read from the staged parents), the trial gene and its
        # seven BF16 digits out
        work, unit, bound, peak = genes * (8 + 8 + 7 * 2), "GB/s", "hbm", peaks["hbm_gbs"]
        achieved = work / launch_s / 1e9
    elif kind == 3:
        work = 2.0 * products * KEPT_DIGIT_PAIRS  # BF16 digit-pair MMA flops (the precision form's algorithm)
        unit, bound, peak = "TFLOP/s", "tensor", peaks["bf16_tflops"]
        achieved = work / launch_s / 1e12
    elif kind == 4:
        work = rows * NT * (16 + 16 + 8)  # partial sums in, estimate + bound out, data / errors in
        unit, bound, peak = "GB/s", "hbm", peaks["hbm_gbs"]
        achieved = work / launch_s / 1e9
    else:  # the exact pass, were every trial re-evaluated; norm_kernel does not run here
        work = 2.0 * products
        unit, bound, peak = "TFLOP/s", "fp64", 1.196
        achieved = work / launch_s / 1e12
    return {"bound": bound, "achieved": achieved, "peak": peak, "unit": unit, "frac": achieved / peak,
            "kernel": KERNEL_NAMES[kind], "work_per_launch": work, "launch_us": launch_s * 1e6}


def load_peaks():
    path = REPO / "MEASURED_PEAKS.json"
    if path.exists():
        d = json.loads(path.read_text())
        return {"hbm_gbs": d["hbm_gbs"], "bf16_tflops": d["bf16_tflops"], "source": "measured (MEASURED_PEAKS.json)"}
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "source": "fallback"}


def make_batch(engine_kind, configs, local, stream, streams):
    import deac_gb300
    b = deac_gb300.Batch(engine=engine_kind, device=local, stream=stream.cuda_stream, streams=streams)
    for cfg, tau, isf, err, freq in configs:
        b.add_run(cfg, tau, isf, err, freq)
    b.setup()
    return b


def timed_engine(engine_kind, configs, args, local, stream, world, sample_clocks, G, streams, flush=None,
                 tuned=False):
    """Set up a batch on `engine_kind`, run the warm-up steps, then time K
    steps of G generations (events on the batch stream).  `tuned`: take the
    launch shapes the autotuner chose for this run mix (from its per-process
    cache, so no generation is run for it)."""
    import torch

    batch = make_batch(engine_kind, configs, local, stream, streams)
    if tuned:
        assert batch.autotune(G)["from_cache"] == 1
    for _ in range(args.warmup):
        batch.launch(G)
    torch.cuda.synchronize()
    assert batch.sync() == 0, "a run finished during warm-up"
    events = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    barrier(world, local)
    clocks = ClockSampler(local) if sample_clocks else None
    if clocks:
        clocks.__enter__()
    try:
        for e0, e1 in events:
            if flush is not None:
                with torch.cuda.stream(stream):
                    flush.zero_()
            e0.record(stream)
            batch.launch(G)
            e1.record(stream)
        stream.synchronize()
        barrier(world, local)
    finally:
        if clocks:
            clocks.__exit__(None, None, None)
    ms = sum(e0.elapsed_time(e1) for e0, e1 in events)
    assert batch.sync() == 0, "a run finished inside the timed region; its generations would not count"
    return batch, ms, (clocks.summary() if clocks else None)


def same_results(a, b, runs):
    """Both batches ran the same generations: identical generation count,
    minimum fitness (chi^2), best member and best spectrum for every run."""
    import numpy as np
    for r in range(runs):
        x, y = a.fetch(r), b.fetch(r)
        if x["generation"] != y["generation"] or x["minimum_fitness"] != y["minimum_fitness"]:
            return False
        if x["best_index"] != y["best_index"] or not np.array_equal(x["dsf"], y["dsf"]):
            return False
    return True


def long_window(configs, local, stream, window):
    """Summed generations/s of both engines over generations 0..window of the
    production-scale runs (reference streams), and the split engine's
    decision counts: the exact FP64 passes grow as the populations converge."""
    import torch
    import deac_gb300
    out = {}
    for name, kind in (("split", deac_gb300.ENGINE_SPLIT_BF16), ("plain", deac_gb300.ENGINE_PLAIN_FP64)):
        b = make_batch(kind, configs, local, stream, "reference")
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        b.launch(window)
        e1.record(stream)
        stream.synchronize()
        done = b.sync()
        ms = e0.elapsed_time(e1)
        # a run that reached its stop executed its reported generations
        executed = 0
        for r in range(len(configs)):
            res_r = b.result(r)
            executed += res_r["generation"] if res_r["finished"] else window
        res = {"value": executed / (ms / 1e3), "seconds": ms / 1e3, "runs_finished": done,
               "generations_executed": executed}
        if kind == deac_gb300.ENGINE_SPLIT_BF16:
            c = [b.split_counts(r) for r in range(len(configs))]
            res["decisions"] = {k: sum(x[k] for x in c) for k in c[0]}
            tot = sum(res["decisions"].values())
            res["exact_fraction"] = res["decisions"]["exact"] / tot if tot else 0.0
        out[name] = (b, res)
    same = same_results(out["split"][0], out["plain"][0], len(configs))
    line = {"generations": window, "runs": len(configs),
            "split": out["split"][1], "plain": out["plain"][1],
            "split_over_plain": out["split"][1]["value"] / out["plain"][1]["value"],
            "same_chi2_and_spectra": same}
    for b, _ in out.values():
        b.close()
    return line


C4_RUNS, C4_PLAIN_RUNS, C4_WARMUP, C4_STEPS = 4096, 256, 2, 4
C4_GB = 272  # device memory the full-size split batch needs


def config4_key(local, stream):
    """The batched split-precision form at full size: 4096 runs of M = 16384,
    P = 64, N_tau = 512 in one split batch (270 GB), C4_STEPS generations
    timed after C4_WARMUP; beside it the plain FP64 engine on the first 256 of
    the same runs, whose chi^2, best member and spectrum must equal the split
    engine's on those runs.  The plain engine's summed generations/s is flat
    once its batch fills the GPU (64 such runs already do; its work per
    generation grows linearly with the runs), so its rate on 256 runs stands
    for its rate on all 4096."""
    import numpy as np
    import torch
    import deac_gb300
    from deac_gb300.data import config4_runs

    free = torch.cuda.mem_get_info(local)[0] / 1e9
    if free < C4_GB:
        return {"skipped": f"needs {C4_GB} GB of device memory, {free:.0f} GB free"}
    tau, freq, runs = config4_runs(C4_RUNS)
    cfgs = [deac_gb300.make_config(temperature=1.35, spectra_type="bfull", population_size=64,
                                   number_of_generations=1_000_000, stop_minimum_fitness=1.0, seed=seed)
            for seed, _, _ in runs]
    out = {"runs": C4_RUNS, "genome_size": len(freq), "population_size": 64, "number_of_timeslices": len(tau),
           "generations_timed": C4_STEPS, "warmup_generations": C4_WARMUP}

    def arm(kind, n):
        b = deac_gb300.Batch(engine=kind, device=local, stream=stream.cuda_stream, streams="counter")
        for cfg, (seed, isf, err) in zip(cfgs[:n], runs[:n]):
            b.add_run(cfg, tau, isf, err, freq)
        t0 = time.perf_counter()
        b.setup()
        setup_s = time.perf_counter() - t0
        b.launch(C4_WARMUP)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        b.launch(C4_STEPS)
        e1.record(stream)
        stream.synchronize()
        assert b.sync() == 0, "a run finished inside the timed window"
        ms = e0.elapsed_time(e1)
        return b, {"value": n * C4_STEPS / (ms / 1e3), "unit": UNIT, "ms_per_generation": ms / C4_STEPS,
                   "setup_s": setup_s}

    split, out["split"] = arm(deac_gb300.ENGINE_SPLIT_BF16, C4_RUNS)
    c = [split.split_counts(r) for r in range(C4_RUNS)]
    out["split"]["decisions"] = {k: sum(x[k] for x in c) for k in c[0]}
    split.enable_timing(True)
    split.launch(1)
    out["split"]["kernel_ms_per_generation"] = {KERNEL_NAMES[k]: round(ms_k / cnt, 3)
                                                for k, (ms_k, cnt) in
                                                ((k, split.kernel_time(k)) for k in range(5)) if cnt}
    split.enable_timing(False)
    ref = [split.fetch(r) for r in range(C4_PLAIN_RUNS)]
    split.close()
    del split
    torch.cuda.empty_cache()
    plain, out["plain"] = arm(deac_gb300.ENGINE_PLAIN_FP64, C4_PLAIN_RUNS)
    out["plain"]["runs"] = C4_PLAIN_RUNS
    plain.launch(1)  # the generation the timing pass added to the split batch
    plain.sync()
    same = True
    for r in range(C4_PLAIN_RUNS):
        y = plain.fetch(r)
        x = ref[r]
        same = same and x["generation"] == y["generation"] and x["minimum_fitness"] == y["minimum_fitness"] \
            and x["best_index"] == y["best_index"] and np.array_equal(x["dsf"], y["dsf"])
    plain.close()
    out["same_chi2_and_spectra_on_plain_runs"] = same
    out["split_over_plain"] = out["split"]["value"] / out["plain"]["value"]
    return out


def engine_arm(args, world, rank, local):
    import torch
    import deac_gb300

    torch.cuda.set_device(local)
    device = torch.device("cuda", local)
    stream = torch.cuda.Stream(device=device)
    configs = run_specs(rank, args.runs)
    G = args.generations_per_step
    n = len(configs)

    # the launch shapes for this run mix: the autotuner on a batch of the
    # same runs set up for it alone (its generations advance that batch
    # only), cached for the process
    tb = make_batch(deac_gb300.ENGINE_SPLIT_BF16, configs, local, stream, "counter")
    tb.launch(G)
    tune = tb.autotune(G)
    tb.close()
    # the headline: the split-precision engine; beside it the plain FP64
    # engine on the same runs and the same generations
    split, ms, clocks = timed_engine(deac_gb300.ENGINE_SPLIT_BF16, configs, args, local, stream, world, True, G,
                                     "counter", tuned=True)
    counts = [split.split_counts(r) for r in range(n)]
    launches_per_generation = split.generation_launches()
    # per-kernel device time (kernels launched one by one, bracketed by
    # events on the batch stream), for the roofline of the dominant kernel
    split.enable_timing(True)
    split.launch(1)
    kt = {k: split.kernel_time(k) for k in range(5)}
    split.enable_timing(False)
    plain, ms_plain, _ = timed_engine(deac_gb300.ENGINE_PLAIN_FP64, configs, args, local, stream, world, False, G,
                                      "counter")
    plain.launch(1)  # the generation the timing pass added to the split batch
    plain.sync()
    identical = same_results(split, plain, n)
    plain.close()
    split.close()
    ms = barrier_max(ms, world, device)
    ms_plain = barrier_max(ms_plain, world, device)
    gens_total = world * n * args.steps * G
    value = gens_total / (ms / 1e3)
    value_plain = gens_total / (ms_plain / 1e3)

    per_gen_us = {k: ms_k * 1e3 for k, (ms_k, cnt) in kt.items() if cnt}
    dominant = max(per_gen_us, key=per_gen_us.get)
    ms_d, n_d = kt[dominant]
    peaks = load_peaks()
    roof = kernel_roofline(dominant, ms_d / n_d / 1e3, peaks, configs)
    roof["peak_source"] = peaks["source"] + (" burst figure" if roof["bound"] != "fp64" else
                                             "; FP64: measured DFMA throughput")
    # DRAM bytes per launch: an ncu capture of the first 64 runs (too large
    # to capture whole), scaled to this launch by its genes or products
    rows_, genes_, products_ = workload_sizes(configs)
    traffic = {0: genes_ * SLICE_DRAM_BYTES_PER_GENE, 3: products_ * CONTRACT_DRAM_BYTES_PER_PRODUCT}.get(dominant)
    roof["traffic"] = traffic
    if traffic is not None:
        roof["traffic_source"] = ("ncu dram__bytes_read.sum + dram__bytes_write.sum of one launch on the first 64 "
                                  "runs, scaled by " + ("genes" if dominant == 0 else "products"))
    roof["per_generation_us"] = {KERNEL_NAMES[k]: round(v, 1) for k, v in per_gen_us.items()}

    # end to end through the public API with host buffers: create + add runs
    # (host arrays) + setup (host build, H2D) + K steps of (G generations,
    # then every run's status read back), then every run's result and best
    # spectrum fetched (Batch.fetch_all)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    b2 = deac_gb300.Batch(engine=deac_gb300.ENGINE_SPLIT_BF16, device=local, stream=stream.cuda_stream,
                          streams="counter")
    for cfg, tau, isf, err, freq in configs:
        b2.add_run(cfg, tau, isf, err, freq)
    b2.setup()
    b2.autotune(G)  # the process's cached choice for this run mix
    for _ in range(args.steps):
        b2.launch(G)
        b2.sync()
    b2.fetch_all()
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    # every byte the engine copied (inputs, initial parents, kernel matrices,
    # work lists, status reads, result snapshot), as it counted them
    h2d, d2h = b2.transfer_bytes()
    b2.close()
    e2e_value = gens_total / barrier_max(e2e_s, world, device)

    # secondary: the single-run production scale, 8 runs
    c1 = config1_specs(rank)
    early = {}
    if not args.no_secondary:
        import copy
        a1 = copy.copy(args)
        a1.steps, a1.warmup = 10, 3
        s1, ms1, _ = timed_engine(deac_gb300.ENGINE_SPLIT_BF16, c1, a1, local, stream, world, False, 32, "reference")
        p1, ms1p, _ = timed_engine(deac_gb300.ENGINE_PLAIN_FP64, c1, a1, local, stream, world, False, 32,
                                   "reference")
        early = {"generations": "32 x 10 after 96 warm-up", "split": 8 * 320 / (ms1 / 1e3),
                 "plain": 8 * 320 / (ms1p / 1e3), "same_chi2_and_spectra": same_results(s1, p1, 8)}
        early["split_over_plain"] = early["split"] / early["plain"]
        s1.close()
        p1.close()
        longw = long_window(c1, local, stream, args.long_window)

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64 (FP64-identical results; contraction from exact bf16 digit slices)",
        "data": DATA,
        "config": {"workload": WORKLOAD if n == RUNS_PER_GPU else f"the first {n} runs of: " + WORKLOAD,
                   "runs_per_gpu": n, "number_of_timeslices": NT,
                   "population_rows": sum(c.population_size for c, *_ in configs),
                   "generations_per_step": G, "engine": "split_bf16", "streams": "counter",
                   "l2": "no flush: the batch's working set (18 GB) is far larger than L2"},
        "plain_fp64": {"value": value_plain, "unit": UNIT, "ms_per_step": ms_plain / args.steps,
                       "split_over_plain": value / value_plain,
                       "same_chi2_and_spectra": identical},
        "split_decisions": {"equal_to_parent": sum(c["equal_to_parent"] for c in counts),
                            "by_interval": sum(c["interval"] for c in counts),
                            "by_exact_fp64": sum(c["exact"] for c in counts)},
        "autotune": {"parts_per_cta": tune["parts_per_cta"], "split_waves": tune["split_waves"],
                     "ms_per_generation": tune["ms_per_generation"],
                     "ms_per_generation_default": tune["ms_per_generation_default"]},
        "roofline": roof,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d // args.steps,
                "d2h_bytes_per_step": d2h // args.steps,
                "includes": "batch creation, set-up from host arrays, K steps with a status read each, "
                            "every run's result and best spectrum fetched at the end (one batched call)"},
        # per generation: trial slices, tensor contraction, (the partial-sum
        # combine where tiles are split), selection, the exact pass
        "gpu_launches": launches_per_generation * G * args.steps,
        "clocks": clocks,
    }
    if early:
        line["config1_early_window"] = early
        line["config1_long_window"] = longw
    if not args.no_config4 and world == 1:
        line["config4_full_size"] = config4_key(local, stream)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(rank)
    if rank == 0:
        print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--generations-per-step", type=int, default=GENS_PER_STEP)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-secondary", action="store_true", help="skip the single-run production-scale keys")
    ap.add_argument("--long-window", type=int, default=LONG_WINDOW)
    ap.add_argument("--no-config4", action="store_true", help="skip the full-size batched split key (270 GB)")
    ap.add_argument("--runs", type=int, default=RUNS_PER_GPU,
                    help="the workload's first RUNS runs (smaller cases for profiling; the line is for 1024)")
    args = ap.parse_args()
    if args.impl == "reference":
        # CPU only: rank 0 measures, the other ranks exit without work
        world = int(os.environ.get("WORLD_SIZE", "1"))
        reference_arm(args, world, int(os.environ.get("RANK", "0")))
        return
    world, rank, local = dist_setup()
    engine_arm(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
