#!/usr/bin/env python3
"""Benchmark: DEAC generations/s summed over runs on GB300.

Workload (the reference's production scale, BASELINE config 1): 8 runs,
seeds 1-8, standard model, two-sided (--spectra_type bfull), T = 1.35,
N_tau = 128 on [0, beta], M = 4096 on omega in [0, 512], P = 8, --normalize,
stop fitness 1.0 (not reached in the timed generations).  Synthetic data by
the benchmark recipe (deac_gb300.data.config1_data).

A step is G generations of every run of the batch.  The headline is the
split-precision engine (contraction from exact BF16 digit slices on the
tcgen05 tensor cores, every selection decision equal to FP64); the plain
FP64 engine runs the same generations beside it, and the line records
whether both ended with identical chi^2 and spectra.  Timing: W untimed
warm-up steps, then K steps, each bracketed by CUDA events on the batch
stream, with a 256 MB L2 flush before each step (outside the events); the K
steps sit between a barrier + device synchronize on both sides; value is
the max over ranks.  With --gpus N (torchrun), each rank runs its own 8
seeds (weak scaling, no data-path collective).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl engine|reference]

--impl reference times the reference's own CPU implementation of the path
(the CPU-order oracle, a restatement of the reference's CPU code path, since
the reference sources are not on the GPU host) on the host cores, one
process per run, on the same workload.
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
RUNS_PER_GPU = 8
P, M, NT, OMEGA_MAX, T = 8, 4096, 128, 512.0, 1.35
GENS_PER_STEP = 32
WORKLOAD = ("deac config 1: 8 runs (seeds 1-8), standard model, two-sided bfull, T=1.35, "
            "N_tau=128, M=4096 on [0,512], P=8, --normalize; split-precision engine, plain FP64 engine beside it")
DATA = "synthetic (benchmark recipe: 0.7 N(5,1) + 0.3 N(20,3), sigma = 1e-4 F, numpy default_rng(seed))"
CPU_SAMPLE_GENERATIONS = 1000


def run_configs(rank):
    import deac_gb300
    from deac_gb300.data import config1_data, uniform_grid

    freq = uniform_grid(M, OMEGA_MAX)
    out = []
    for k in range(RUNS_PER_GPU):
        seed = rank * RUNS_PER_GPU + k + 1
        cfg = deac_gb300.make_config(temperature=T, spectra_type="bfull", population_size=P,
                                     number_of_generations=1_600_000, normalize=True, stop_minimum_fitness=1.0,
                                     seed=seed)
        tau, isf, err = config1_data(seed, T)
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
    """One reconstruction of `gens` generations with the CPU-order oracle (the
    reference's CPU path); returns (generations executed, seconds)."""
    seed, gens = args
    sys.path.insert(0, str(REPO / "tests"))
    sys.path.insert(0, str(REPO / "deac-cpp_gb300"))
    from deac_testlib import CPU_ORDER, Oracle
    import deac_gb300
    from deac_gb300.data import config1_data, uniform_grid
    cfg = deac_gb300.make_config(temperature=T, spectra_type="bfull", population_size=P,
                                 number_of_generations=gens + 1, normalize=True, stop_minimum_fitness=-1.0,
                                 seed=seed)
    tau, isf, err = config1_data(seed, T)
    t0 = time.perf_counter()
    r = Oracle().run(cfg, tau, isf, err, uniform_grid(M, OMEGA_MAX), order=CPU_ORDER)
    return r["executed"], time.perf_counter() - t0


def ensure_oracle():
    subprocess.run(["make", "-s", "-C", str(REPO / "oracle"), "all"], check=True)


def cpu_baseline():
    """Bounded single-core sample of the reference CPU path on the workload."""
    ensure_oracle()
    gens, secs = _cpu_worker((1, CPU_SAMPLE_GENERATIONS))
    return {"value": gens / secs, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"seed 1 of the workload, {gens} generations, one core "
                      f"(CPU-order oracle = the reference's CPU code path), {secs:.1f} s"}


def reference_arm(args, world, rank):
    if rank != 0:
        return
    import multiprocessing as mp
    ensure_oracle()
    gens = 48  # per run per step: ~0.6 s of CPU work per run
    cores = min(RUNS_PER_GPU, os.cpu_count() or 1)
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores) as pool:
        for _ in range(args.warmup):
            pool.map(_cpu_worker, [(s + 1, gens) for s in range(RUNS_PER_GPU)])
        t0 = time.perf_counter()
        total = 0
        for _ in range(args.steps):
            res = pool.map(_cpu_worker, [(s + 1, gens) for s in range(RUNS_PER_GPU)])
            total += sum(g for g, _ in res)
        dt = time.perf_counter() - t0
    value = total / dt
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3 / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": DATA,
        "config": {"workload": WORKLOAD + " (reference CPU path)", "runs": RUNS_PER_GPU,
                   "generations_per_run_per_step": gens, "processes": cores},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"{RUNS_PER_GPU} runs x {gens} generations per step, one process per run "
                                   f"(CPU-order oracle: the reference's CPU code path restated; the reference "
                                   f"sources are not present on the GPU host)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- GPU side

# Algorithmic work per launch of each kernel kind of the split engine
# (deac_batch_kernel_time kinds), for the roofline of the dominant one.
BYTES_PER_TRIAL_GENE = 4 * 8 + 2 * 32 + 8 + 7 * 2   # parent+3 donors, PRNG state in/out, gene out, 7 BF16 digits out
BYTES_PER_NORM_GENE = 8 + 8                         # raw gene and its weight in
KEPT_DIGIT_PAIRS = 28                               # digit pairs a+b <= 6 of seven 7-bit digits


def kernel_roofline(kind, launch_s, peaks, split_ctas):
    S, rows = 2, RUNS_PER_GPU * P
    genes = RUNS_PER_GPU * P * S * M
    if kind == 0:
        work, unit, bound, peak = genes * BYTES_PER_TRIAL_GENE, "GB/s", "hbm", peaks["hbm_gbs"]
        achieved = work / launch_s / 1e9
        name = "trial_part_kernel"
    elif kind == 2:
        # exact normalisation row sums: each trial's raw genes and the weights
        work, unit, bound, peak = genes * BYTES_PER_NORM_GENE, "GB/s", "hbm", peaks["hbm_gbs"]
        achieved = work / launch_s / 1e9
        name = "norm_kernel"
    elif kind == 3:
        work = 2.0 * rows * NT * M * S * KEPT_DIGIT_PAIRS
        unit, bound, peak = "TFLOP/s", "tensor", peaks["bf16_tflops"]
        achieved = work / launch_s / 1e12
        name = "split_contract_kernel"
    elif kind == 4:
        work = 16.0 * rows * NT * split_ctas + rows * NT * 16  # partial sums in, estimate + bound out
        unit, bound, peak = "GB/s", "hbm", peaks["hbm_gbs"]
        achieved = work / launch_s / 1e9
        name = "split_combine_kernel+split_select_kernel"
    else:  # kind 1
        work = 2.0 * 2 * rows * NT * M  # FP64 FMA chains, were every trial re-evaluated
        unit, bound, peak = "TFLOP/s", "fp64", 1.196
        achieved = work / launch_s / 1e12
        name = "contract_kernel (exact pass)"
    return {"bound": bound, "achieved": achieved, "peak": peak, "unit": unit, "frac": achieved / peak,
            "kernel": name, "work_per_launch": work, "launch_us": launch_s * 1e6}


def load_peaks():
    path = REPO / "MEASURED_PEAKS.json"
    if path.exists():
        d = json.loads(path.read_text())
        return {"hbm_gbs": d["hbm_gbs"], "bf16_tflops": d["bf16_tflops"], "source": "measured (MEASURED_PEAKS.json)"}
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "source": "fallback"}


def timed_engine(engine_kind, configs, args, local, stream, flush, world, sample_clocks):
    """Set up a batch of the workload on `engine_kind`, run the warm-up steps,
    then time K steps of G generations (events on the batch stream, L2
    flushed before every step)."""
    import torch
    import deac_gb300

    G = args.generations_per_step
    batch = deac_gb300.Batch(engine=engine_kind, device=local, stream=stream.cuda_stream)
    for cfg, tau, isf, err, freq in configs:
        batch.add_run(cfg, tau, isf, err, freq)
    batch.setup()
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
    """Both batches ran the same generations: identical minimum fitness (chi^2),
    best member and best spectrum for every run."""
    import numpy as np
    for r in range(runs):
        x, y = a.fetch(r), b.fetch(r)
        if x["generation"] != y["generation"] or x["minimum_fitness"] != y["minimum_fitness"]:
            return False
        if x["best_index"] != y["best_index"] or not np.array_equal(x["dsf"], y["dsf"]):
            return False
    return True


def engine_arm(args, world, rank, local):
    import torch
    import deac_gb300

    torch.cuda.set_device(local)
    device = torch.device("cuda", local)
    stream = torch.cuda.Stream(device=device)
    configs = run_configs(rank)
    G = args.generations_per_step
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=device)

    # the headline: the split-precision engine; beside it the plain FP64
    # engine on the same runs and the same generations
    split, ms, clocks = timed_engine(deac_gb300.ENGINE_SPLIT_BF16, configs, args, local, stream, flush, world, True)
    plain, ms_plain, _ = timed_engine(deac_gb300.ENGINE_PLAIN_FP64, configs, args, local, stream, flush, world,
                                      False)
    identical = same_results(split, plain, len(configs))
    counts = [split.split_counts(r) for r in range(len(configs))]
    plain.close()
    ms = barrier_max(ms, world, device)
    ms_plain = barrier_max(ms_plain, world, device)
    gens_total = world * RUNS_PER_GPU * args.steps * G
    value = gens_total / (ms / 1e3)
    value_plain = gens_total / (ms_plain / 1e3)

    # per-kernel device time (separate pass, kernels launched one by one and
    # bracketed by events on the batch stream)
    split.enable_timing(True)
    split.launch(G)
    kt = {k: split.kernel_time(k) for k in range(5)}
    split.enable_timing(False)
    split.close()
    # CTAs of the split contraction: one tile (64 rows x 128 timeslices) whose
    # M/32 chunks are spread over the SMs the normalisation row sums (one CTA
    # per trial, beside it) leave free
    chunks = M // 32
    sms = torch.cuda.get_device_properties(device).multi_processor_count
    free = sms - min(RUNS_PER_GPU * P, sms // 2)
    per = -(-chunks // min(max(1, free), chunks))
    split_ctas = -(-chunks // per)
    per_gen_us = {k: ms_k / G * 1e3 for k, (ms_k, n) in kt.items() if n}
    dominant = max(per_gen_us, key=per_gen_us.get)
    ms_d, n_d = kt[dominant]
    peaks = load_peaks()
    roof = kernel_roofline(dominant, ms_d / n_d / 1e3, peaks, split_ctas)
    roof["peak_source"] = peaks["source"] + (" burst figure" if roof["bound"] != "fp64" else
                                             "; FP64: measured DFMA throughput (profiles/fp64_pipe_gb300.md)")
    tpath = REPO / "profiles" / f"{roof['kernel'].split('+')[0].split(' ')[0]}_config1_traffic.json"
    roof["traffic"] = json.loads(tpath.read_text()).get("bytes_per_launch") if tpath.exists() else None
    names = {0: "trial_part_kernel", 1: "contract_kernel (exact pass)", 2: "norm_kernel",
             3: "split_contract_kernel", 4: "split_combine_kernel+split_select_kernel"}
    roof["per_generation_us"] = {names[k]: round(v, 2) for k, v in per_gen_us.items()}

    # end to end through the public API with host buffers: create + add runs
    # (host arrays) + setup (host build, H2D) + K steps of (G generations,
    # then every run's best spectrum and minimum fitness read back)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    b2 = deac_gb300.Batch(engine=deac_gb300.ENGINE_SPLIT_BF16, device=local, stream=stream.cuda_stream)
    h2d = 0
    for cfg, tau, isf, err, freq in configs:
        b2.add_run(cfg, tau, isf, err, freq)
        # isf and its errors, the normalisation weights of both sides, the
        # initial parents, CR and F (the PRNG table and K's digit planes
        # are formed on the device)
        s = 2
        h2d += 8 * (2 * NT + s * M + s * P * M + 4 * s * P)
    h2d += 8 * 2 * NT * M  # the shared kernel matrix
    b2.setup()
    d2h = 0
    for _ in range(args.steps):
        b2.launch(G)
        for r in range(len(configs)):
            out = b2.fetch(r)
            d2h += 8 * (len(out["dsf"]) + P) + P
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    b2.close()
    e2e_value = gens_total / barrier_max(e2e_s, world, device)

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64 (FP64-identical results; contraction from exact bf16 digit slices)",
        "data": DATA,
        "config": {"workload": WORKLOAD, "runs_per_gpu": RUNS_PER_GPU, "population_size": P, "genome_size": M,
                   "number_of_timeslices": NT, "normalize": True, "generations_per_step": G,
                   "engine": "split_bf16", "l2": "flushed before every timed step (256 MB write, untimed)"},
        "plain_fp64": {"value": value_plain, "unit": UNIT, "ms_per_step": ms_plain / args.steps,
                       "split_over_plain": value / value_plain,
                       "same_chi2_and_spectra": identical},
        "split_decisions": {"equal_to_parent": sum(c["equal_to_parent"] for c in counts),
                            "by_interval": sum(c["interval"] for c in counts),
                            "by_exact_fp64": sum(c["exact"] for c in counts)},
        "roofline": roof,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d // args.steps,
                "d2h_bytes_per_step": d2h // args.steps},
        # per generation: trial parts, normalisation row sums, tensor
        # contraction, combine, selection, the exact pass
        "gpu_launches": 6 * G * args.steps,
        "clocks": clocks,
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline()
    if rank == 0:
        print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--generations-per-step", type=int, default=GENS_PER_STEP)
    ap.add_argument("--no-cpu-baseline", action="store_true")
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
