"""Shared helpers for the DEAC tests and bench.

- ``DeacConfig``: ctypes mirror of ``deac_config`` (include/deac_gb300.h).
- ``Oracle``: ctypes binding of the CPU oracle (oracle/_build/libdeac_oracle.so),
  which is test infrastructure only.
- ``make_isf``: the synthetic-data recipe of the benchmark configurations
  (Gaussian-mixture S(omega), detailed-balance F(tau), sigma = rel * F,
  F_data = F + sigma * N(0,1) from numpy's default_rng(seed)).
- ``run_reference`` / ``read_outputs``: run a deac.e-compatible executable and
  read back the files it writes (format of deac.cpp:51-56, 1687-1769).
"""
from __future__ import annotations

import ctypes
import os
import re
import struct
import subprocess
import sys
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parents[1]
ORACLE_SO = REPO / "oracle" / "_build" / "libdeac_oracle.so"
REF_DIR = REPO / "oracle" / "_ref"

GPU_ORDER, CPU_ORDER, GPU_ORDER_COUNTER = 0, 1, 2

PKG_DIR = REPO / "deac-cpp_gb300"
if str(PKG_DIR) not in sys.path:
    sys.path.insert(0, str(PKG_DIR))
from deac_gb300 import MODEL, SPECTRA, DeacConfig, make_config  # noqa: E402


class OracleOut(ctypes.Structure):
    _fields_ = [
        ("generation", ctypes.c_uint64),
        ("minimum_fitness", ctypes.c_double),
        ("best_index", ctypes.c_uint64),
        ("spectrum_length", ctypes.c_uint64),
        ("stats_length", ctypes.c_uint64),
        ("generations_executed", ctypes.c_uint64),
    ]


_dp = ctypes.POINTER(ctypes.c_double)


def _ptr(a):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_dp)


class Oracle:
    """ctypes binding of the C oracle (test infrastructure)."""

    def __init__(self, path: Path = ORACLE_SO):
        if not Path(path).exists():
            raise FileNotFoundError(f"{path} not built (run `make -C oracle`)")
        self.lib = ctypes.CDLL(str(path))
        self.lib.deac_oracle_run.restype = ctypes.c_int
        self.lib.deac_oracle_run.argtypes = [
            ctypes.POINTER(DeacConfig), ctypes.c_int32,
            _dp, _dp, _dp, ctypes.c_uint64, _dp, ctypes.c_uint64,
            ctypes.POINTER(OracleOut), _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp,
            ctypes.c_uint64,
        ]
        self.lib.deac_oracle_kernel_matrix.restype = ctypes.c_int
        self.lib.deac_oracle_kernel_matrix.argtypes = [
            ctypes.POINTER(DeacConfig), _dp, ctypes.c_uint64, _dp, ctypes.c_uint64, _dp, _dp]
        self.lib.deac_oracle_rng_next.restype = ctypes.c_uint64
        self.lib.deac_oracle_rng_next.argtypes = [ctypes.POINTER(ctypes.c_uint64)]
        self.lib.deac_oracle_rng_init.argtypes = [ctypes.c_uint64, ctypes.POINTER(ctypes.c_uint64)]
        self.lib.deac_oracle_rng_jump.argtypes = [ctypes.POINTER(ctypes.c_uint64)]
        self.lib.deac_oracle_stream_draw.restype = ctypes.c_uint64
        self.lib.deac_oracle_stream_draw.argtypes = [ctypes.c_uint64, ctypes.c_uint64]
        self.lib.deac_oracle_stream_keys.argtypes = [ctypes.c_uint64, ctypes.POINTER(ctypes.c_uint64)]

    def run(self, cfg: DeacConfig, tau, isf, err, freq, order=GPU_ORDER, trace=0,
            state=False):
        tau, isf, err, freq = (np.ascontiguousarray(x, dtype=np.float64) for x in (tau, isf, err, freq))
        nt, m = len(tau), len(freq)
        p = cfg.population_size
        s = 1 if cfg.bosonic else 2
        spec = 2 * m - 1 if s == 2 else m
        n = cfg.number_of_generations
        out = OracleOut()
        dsf = np.zeros(spec)
        fr = np.zeros(spec)
        st = [np.zeros(n) for _ in range(3)] if cfg.track_stats else [None] * 3
        pop = np.zeros(s * p * m) if state else None
        fit = np.zeros(p) if state else None
        tr = np.zeros(trace * p) if trace else None
        rc = self.lib.deac_oracle_run(
            ctypes.byref(cfg), order, _ptr(tau), _ptr(isf), _ptr(err), nt, _ptr(freq), m,
            ctypes.byref(out), _ptr(dsf), _ptr(fr), _ptr(st[0]), _ptr(st[1]), _ptr(st[2]),
            _ptr(pop), _ptr(fit), _ptr(tr), trace)
        if rc != 0:
            raise ValueError("oracle rejected the configuration")
        res = {
            "generation": out.generation,
            "minimum_fitness": out.minimum_fitness,
            "best_index": out.best_index,
            "executed": out.generations_executed,
            "dsf": dsf,
            "frequency": fr,
        }
        if cfg.track_stats:
            k = out.stats_length
            res["stats_mean"], res["stats_minimum"], res["stats_squared_mean"] = (a[:k] for a in st)
        if state:
            res["population"] = pop.reshape(s, p, m)
            res["fitness"] = fit
        if trace:
            res["trace"] = tr.reshape(trace, p)[: min(trace, out.generations_executed)]
        return res

    def kernel_matrix(self, cfg, tau, freq):
        tau = np.ascontiguousarray(tau, dtype=np.float64)
        freq = np.ascontiguousarray(freq, dtype=np.float64)
        kp = np.zeros((len(tau), len(freq)))
        kn = np.zeros((len(tau), len(freq))) if not cfg.bosonic else None
        rc = self.lib.deac_oracle_kernel_matrix(ctypes.byref(cfg), _ptr(tau), len(tau), _ptr(freq),
                                                len(freq), _ptr(kp), _ptr(kn))
        assert rc == 0
        return kp, kn

    def stream_draw(self, key: int, pos: int) -> int:
        return self.lib.deac_oracle_stream_draw(key, pos)

    def stream_keys(self, seed: int):
        k = (ctypes.c_uint64 * 2)()
        self.lib.deac_oracle_stream_keys(seed, k)
        return k[0], k[1]

    def rng_stream(self, seed: int, n: int, jumps: int = 0):
        s = (ctypes.c_uint64 * 4)()
        self.lib.deac_oracle_rng_init(seed, s)
        for _ in range(jumps):
            self.lib.deac_oracle_rng_jump(s)
        return [self.lib.deac_oracle_rng_next(s) for _ in range(n)]


# ----------------------------------------------------------------- data recipe
from deac_gb300.data import (config0_data, config1_data, config2_data, gaussian, make_isf,  # noqa: E402,F401
                             uniform_grid)


# ------------------------------------------------------------ files / binaries

def write_doubles(path, values):
    Path(path).write_bytes(np.asarray(values, dtype="<f8").tobytes())


def read_doubles(path):
    data = Path(path).read_bytes()
    assert len(data) % 8 == 0
    return np.frombuffer(data, dtype="<f8").copy()


def write_isf(path, tau, isf, err):
    write_doubles(path, np.concatenate([tau, isf, err]))


def read_log_value(path, key):
    m = re.search(rf"^{re.escape(key)}: (.+)$", Path(path).read_text(), re.MULTILINE)
    return m.group(1) if m else None


def run_exe(exe, args, workdir, timeout=600):
    return subprocess.run([str(exe)] + [str(a) for a in args], cwd=workdir,
                          stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True,
                          timeout=timeout)


def read_outputs(save_dir, prefix, uuid, track_stats=False):
    save_dir = Path(save_dir)
    out = {
        "dsf": read_doubles(save_dir / f"{prefix}_dsf_{uuid}.bin"),
        "frequency": read_doubles(save_dir / f"{prefix}_frequency_{uuid}.bin"),
        "log": (save_dir / f"{prefix}_log_{uuid}.dat").read_text(),
    }
    log = save_dir / f"{prefix}_log_{uuid}.dat"
    out["generation"] = int(read_log_value(log, "generation"))
    out["minimum_fitness_text"] = read_log_value(log, "minimum_fitness")
    if track_stats:
        for k, name in (("stats_mean", "fitness-mean"), ("stats_minimum", "fitness-minimum"),
                        ("stats_squared_mean", "fitness-squared-mean")):
            out[k] = read_doubles(save_dir / f"{prefix}_stats_{name}_{uuid}.bin")
    return out


def cli_args(cfg: DeacConfig, isf_file, save_dir, frequency_file=None, genome_size=None,
             omega_max=None, uuid=None):
    """deac.e arguments that reproduce ``cfg`` (reference flag names)."""
    a = ["-T", repr(cfg.temperature), "-N", cfg.number_of_generations,
         "-P", cfg.population_size, "--seed", cfg.seed,
         "-r", repr(cfg.crossover_probability), "-u", repr(cfg.self_adapting_crossover_probability),
         "-F", repr(cfg.differential_weight), "-v", repr(cfg.self_adapting_differential_weight_probability),
         "--stop_minimum_fitness", repr(cfg.stop_minimum_fitness),
         "--save_directory", save_dir]
    if frequency_file is not None:
        a += ["--frequency_file", frequency_file]
    else:
        a += ["-M", genome_size, "--omega_max", repr(omega_max)]
    if cfg.normalize:
        a.append("--normalize")
    if cfg.use_negative_first_moment:
        a.append("--use_negative_first_moment")
    if cfg.first_moment >= 0:
        a += ["--first_moment", repr(cfg.first_moment)]
    if cfg.third_moment >= 0:
        a += ["--third_moment", repr(cfg.third_moment), "--third_moment_error", repr(cfg.third_moment_error)]
    if cfg.track_stats:
        a.append("--track_stats")
    inv = {v: k for k, v in SPECTRA.items()}
    a += ["--spectra_type", inv[cfg.spectra_type]]
    if uuid is not None:
        a += ["--uuid", uuid]
    a.append(isf_file)
    return a


def reference_exe_for(cfg: DeacConfig):
    """oracle/_ref executable for the variant of ``cfg`` (None if absent)."""
    name = {0: "std", 1: "hyp", 2: "norm"}[cfg.model]
    if cfg.zero_temperature:
        name = "zT"
    if cfg.bosonic:
        name += "_bos"
    if cfg.allow_negative_weight:
        name += "_neg"
    exe = REF_DIR / f"deac_{name}.e"
    return exe if exe.exists() else None


def output_prefix(cfg: DeacConfig):
    inv = {v: k for k, v in SPECTRA.items()}
    return ("deac-zT" if cfg.zero_temperature else "deac-") + inv[cfg.spectra_type]
