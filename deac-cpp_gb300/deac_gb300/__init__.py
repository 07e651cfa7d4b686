"""Python binding of the GB300 DEAC engine (include/deac_gb300.h).

A thin ctypes layer over lib/libdeac_gb300.so: no torch types, no CPU
fallback.  Loading fails with an ImportError-like RuntimeError when the
library has not been built (``python deac-cpp_gb300/build.py``).

    from deac_gb300 import Batch, make_config
    b = Batch()
    run = b.add_run(make_config(temperature=1.35, spectra_type="bfull",
                                population_size=8, number_of_generations=1000),
                    tau, isf, err, frequency)
    b.run()
    res = b.result(run); out = b.fetch(run)
"""
from __future__ import annotations

import ctypes
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parents[1]
LIB_PATH = PKG / "lib" / "libdeac_gb300.so"
DEBUG_LIB_PATH = PKG / "lib" / "libdeac_gb300_debug.so"
EXE_PATH = PKG / "bin" / "deac.e"

MODEL = {"standard": 0, "hyperbolic": 1, "normalization": 2}
SPECTRA = {"spbsf": 0, "spfsf": 1, "bfull": 2, "ffull": 3, "bdsf": 4}
ENGINE_PLAIN_FP64 = 0
ENGINE_SPLIT_BF16 = 1
STREAMS = {"reference": 0, "counter": 1}
FIRST_MOMENT_FORMULA = {"gpu": 0, "cpu": 1}


class DeacConfig(ctypes.Structure):
    """Mirror of ``deac_config``."""

    _fields_ = [
        ("model", ctypes.c_int32),
        ("zero_temperature", ctypes.c_int32),
        ("bosonic", ctypes.c_int32),
        ("allow_negative_weight", ctypes.c_int32),
        ("spectra_type", ctypes.c_int32),
        ("normalize", ctypes.c_int32),
        ("use_negative_first_moment", ctypes.c_int32),
        ("track_stats", ctypes.c_int32),
        ("temperature", ctypes.c_double),
        ("first_moment", ctypes.c_double),
        ("third_moment", ctypes.c_double),
        ("third_moment_error", ctypes.c_double),
        ("crossover_probability", ctypes.c_double),
        ("self_adapting_crossover_probability", ctypes.c_double),
        ("differential_weight", ctypes.c_double),
        ("self_adapting_differential_weight_probability", ctypes.c_double),
        ("self_adapting_differential_weight_shift", ctypes.c_double),
        ("self_adapting_differential_weight", ctypes.c_double),
        ("stop_minimum_fitness", ctypes.c_double),
        ("number_of_generations", ctypes.c_uint64),
        ("population_size", ctypes.c_uint64),
        ("seed", ctypes.c_uint64),
        ("first_moment_formula", ctypes.c_int32),
    ]


class TuneReport(ctypes.Structure):
    """Mirror of ``deac_tune_report``."""

    _fields_ = [
        ("parts_per_cta", ctypes.c_uint32),
        ("split_waves", ctypes.c_uint32),
        ("candidates", ctypes.c_uint32),
        ("from_cache", ctypes.c_uint32),
        ("ms_per_generation", ctypes.c_double),
        ("ms_per_generation_default", ctypes.c_double),
    ]


class RunResult(ctypes.Structure):
    """Mirror of ``deac_run_result``."""

    _fields_ = [
        ("generation", ctypes.c_uint64),
        ("minimum_fitness", ctypes.c_double),
        ("best_index", ctypes.c_uint64),
        ("spectrum_length", ctypes.c_uint64),
        ("stats_length", ctypes.c_uint64),
        ("population_size", ctypes.c_uint64),
        ("genome_size", ctypes.c_uint64),
        ("number_of_timeslices", ctypes.c_uint64),
        ("sides", ctypes.c_int32),
        ("finished", ctypes.c_int32),
    ]


def make_config(**kw) -> DeacConfig:
    """The reference command-line defaults (deac.cpp:1927-2024) overridden by
    keyword arguments; ``model`` and ``spectra_type`` accept names."""
    c = DeacConfig()
    c.model = 0
    c.spectra_type = SPECTRA["spfsf"]
    c.temperature = 0.0
    c.first_moment = -1.0
    c.third_moment = -1.0
    c.third_moment_error = 0.0
    c.crossover_probability = 0.9
    c.self_adapting_crossover_probability = 0.1
    c.differential_weight = 0.9
    c.self_adapting_differential_weight_probability = 0.1
    c.self_adapting_differential_weight_shift = 0.1
    c.self_adapting_differential_weight = 0.9
    c.stop_minimum_fitness = 1.0
    c.number_of_generations = 100000
    c.population_size = 512
    c.seed = 0
    for k, v in kw.items():
        if k == "model" and isinstance(v, str):
            v = MODEL[v]
        if k == "spectra_type" and isinstance(v, str):
            v = SPECTRA[v]
        if k == "first_moment_formula" and isinstance(v, str):
            v = FIRST_MOMENT_FORMULA[v]
        if isinstance(v, bool):
            v = int(v)
        if not hasattr(c, k):
            raise AttributeError(f"deac_config has no field {k!r}")
        setattr(c, k, v)
    if kw.get("bosonic") and "spectra_type" not in kw:
        c.spectra_type = SPECTRA["bdsf"]
    return c


_dp = ctypes.POINTER(ctypes.c_double)
_lib = None

# C-ABI symbols and their signatures (include/deac_gb300.h)
SIGNATURES = {
    "deac_config_default": (None, [ctypes.POINTER(DeacConfig)]),
    "deac_config_check": (ctypes.c_int, [ctypes.POINTER(DeacConfig)]),
    "deac_last_error": (ctypes.c_char_p, []),
    "deac_version": (ctypes.c_char_p, []),
    "deac_batch_create": (ctypes.c_int, [ctypes.c_int, ctypes.c_void_p, ctypes.c_int32, ctypes.POINTER(ctypes.c_void_p)]),
    "deac_batch_add_run": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(DeacConfig), _dp, _dp, _dp, ctypes.c_uint64,
                                          _dp, ctypes.c_uint64, ctypes.POINTER(ctypes.c_uint32)]),
    "deac_batch_setup": (ctypes.c_int, [ctypes.c_void_p]),
    "deac_batch_launch": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint64]),
    "deac_batch_sync": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint32)]),
    "deac_batch_run": (ctypes.c_int, [ctypes.c_void_p]),
    "deac_batch_size": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint32)]),
    "deac_batch_result": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint32, ctypes.POINTER(RunResult)]),
    "deac_batch_fetch": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint32, _dp, _dp, _dp, _dp, _dp]),
    "deac_batch_fetch_all": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(RunResult), _dp, _dp]),
    "deac_batch_spectra_length": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint64)]),
    "deac_batch_fetch_state": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint32, _dp, _dp, _dp, _dp]),
    "deac_batch_checkpoint": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_uint64,
                                             ctypes.POINTER(ctypes.c_uint64)]),
    "deac_batch_restore": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_uint64]),
    "deac_batch_set_streams": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32]),
    "deac_batch_enable_trace": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint64]),
    "deac_batch_fetch_trace": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint32, _dp, ctypes.c_uint64]),
    "deac_batch_enable_timing": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32]),
    "deac_batch_autotune": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint64, ctypes.POINTER(TuneReport)]),
    "deac_batch_generation_launches": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint32)]),
    "deac_batch_transfer_bytes": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint64),
                                                 ctypes.POINTER(ctypes.c_uint64)]),
    "deac_batch_split_counts": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint32, ctypes.POINTER(ctypes.c_uint64)]),
    "deac_batch_kernel_time": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, _dp, ctypes.POINTER(ctypes.c_uint64)]),
    "deac_batch_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "deac_reconstruct": (ctypes.c_int, [ctypes.POINTER(DeacConfig), _dp, _dp, _dp, ctypes.c_uint64, _dp,
                                        ctypes.c_uint64, ctypes.POINTER(RunResult), _dp, _dp, _dp, _dp, _dp]),
    "deac_population_fitness_noalloc": (ctypes.c_int, [ctypes.c_int, ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p,
                                                       ctypes.c_uint64, ctypes.c_uint64, ctypes.c_void_p,
                                                       ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                                       ctypes.c_uint64, ctypes.c_void_p]),
}


def load_library(path: Path = LIB_PATH):
    """Load the C-ABI library (once).  Raises RuntimeError if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not Path(path).exists():
        raise RuntimeError(f"{path} is not built; run `python deac-cpp_gb300/build.py` "
                           "(the DEAC engine has no CPU fallback)")
    lib = ctypes.CDLL(str(path))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def load_debug_library(path: Path = DEBUG_LIB_PATH):
    """The test aids' library (include/deac_gb300_debug.h); not the engine."""
    if not Path(path).exists():
        raise RuntimeError(f"{path} is not built; run `python deac-cpp_gb300/build.py`")
    lib = ctypes.CDLL(str(path))
    lib.deac_debug_last_error.restype = ctypes.c_char_p
    lib.deac_debug_last_error.argtypes = []
    return lib


class DeacError(RuntimeError):
    pass


def _check(rc: int):
    if rc != 0:
        raise DeacError(f"deac error {rc}: {load_library().deac_last_error().decode()}")


def _as_f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _ptr(a):
    return None if a is None else a.ctypes.data_as(_dp)


class Batch:
    """A batch of independent DEAC runs on one GPU (deac_batch_*)."""

    def __init__(self, device: int = 0, stream: int | None = None, engine: int = ENGINE_PLAIN_FP64,
                 streams: str = "reference"):
        """``streams``: "reference" (the reference's per-gene PRNG table, its
        draws bit for bit) or "counter" (the compact counter-stream layout of
        the batched forms, deac_batch_set_streams)."""
        lib = load_library()
        h = ctypes.c_void_p()
        _check(lib.deac_batch_create(device, ctypes.c_void_p(stream or 0), engine, ctypes.byref(h)))
        self._h = h
        self._lib = lib
        self._runs = []
        if streams != "reference":
            _check(lib.deac_batch_set_streams(h, STREAMS[streams]))

    def close(self):
        if self._h:
            self._lib.deac_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def add_run(self, cfg: DeacConfig, tau, isf, err, frequency) -> int:
        tau, isf, err, frequency = (_as_f64(x) for x in (tau, isf, err, frequency))
        idx = ctypes.c_uint32()
        _check(self._lib.deac_batch_add_run(self._h, ctypes.byref(cfg), _ptr(tau), _ptr(isf), _ptr(err), len(tau),
                                            _ptr(frequency), len(frequency), ctypes.byref(idx)))
        self._runs.append((DeacConfig.from_buffer_copy(cfg), len(tau), len(frequency)))
        return idx.value

    def enable_trace(self, run: int, generations: int):
        _check(self._lib.deac_batch_enable_trace(self._h, run, generations))

    def setup(self):
        _check(self._lib.deac_batch_setup(self._h))

    def launch(self, generations: int):
        _check(self._lib.deac_batch_launch(self._h, generations))

    def sync(self) -> int:
        n = ctypes.c_uint32()
        _check(self._lib.deac_batch_sync(self._h, ctypes.byref(n)))
        return n.value

    def run(self):
        _check(self._lib.deac_batch_run(self._h))

    def enable_timing(self, on: bool = True):
        _check(self._lib.deac_batch_enable_timing(self._h, int(on)))

    def kernel_time(self, kind: int):
        ms = ctypes.c_double()
        n = ctypes.c_uint64()
        _check(self._lib.deac_batch_kernel_time(self._h, kind, ctypes.byref(ms), ctypes.byref(n)))
        return ms.value, n.value

    def autotune(self, generations: int = 16) -> dict:
        """Choose the split engine's launch shapes (deac_batch_autotune)."""
        r = TuneReport()
        _check(self._lib.deac_batch_autotune(self._h, generations, ctypes.byref(r)))
        return {k: getattr(r, k) for k, _ in TuneReport._fields_}

    def generation_launches(self) -> int:
        """Kernel launches per generation of this batch (after setup)."""
        n = ctypes.c_uint32()
        _check(self._lib.deac_batch_generation_launches(self._h, ctypes.byref(n)))
        return n.value

    def transfer_bytes(self):
        """(host -> device, device -> host) bytes this batch has copied."""
        a, b = ctypes.c_uint64(), ctypes.c_uint64()
        _check(self._lib.deac_batch_transfer_bytes(self._h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def split_counts(self, run: int) -> dict:
        c = (ctypes.c_uint64 * 3)()
        _check(self._lib.deac_batch_split_counts(self._h, run, c))
        return {"equal_to_parent": c[0], "interval": c[1], "exact": c[2]}

    def result(self, run: int) -> dict:
        r = RunResult()
        _check(self._lib.deac_batch_result(self._h, run, ctypes.byref(r)))
        return {k: getattr(r, k) for k, _ in RunResult._fields_}

    def fetch(self, run: int) -> dict:
        res = self.result(run)
        cfg = self._runs[run][0]
        spec = np.zeros(res["spectrum_length"])
        freq = np.zeros(res["spectrum_length"])
        st = [np.zeros(res["stats_length"]) for _ in range(3)] if cfg.track_stats else [None] * 3
        _check(self._lib.deac_batch_fetch(self._h, run, _ptr(spec), _ptr(freq), _ptr(st[0]), _ptr(st[1]),
                                          _ptr(st[2])))
        out = dict(res, dsf=spec, frequency=freq)
        if cfg.track_stats:
            out["stats_mean"], out["stats_minimum"], out["stats_squared_mean"] = st
        return out

    def fetch_all(self) -> list:
        """Every run's summary and best spectrum (as fetch, without the
        statistics arrays), in one call: the spectra are formed on host
        threads into one array, each run's dsf and frequency a view of it."""
        n = len(self._runs)
        total = ctypes.c_uint64(0)
        _check(self._lib.deac_batch_spectra_length(self._h, ctypes.byref(total)))
        res = (RunResult * n)()
        spec = np.empty(total.value)
        freq = np.empty(total.value)
        _check(self._lib.deac_batch_fetch_all(self._h, res, _ptr(spec), _ptr(freq)))
        out, o = [], 0
        for r in range(n):
            d = {k: getattr(res[r], k) for k, _ in RunResult._fields_}
            L = d["spectrum_length"]
            d["dsf"], d["frequency"] = spec[o:o + L], freq[o:o + L]
            o += L
            out.append(d)
        return out

    def fetch_state(self, run: int) -> dict:
        cfg, nt, m = self._runs[run]
        p = cfg.population_size
        s = 1 if cfg.bosonic else 2
        pop = np.zeros(s * p * m)
        fit = np.zeros(p)
        cr = np.zeros(s * p)
        fw = np.zeros(s * p)
        _check(self._lib.deac_batch_fetch_state(self._h, run, _ptr(pop), _ptr(fit), _ptr(cr), _ptr(fw)))
        return {"population": pop.reshape(s, p, m), "fitness": fit, "crossover": cr.reshape(s, p),
                "weights": fw.reshape(s, p)}

    def checkpoint(self, run: int) -> bytes:
        """The run's state as one byte block (plain engine, after setup)."""
        n = ctypes.c_uint64(0)
        _check(self._lib.deac_batch_checkpoint(self._h, run, None, 0, ctypes.byref(n)))
        buf = ctypes.create_string_buffer(n.value)
        _check(self._lib.deac_batch_checkpoint(self._h, run, buf, n.value, ctypes.byref(n)))
        return buf.raw

    def restore(self, run: int, block: bytes):
        """Continue run ``run`` from a checkpoint (after setup)."""
        _check(self._lib.deac_batch_restore(self._h, run, block, len(block)))

    def fetch_trace(self, run: int, generations: int) -> np.ndarray:
        cfg = self._runs[run][0]
        buf = np.full(generations * cfg.population_size, np.nan)
        _check(self._lib.deac_batch_fetch_trace(self._h, run, _ptr(buf), generations))
        return buf.reshape(generations, cfg.population_size)


def reconstruct(cfg: DeacConfig, tau, isf, err, frequency) -> dict:
    """One reconstruction through ``deac_reconstruct`` (the deac() drop-in)."""
    lib = load_library()
    tau, isf, err, frequency = (_as_f64(x) for x in (tau, isf, err, frequency))
    m = len(frequency)
    s = 1 if cfg.bosonic else 2
    spec_len = 2 * m - 1 if s == 2 else m
    n = cfg.number_of_generations
    r = RunResult()
    dsf = np.zeros(spec_len)
    fr = np.zeros(spec_len)
    st = [np.zeros(n) for _ in range(3)] if cfg.track_stats else [None] * 3
    _check(lib.deac_reconstruct(ctypes.byref(cfg), _ptr(tau), _ptr(isf), _ptr(err), len(tau), _ptr(frequency), m,
                                ctypes.byref(r), _ptr(dsf), _ptr(fr), _ptr(st[0]), _ptr(st[1]), _ptr(st[2])))
    out = {k: getattr(r, k) for k, _ in RunResult._fields_}
    out.update(dsf=dsf, frequency=fr)
    if cfg.track_stats:
        k = r.stats_length
        out["stats_mean"], out["stats_minimum"], out["stats_squared_mean"] = (a[:k] for a in st)
    return out
