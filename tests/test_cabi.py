"""The C-ABI library builds, loads without a GPU, and exports every function
include/deac_gb300.h declares; host-side argument checks work on CPU."""
import ctypes
import re
import subprocess

import pytest

from deac_testlib import REPO


def _declared():
    text = (REPO / "include" / "deac_gb300.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(deac_\w+)\s*\(", text)))


def test_header_declares_the_boundary():
    names = _declared()
    for must in ("deac_batch_create", "deac_batch_add_run", "deac_batch_setup", "deac_batch_run",
                 "deac_batch_fetch", "deac_reconstruct", "deac_config_check"):
        assert must in names


def test_library_exports_every_declared_symbol(engine):
    lib = engine.load_library()
    out = subprocess.run(["nm", "-D", "--defined-only", str(engine.LIB_PATH)], capture_output=True, text=True,
                         check=True).stdout
    exported = set(re.findall(r"\s[TW]\s+(deac_\w+)$", out, flags=re.M))
    missing = [n for n in _declared() if n not in exported]
    assert not missing, missing
    for n in _declared():
        getattr(lib, n)  # resolvable through ctypes
    assert set(engine.SIGNATURES) <= exported


def test_no_cxx_symbols_leak_into_the_abi(engine):
    out = subprocess.run(["nm", "-D", "--defined-only", str(engine.LIB_PATH)], capture_output=True, text=True,
                         check=True).stdout
    for line in out.splitlines():
        if " T " in line and "deac" in line:
            assert not line.split()[-1].startswith("_Z4deac"), line


@pytest.mark.parametrize("field,value,message", [
    ("population_size", 3, "population_size must be at least 4"),
    ("number_of_generations", 1, "number_of_generations must be at least 2"),
    ("temperature", 0.0, "temperature must be positive for non-ZeroT builds"),
    ("third_moment", 1.0, "third_moment_error must be positive when third_moment is used"),
    ("spectra_type", 4, "Please choose spectra_type"),
])
def test_config_check_messages(engine, field, value, message):
    cfg = engine.make_config(temperature=1.0, population_size=8, number_of_generations=10)
    setattr(cfg, field, value)
    lib = engine.load_library()
    assert lib.deac_config_check(ctypes.byref(cfg)) == -1
    assert message in lib.deac_last_error().decode()


def test_zero_temperature_needs_one_sided_genome(engine):
    cfg = engine.make_config(zero_temperature=True, population_size=8, number_of_generations=10)
    lib = engine.load_library()
    assert lib.deac_config_check(ctypes.byref(cfg)) == -1
    cfg = engine.make_config(zero_temperature=True, bosonic=True, population_size=8, number_of_generations=10)
    assert lib.deac_config_check(ctypes.byref(cfg)) == 0


def test_defaults_match_reference_cli(engine):
    lib = engine.load_library()
    c = engine.DeacConfig()
    lib.deac_config_default(ctypes.byref(c))
    assert (c.number_of_generations, c.population_size, c.seed) == (100000, 512, 0)
    assert (c.crossover_probability, c.self_adapting_crossover_probability) == (0.9, 0.1)
    assert (c.differential_weight, c.self_adapting_differential_weight_probability) == (0.9, 0.1)
    assert (c.stop_minimum_fitness, c.first_moment, c.third_moment) == (1.0, -1.0, -1.0)
    assert c.spectra_type == engine.SPECTRA["spfsf"]


def test_test_aids_live_in_their_own_library(engine):
    """The debug hooks (include/deac_gb300_debug.h) are not linked into the
    engine's library; their own library exports them."""
    out = subprocess.run(["nm", "-D", "--defined-only", str(engine.LIB_PATH)], capture_output=True, text=True,
                         check=True).stdout
    assert "deac_debug_" not in out
    dbg = subprocess.run(["nm", "-D", "--defined-only", str(engine.DEBUG_LIB_PATH)], capture_output=True,
                         text=True, check=True).stdout
    for name in ("deac_debug_fma_chains", "deac_debug_last_error"):
        assert name in dbg
    engine.load_debug_library()
