"""Pin the oracle against the reference itself.

The reference's CPU executables are compiled from the unmodified reference
sources into oracle/_ref (oracle/Makefile; only where the reference tree is
present).  The oracle in CPU order must reproduce them bit for bit -- best
spectrum, frequency axis, generation count and all three per-generation
statistics arrays (which hold the exact minimum fitness of every
generation) -- for every model, side count, spectra type and moment option.
The oracle in GPU order must agree with them at generation 0, the case the
reference's own backend-parity test compares (test/deac_parity_test.py).
"""
import tempfile

import numpy as np
import pytest

from deac_testlib import (CPU_ORDER, GPU_ORDER, cli_args, config0_data, make_config, output_prefix,
                          read_outputs, reference_exe_for, run_exe, uniform_grid, write_doubles, write_isf)

VARIANTS = {
    "standard-bfull": dict(spectra_type="bfull"),
    "standard-bfull-normalize": dict(spectra_type="bfull", normalize=True),
    "hyperbolic-bfull": dict(model="hyperbolic", spectra_type="bfull"),
    "normalization-bfull": dict(model="normalization", spectra_type="bfull", normalize=True),
    "standard-ffull": dict(spectra_type="ffull"),
    "standard-spfsf": dict(spectra_type="spfsf", negate=True),
    "standard-spbsf": dict(spectra_type="spbsf", negate=True),
    "hyperbolic-spbsf": dict(model="hyperbolic", spectra_type="spbsf", negate=True),
    "hyperbolic-spfsf": dict(model="hyperbolic", spectra_type="spfsf", negate=True),
    "normalization-spbsf": dict(model="normalization", spectra_type="spbsf", negate=True),
    "standard-moments": dict(spectra_type="bfull", first_moment=2.0, third_moment=50.0, third_moment_error=1.0),
    "bosonic-standard-negfirst": dict(bosonic=True, use_negative_first_moment=True),
    "bosonic-hyperbolic": dict(bosonic=True, model="hyperbolic"),
    "bosonic-normalization": dict(bosonic=True, model="normalization", normalize=True),
    "zero-temperature": dict(bosonic=True, zero_temperature=True),
    "signed-weights": dict(spectra_type="bfull", allow_negative_weight=True),
}


def _run_reference(cfg, tau, isf, err, m, omega_max, frequency=None):
    exe = reference_exe_for(cfg)
    if exe is None:
        pytest.skip("reference executables not built (reference sources absent)")
    with tempfile.TemporaryDirectory() as d:
        write_isf(f"{d}/isf.bin", tau, isf, err)
        ff = None
        if frequency is not None:
            ff = f"{d}/freq.bin"
            write_doubles(ff, frequency)
        r = run_exe(exe, cli_args(cfg, f"{d}/isf.bin", f"{d}/res", genome_size=m, omega_max=omega_max,
                                  frequency_file=ff, uuid="t"), d)
        assert r.returncode == 0, r.stdout
        return read_outputs(f"{d}/res", output_prefix(cfg), "t", cfg.track_stats)


@pytest.mark.parametrize("name", sorted(VARIANTS))
def test_cpu_order_bit_exact_with_reference_build(name, oracle):
    over = dict(VARIANTS[name])
    negate = over.pop("negate", False)
    cfg = make_config(temperature=1.35, population_size=8, number_of_generations=1500, seed=11,
                      track_stats=True, **over)
    tau, isf, err = config0_data(1)
    if negate:
        isf = -isf
    ref = _run_reference(cfg, tau, isf, err, 64, 64.0)
    orc = oracle.run(cfg, tau, isf, err, uniform_grid(64, 64.0), order=CPU_ORDER)
    assert orc["generation"] == ref["generation"]
    assert np.array_equal(orc["frequency"].view(np.uint64), ref["frequency"].view(np.uint64))
    assert np.array_equal(orc["dsf"], ref["dsf"])
    for k in ("stats_mean", "stats_minimum", "stats_squared_mean"):
        assert np.array_equal(orc[k], ref[k]), k
    assert f"{orc['minimum_fitness']:.6g}" == ref["minimum_fitness_text"]


def test_cpu_order_stops_like_reference(oracle):
    """A reachable stop fitness ends both at the same generation."""
    cfg = make_config(temperature=1.35, spectra_type="bfull", population_size=8, number_of_generations=20000,
                      seed=3, stop_minimum_fitness=5e4, track_stats=True)
    tau, isf, err = config0_data(1)
    ref = _run_reference(cfg, tau, isf, err, 64, 64.0)
    orc = oracle.run(cfg, tau, isf, err, uniform_grid(64, 64.0), order=CPU_ORDER)
    assert ref["generation"] < 19999
    assert orc["generation"] == ref["generation"]
    assert np.array_equal(orc["dsf"], ref["dsf"])


def test_frequency_file_grid(oracle):
    """Non-uniform --frequency_file grid (trapezoid weights, deac.cpp:351-358)."""
    freq = np.array([0.0, 0.3, 0.7, 1.5, 2.0, 3.1, 4.0, 6.5, 9.0, 14.0, 20.0, 31.0])
    cfg = make_config(temperature=1.35, spectra_type="bfull", population_size=6, number_of_generations=800,
                      seed=5, track_stats=True)
    tau, isf, err = config0_data(4)
    ref = _run_reference(cfg, tau, isf, err, None, None, frequency=freq)
    orc = oracle.run(cfg, tau, isf, err, freq, order=CPU_ORDER)
    assert orc["generation"] == ref["generation"]
    assert np.array_equal(orc["dsf"], ref["dsf"])
    assert np.array_equal(orc["stats_minimum"], ref["stats_minimum"])


def test_gpu_order_matches_reference_at_generation_zero(oracle):
    """The reference's backend-parity scenario (test/deac_parity_test.py:45-73):
    T=1, N=2, P=8, a 4-point grid, seed 17, stop 1e300 (the loop breaks
    before any mutation), 1e-9 tolerance.  The GPU-order oracle must match
    the reference CPU build there; spectrum and frequencies exactly."""
    tau = np.array([0.0, 0.2, 0.4, 0.6])
    isf = np.array([-1.0, -0.85, -0.72, -0.61])
    err = np.array([0.05, 0.05, 0.05, 0.05])
    freq = np.array([0.0, 0.7, 1.8, 3.0])
    cfg = make_config(temperature=1.0, number_of_generations=2, population_size=8, seed=17,
                      stop_minimum_fitness=1e300, track_stats=True)
    ref = _run_reference(cfg, tau, isf, err, None, None, frequency=freq)
    orc = oracle.run(cfg, tau, isf, err, freq, order=GPU_ORDER)
    # the loop breaks at ii = 0 = N-2, which the reference reports as N-1
    assert orc["generation"] == ref["generation"] == 1
    assert np.array_equal(orc["dsf"], ref["dsf"])
    assert np.array_equal(orc["frequency"].view(np.uint64), ref["frequency"].view(np.uint64))
    for k in ("stats_mean", "stats_minimum", "stats_squared_mean"):
        np.testing.assert_allclose(orc[k], ref[k], rtol=1e-9, atol=1e-9)
