"""Parity at the benchmark configurations' shapes, on the GPU.

The plain FP64 engine is compared with the GPU-order oracle bit for bit
(generation count, minimum fitness, spectrum, final population and fitness,
and the trial fitness of every member at every generation, which pins every
selection decision), and the split-precision engine with the plain engine on
the same runs, at:

* the reference's production scale (N_tau = 128 on [0, beta], M = 4096 on
  [0, 512], P = 8, --normalize) for the standard, hyperbolic and
  normalization models and the zero-temperature kernel K = e^{-tau omega}:
  several 128-gene shared-memory stages per contraction chain, 128
  timeslices in the chi^2 tree, 4096-gene normalisation chains;
* the precision-form single run (N_tau = 256, M = 16384 on [0, 512], P = 64,
  three peaks, sigma = 1e-5 F): the trial kernel's global-memory path
  (S*M beyond its shared-memory cap), 128 shared-memory stages, two
  128-timeslice tiles of the tensor-core contraction;
* a run of the batched split configuration (N_tau = 512, M = 16384 on
  [0, 1024], P = 64, sigma = 1e-5 F): four 128-timeslice tiles, K values
  down to e^{-760};
* a non-uniform frequency grid (trapezoid weights, deac.cpp:351-358).

Reference loops: deac.cpp:1137-1574 (generation), deac_gpu.cu:277-315
(contraction)."""
import numpy as np
import pytest

from deac_testlib import GPU_ORDER, config0_data, config1_data, config2_data, uniform_grid

pytestmark = pytest.mark.gpu


def _quadratic_grid(m, omega_max):
    """A sorted non-uniform grid, dense near zero: omega_max (j / (M-1))^2."""
    j = np.arange(m, dtype=np.float64)
    return omega_max * (j / (m - 1)) ** 2


CASES = {
    # name: (data, frequency grid, generations, config overrides)
    "cfg1-standard": ("cfg1", ("uniform", 4096, 512.0), 120, dict(spectra_type="bfull", normalize=True)),
    "cfg1-hyperbolic": ("cfg1", ("uniform", 4096, 512.0), 120,
                        dict(model="hyperbolic", spectra_type="bfull", normalize=True)),
    "cfg1-normalization": ("cfg1", ("uniform", 4096, 512.0), 120,
                           dict(model="normalization", spectra_type="bfull", normalize=True)),
    "cfg1-zero-temperature": ("cfg1", ("uniform", 4096, 512.0), 120,
                              dict(bosonic=True, zero_temperature=True, normalize=True)),
    "cfg2": ("cfg2", ("uniform", 16384, 512.0), 12, dict(spectra_type="bfull", population_size=64)),
    "cfg2-normalize": ("cfg2", ("uniform", 16384, 512.0), 8,
                       dict(spectra_type="bfull", population_size=64, normalize=True)),
    # the batched split configuration's runs: N_tau = 512, M = 16384 on
    # [0, 1024], P = 64, a random mixture of 1-4 peaks up to omega = 800,
    # sigma = 1e-5 F (the ISF falls by ~11 decades towards mid-tau), K down
    # to e^{-760}
    "cfg4-run": ("cfg4", ("uniform", 16384, 1024.0), 4, dict(spectra_type="bfull", population_size=64)),
    "nonuniform-grid": ("cfg0", ("quadratic", 512, 64.0), 300, dict(spectra_type="bfull", normalize=True)),
    "nonuniform-grid-bosonic": ("cfg0", ("quadratic", 256, 64.0), 300, dict(bosonic=True)),
}


def _setup(engine, name):
    kind, (grid, m, omax), n, over = CASES[name]
    kw = dict(temperature=1.35, population_size=8, number_of_generations=n, seed=5, stop_minimum_fitness=1.0,
              track_stats=True)
    kw.update(over)
    cfg = engine.make_config(**kw)
    if kind == "cfg4":
        from deac_gb300.data import config4_runs
        tau, _, runs = config4_runs(3)
        _, isf, err = runs[2]
        data = (tau, isf, err)
    else:
        data = {"cfg0": config0_data, "cfg1": config1_data, "cfg2": config2_data}[kind](5)
    freq = uniform_grid(m, omax) if grid == "uniform" else _quadratic_grid(m, omax)
    return cfg, data, freq, n


def _engine_run(engine, kind, cfg, data, freq, n):
    with engine.Batch(engine=kind) as b:
        r = b.add_run(cfg, *data, freq)
        if kind == engine.ENGINE_PLAIN_FP64:
            b.enable_trace(r, n)
        b.run()
        out = b.fetch(r)
        out.update(b.fetch_state(r))
        if kind == engine.ENGINE_PLAIN_FP64:
            out["trace"] = b.fetch_trace(r, n)
        else:
            out["counts"] = b.split_counts(r)
    return out


@pytest.mark.parametrize("name", sorted(CASES))
def test_plain_engine_matches_oracle_and_split_matches_plain(engine, oracle, name):
    cfg, data, freq, n = _setup(engine, name)
    ref = oracle.run(cfg, *data, freq, order=GPU_ORDER, trace=n, state=True)
    plain = _engine_run(engine, engine.ENGINE_PLAIN_FP64, cfg, data, freq, n)
    # plain FP64 engine == oracle, bit for bit
    assert plain["generation"] == ref["generation"]
    assert plain["minimum_fitness"] == ref["minimum_fitness"]
    rows = ref["trace"].shape[0]
    assert rows > 0
    t = plain["trace"][:rows]
    bad = np.nonzero(~np.all(t == ref["trace"], axis=1))[0]
    assert bad.size == 0, f"trial fitness differs first at generation {bad[0]}"
    assert np.array_equal(plain["frequency"].view(np.uint64), ref["frequency"].view(np.uint64))
    assert np.array_equal(plain["dsf"], ref["dsf"])
    assert np.array_equal(plain["population"], ref["population"])
    assert np.array_equal(plain["fitness"], ref["fitness"])
    for k in ("stats_mean", "stats_minimum", "stats_squared_mean"):
        assert np.array_equal(plain[k], ref[k]), k
    # split-precision engine == plain FP64 engine on the same run
    m = len(freq)
    if m % 32:
        return
    split = _engine_run(engine, engine.ENGINE_SPLIT_BF16, cfg, data, freq, n)
    for k in ("generation", "minimum_fitness", "best_index"):
        assert split[k] == plain[k], k
    for k in ("dsf", "population", "fitness", "crossover", "weights", "stats_mean", "stats_minimum",
              "stats_squared_mean"):
        assert np.array_equal(split[k], plain[k]), k
    c = split["counts"]
    decided = c["equal_to_parent"] + c["interval"] + c["exact"]
    assert decided == cfg.population_size * split["generation"]
