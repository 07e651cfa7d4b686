"""GPU engine vs CPU oracle (reference CUDA-path semantics), bit for bit.

Every case runs the plain FP64 engine through the C-ABI and the oracle in
GPU order on the same seeded inputs, then requires identical generation
counts, minimum fitness, best spectrum, final population and fitness, the
trial fitness of every member at every generation (which pins every
selection decision), and the three stats arrays.
"""
import numpy as np
import pytest

from deac_testlib import GPU_ORDER, config0_data, make_isf, uniform_grid

pytestmark = pytest.mark.gpu


def _data(kind, seed=1):
    if kind == "cfg0":
        return config0_data(seed)
    if kind == "cfg0-neg":
        tau, isf, err = config0_data(seed)
        return tau, -isf, err
    if kind == "odd":  # N_tau not a power of two, T=0.5
        return make_isf(50, 0.5, [(0.6, 3.0, 1.0), (0.4, 9.0, 2.0)], 1e-3, seed)
    raise KeyError(kind)


CASES = {
    # name: (data, M, omega_max, N, config overrides)
    "standard-bfull": ("cfg0", 64, 64.0, 600, dict(spectra_type="bfull")),
    "standard-normalize": ("cfg0", 64, 64.0, 600, dict(spectra_type="bfull", normalize=True)),
    "hyperbolic-bfull": ("cfg0", 64, 64.0, 400, dict(model="hyperbolic", spectra_type="bfull")),
    "normalization-bfull-normalize": ("cfg0", 64, 64.0, 400,
                                      dict(model="normalization", spectra_type="bfull", normalize=True)),
    "standard-spfsf": ("cfg0-neg", 64, 64.0, 400, dict(spectra_type="spfsf")),
    "hyperbolic-spbsf": ("cfg0-neg", 64, 64.0, 400, dict(model="hyperbolic", spectra_type="spbsf")),
    "standard-ffull-moments": ("cfg0", 64, 64.0, 400,
                               dict(spectra_type="ffull", first_moment=2.0, third_moment=50.0,
                                    third_moment_error=2.0)),
    "bosonic-standard-negfirst": ("cfg0", 64, 64.0, 400, dict(bosonic=True, use_negative_first_moment=True)),
    # the reference CPU build's first-moment term, (m_i - m)^2 / m (deac.cpp:969)
    "first-moment-cpu-formula": ("cfg0", 64, 64.0, 400, dict(spectra_type="bfull", first_moment=2.0,
                                                             first_moment_formula="cpu")),
    "first-moment-cpu-formula-bosonic-normalize": ("cfg0", 64, 64.0, 400,
                                                   dict(bosonic=True, normalize=True, first_moment=1.5,
                                                        third_moment=40.0, third_moment_error=3.0,
                                                        first_moment_formula="cpu")),
    "bosonic-hyperbolic-normalize": ("cfg0", 64, 64.0, 400, dict(bosonic=True, model="hyperbolic", normalize=True)),
    "bosonic-normalization": ("cfg0", 64, 64.0, 400, dict(bosonic=True, model="normalization")),
    "zero-temperature": ("cfg0", 64, 64.0, 400, dict(bosonic=True, zero_temperature=True)),
    "signed-weights": ("cfg0", 64, 64.0, 400, dict(spectra_type="bfull", allow_negative_weight=True)),
    "odd-sizes": ("odd", 37, 20.0, 400, dict(spectra_type="bfull", population_size=13, normalize=True,
                                             first_moment=1.0)),
    "stop-immediately": ("cfg0", 64, 64.0, 100, dict(spectra_type="bfull", stop_minimum_fitness=1e300)),
    "two-generations": ("cfg0", 64, 64.0, 2, dict(spectra_type="bfull")),
    "early-stop": ("cfg0", 64, 64.0, 5000, dict(spectra_type="bfull", stop_minimum_fitness=5e4)),
}


def _compare(eng, ref, trace_eng, n_trace):
    assert eng["generation"] == ref["generation"]
    assert eng["minimum_fitness"] == ref["minimum_fitness"]
    n = ref["trace"].shape[0] if n_trace else 0
    if n:
        t = trace_eng[:n]
        bad = np.nonzero(~np.all(t == ref["trace"], axis=1))[0]
        assert bad.size == 0, (
            f"trial fitness differs first at generation {bad[0]}: "
            f"engine {t[bad[0]]} oracle {ref['trace'][bad[0]]}")
    assert np.array_equal(eng["frequency"].view(np.uint64), ref["frequency"].view(np.uint64))
    assert np.array_equal(eng["dsf"], ref["dsf"])
    for k in ("stats_mean", "stats_minimum", "stats_squared_mean"):
        if k in ref:
            assert np.array_equal(eng[k], ref[k]), k


@pytest.mark.parametrize("name", sorted(CASES))
def test_engine_matches_oracle(name, engine, oracle):
    kind, m, omax, n, over = CASES[name]
    kw = dict(temperature=1.35 if kind != "odd" else 0.5, population_size=8, number_of_generations=n, seed=3,
              track_stats=True, stop_minimum_fitness=1.0)
    kw.update(over)
    cfg = engine.make_config(**kw)
    tau, isf, err = _data(kind)
    freq = uniform_grid(m, omax)
    ref = oracle.run(cfg, tau, isf, err, freq, order=GPU_ORDER, trace=n, state=True)
    with engine.Batch() as b:
        run = b.add_run(cfg, tau, isf, err, freq)
        b.enable_trace(run, n)
        b.run()
        eng = b.fetch(run)
        state = b.fetch_state(run)
        trace = b.fetch_trace(run, n)
    _compare(eng, ref, trace, n)
    assert np.array_equal(state["population"], ref["population"])
    assert np.array_equal(state["fitness"], ref["fitness"])


def test_batched_ragged_runs_match_oracle(engine, oracle):
    """Runs of different sizes, models and seeds in one batch: each must
    equal its own single-run oracle."""
    specs = [
        (dict(spectra_type="bfull", population_size=8, seed=1), "cfg0", 64, 64.0),
        (dict(spectra_type="bfull", population_size=16, seed=2, normalize=True), "cfg0", 48, 40.0),
        (dict(model="hyperbolic", spectra_type="bfull", population_size=5, seed=3), "odd", 33, 20.0),
        (dict(bosonic=True, population_size=12, seed=4), "cfg0", 80, 64.0),
        (dict(spectra_type="bfull", population_size=8, seed=5, stop_minimum_fitness=1e9), "cfg0", 64, 64.0),
    ]
    n = 300
    runs = []
    with engine.Batch() as b:
        for over, kind, m, omax in specs:
            kw = dict(temperature=1.35 if kind != "odd" else 0.5, number_of_generations=n, track_stats=True)
            kw.update(over)
            cfg = engine.make_config(**kw)
            tau, isf, err = _data(kind)
            freq = uniform_grid(m, omax)
            r = b.add_run(cfg, tau, isf, err, freq)
            b.enable_trace(r, n)
            runs.append((r, cfg, tau, isf, err, freq))
        b.run()
        for r, cfg, tau, isf, err, freq in runs:
            ref = oracle.run(cfg, tau, isf, err, freq, order=GPU_ORDER, trace=n)
            _compare(b.fetch(r), ref, b.fetch_trace(r, n), n)


def test_reconstruct_one_call(engine, oracle):
    """deac_reconstruct (the one-call deac() drop-in) equals the oracle."""
    cfg = engine.make_config(temperature=1.35, spectra_type="bfull", population_size=8,
                             number_of_generations=300, seed=9, track_stats=True)
    tau, isf, err = config0_data(2)
    freq = uniform_grid(64, 64.0)
    got = engine.reconstruct(cfg, tau, isf, err, freq)
    ref = oracle.run(cfg, tau, isf, err, freq, order=GPU_ORDER)
    assert got["generation"] == ref["generation"]
    assert np.array_equal(got["dsf"], ref["dsf"])
    assert np.array_equal(got["stats_mean"], ref["stats_mean"])
