"""Split-precision engine (tcgen05 BF16 digit slices + intervals) vs the plain
FP64 engine: every selection decision must be the FP64 one, so the two
engines must produce bit-identical results -- generation count, minimum
fitness, best spectrum, final population and final fitness -- on the same
runs.  Each case also checks that the tensor-core intervals settled most
trials (the exact FP64 chains only see the undecided ones)."""
import numpy as np
import pytest

from deac_testlib import config0_data, make_isf, uniform_grid

pytestmark = pytest.mark.gpu


def _data(kind, seed=1):
    if kind == "cfg0":
        return config0_data(seed)
    if kind == "neg":
        tau, isf, err = config0_data(seed)
        return tau, -isf, err
    if kind == "odd":
        return make_isf(50, 0.5, [(0.6, 3.0, 1.0), (0.4, 9.0, 2.0)], 1e-3, seed)
    if kind == "high":  # peaks up to omega = 700, sigma = 1e-5 F: F(tau) ~ 1e-100 mid-range
        return make_isf(64, 1.35, [(0.5, 700.0, 30.0), (0.3, 300.0, 20.0), (0.2, 40.0, 5.0)], 1e-5, seed,
                        omega_max_data=1500.0)
    if kind == "only-high":  # all weight above omega = 400: F(mid tau) ~ 1e-80, residuals ~ 1e84 sigma
        return make_isf(64, 1.35, [(0.6, 700.0, 30.0), (0.4, 500.0, 20.0)], 1e-5, seed, omega_max_data=1500.0)
    if kind == "tight":  # sigma = 1e-5 F, three peaks
        return make_isf(96, 1.35, [(0.5, 3.0, 0.5), (0.3, 40.0, 5.0), (0.2, 200.0, 30.0)], 1e-5, seed,
                        omega_max_data=512.0)
    raise KeyError(kind)


CASES = {
    # name: (data kind, M, omega_max, N, overrides)
    "standard-bfull": ("cfg0", 64, 64.0, 1500, dict(spectra_type="bfull")),
    "normalize": ("cfg0", 64, 64.0, 800, dict(spectra_type="bfull", normalize=True)),
    "hyperbolic": ("cfg0", 96, 64.0, 800, dict(model="hyperbolic", spectra_type="bfull")),
    "fermionic-negative-K": ("neg", 64, 64.0, 800, dict(spectra_type="spfsf")),
    "bosonic": ("cfg0", 64, 64.0, 800, dict(bosonic=True)),
    "zero-temperature": ("cfg0", 64, 64.0, 800, dict(bosonic=True, zero_temperature=True)),
    "signed-weights": ("cfg0", 64, 64.0, 800, dict(spectra_type="bfull", allow_negative_weight=True)),
    "odd-population-and-timeslices": ("odd", 64, 20.0, 800, dict(spectra_type="bfull", population_size=13)),
    "track-stats": ("cfg0", 64, 64.0, 500, dict(spectra_type="bfull", track_stats=True)),
    "wide-genome-tight-errors": ("tight", 512, 512.0, 300, dict(spectra_type="bfull", population_size=64)),
    # K = e^{-tau omega} over [0, 1024]: model ISF and sigma hundreds of
    # binades below the float range in mid-tau (accumulators in scaled
    # units, 1/sigma carried as a float times a power of two)
    "high-frequencies-tiny-sigma": ("high", 1024, 1024.0, 300, dict(spectra_type="bfull", population_size=16)),
    "only-high-frequencies": ("only-high", 1024, 1024.0, 300, dict(spectra_type="bfull", population_size=16)),
    "early-stop": ("cfg0", 64, 64.0, 20000, dict(spectra_type="bfull", stop_minimum_fitness=5e4)),
    # --normalize: the trials stay raw until the decisions, their exact
    # normalisation row sums run beside the tensor-core contraction
    "normalize-bosonic": ("cfg0", 64, 64.0, 600, dict(bosonic=True, normalize=True)),
    "normalize-hyperbolic": ("cfg0", 96, 64.0, 600, dict(model="hyperbolic", spectra_type="bfull", normalize=True)),
    "normalize-signed-weights": ("cfg0", 64, 64.0, 600, dict(spectra_type="bfull", normalize=True,
                                                          allow_negative_weight=True)),
    "normalize-two-superblocks-ragged": ("cfg0", 2080, 512.0, 150, dict(spectra_type="bfull", normalize=True)),
    "normalize-early-stop": ("cfg0", 64, 64.0, 20000, dict(spectra_type="bfull", normalize=True,
                                                         stop_minimum_fitness=5e4)),
}


def _results(engine, kind, specs):
    out = []
    with engine.Batch(engine=kind) as b:
        ids = [b.add_run(cfg, *data, freq) for cfg, data, freq in specs]
        b.run()
        for r in ids:
            res = b.fetch(r)
            res.update(b.fetch_state(r))
            if kind == engine.ENGINE_SPLIT_BF16:
                res["counts"] = b.split_counts(r)
            out.append(res)
    return out


def _same(a, b):
    assert a["generation"] == b["generation"]
    assert a["minimum_fitness"] == b["minimum_fitness"]
    assert a["best_index"] == b["best_index"]
    assert np.array_equal(a["dsf"], b["dsf"])
    assert np.array_equal(a["population"], b["population"])
    assert np.array_equal(a["fitness"], b["fitness"])
    assert np.array_equal(a["crossover"], b["crossover"])
    assert np.array_equal(a["weights"], b["weights"])
    for k in ("stats_mean", "stats_minimum", "stats_squared_mean"):
        if k in a:
            assert np.array_equal(a[k], b[k]), k


@pytest.mark.parametrize("name", sorted(CASES))
def test_split_matches_plain(name, engine):
    kind, m, omax, n, over = CASES[name]
    kw = dict(temperature=1.35 if kind != "odd" else 0.5, population_size=8, number_of_generations=n, seed=5,
              stop_minimum_fitness=1.0)
    kw.update(over)
    cfg = engine.make_config(**kw)
    spec = [(cfg, _data(kind), uniform_grid(m, omax))]
    plain = _results(engine, engine.ENGINE_PLAIN_FP64, spec)[0]
    split = _results(engine, engine.ENGINE_SPLIT_BF16, spec)[0]
    _same(plain, split)
    c = split["counts"]
    total = sum(c.values())
    assert total > 0
    # the intervals settle trials; a run whose population has converged (a
    # stagnating one) needs the FP64 chains for nearly every decision
    assert c["interval"] > 0, c
    if not name.startswith("normalize-early-stop"):
        assert c["interval"] >= c["exact"], c


def test_split_batch_shares_tiles_across_runs(engine):
    """Several runs sharing one kernel matrix are packed into the same
    128-row MMA tiles; another run has its own matrix.  Each must still match
    its plain-engine twin."""
    tau, isf, err = config0_data(1)
    freq = uniform_grid(64, 64.0)
    specs = []
    for seed, p in ((1, 40), (2, 40), (3, 64), (4, 8)):
        cfg = engine.make_config(temperature=1.35, spectra_type="bfull", population_size=p,
                                 number_of_generations=400, seed=seed)
        specs.append((cfg, config0_data(seed), freq))
    cfg = engine.make_config(temperature=0.5, spectra_type="bfull", population_size=16, number_of_generations=400,
                             seed=9)
    specs.append((cfg, make_isf(64, 0.5, [(1.0, 4.0, 1.0)], 1e-4, 9), uniform_grid(96, 30.0)))
    plain = _results(engine, engine.ENGINE_PLAIN_FP64, specs)
    split = _results(engine, engine.ENGINE_SPLIT_BF16, specs)
    for a, b in zip(plain, split):
        _same(a, b)


def test_split_ragged_batch_with_normalization(engine):
    """One batch mixing --normalize and plain runs, one- and two-sided
    genomes, genome sizes, population sizes and stop fitnesses (runs finish
    at different generations); every run must match its plain-engine twin."""
    specs = []
    for k, (bos, norm, m, p, stop) in enumerate([(False, True, 64, 8, 1.0), (True, True, 96, 13, 1.0),
                                                 (False, False, 128, 24, 1.0), (False, True, 2080, 8, 1.0),
                                                 (False, True, 64, 16, 8e4), (True, False, 64, 8, 1.0)]):
        kw = dict(temperature=1.35, population_size=p, number_of_generations=300, seed=20 + k, normalize=norm,
                  stop_minimum_fitness=stop)
        if bos:
            kw["bosonic"] = True
        else:
            kw["spectra_type"] = "bfull"
        cfg = engine.make_config(**kw)
        specs.append((cfg, config0_data(20 + k), uniform_grid(m, 64.0 if m < 1000 else 512.0)))
    plain = _results(engine, engine.ENGINE_PLAIN_FP64, specs)
    split = _results(engine, engine.ENGINE_SPLIT_BF16, specs)
    for a, b in zip(plain, split):
        _same(a, b)


def test_split_rejects_unsupported(engine):
    cfg = engine.make_config(temperature=1.35, spectra_type="bfull", population_size=8, number_of_generations=10)
    tau, isf, err = config0_data(1)
    with engine.Batch(engine=engine.ENGINE_SPLIT_BF16) as b:
        with pytest.raises(engine.DeacError, match="multiple of 32"):
            b.add_run(cfg, tau, isf, err, uniform_grid(50, 64.0))


# Moment terms (deac.cpp:605-924): the first and third moments of each trial
# come from exact row sums beside the tensor cores and enter the interval
# decision exactly; the negative first moment (from the model ISF) is decided
# by the FP64 chains.  Every case must equal the plain engine.
MOMENT_CASES = {
    "first-moment": ("cfg0", 64, 64.0, 800, dict(spectra_type="bfull", first_moment=2.0)),
    "first-moment-cpu-formula": ("cfg0", 64, 64.0, 800, dict(spectra_type="bfull", first_moment=2.0,
                                                             first_moment_formula="cpu")),
    "first-and-third-normalize": ("cfg0", 96, 64.0, 600, dict(spectra_type="ffull", normalize=True,
                                                              first_moment=1.5, third_moment=50.0,
                                                              third_moment_error=2.0)),
    "third-moment-bosonic": ("cfg0", 64, 64.0, 600, dict(bosonic=True, third_moment=40.0, third_moment_error=3.0)),
    "negative-first-moment": ("cfg0", 64, 64.0, 600, dict(bosonic=True, use_negative_first_moment=True)),
    "moments-wide-genome": ("tight", 512, 512.0, 200, dict(spectra_type="bfull", population_size=32,
                                                          first_moment=40.0, normalize=True)),
}


@pytest.mark.parametrize("name", sorted(MOMENT_CASES))
def test_split_moment_terms_match_plain(name, engine):
    kind, m, omax, n, over = MOMENT_CASES[name]
    kw = dict(temperature=1.35, population_size=8, number_of_generations=n, seed=6, stop_minimum_fitness=1.0)
    kw.update(over)
    cfg = engine.make_config(**kw)
    spec = [(cfg, _data(kind), uniform_grid(m, omax))]
    plain = _results(engine, engine.ENGINE_PLAIN_FP64, spec)[0]
    split = _results(engine, engine.ENGINE_SPLIT_BF16, spec)[0]
    _same(plain, split)
    c = split["counts"]
    if not over.get("use_negative_first_moment"):
        assert c["interval"] > 0, c


def test_fetch_all_matches_fetch(engine):
    """The batch form of the outputs (every run's summary and best spectrum
    in one call, spectra formed on host threads) equals the per-run fetch,
    on both engines, over runs of every model, one- and two-sided."""
    specs = []
    for k, kw in enumerate([dict(spectra_type="bfull"), dict(model="hyperbolic", spectra_type="bfull"),
                            dict(model="normalization", spectra_type="bfull"), dict(bosonic=True),
                            dict(model="hyperbolic", bosonic=True), dict(spectra_type="spbsf")]):
        cfg = engine.make_config(temperature=1.35, population_size=8 + 8 * (k % 3), number_of_generations=200,
                                 seed=40 + k, **kw)
        specs.append((cfg, config0_data(40 + k), uniform_grid(64 + 32 * k, 64.0)))
    for kind in (engine.ENGINE_PLAIN_FP64, engine.ENGINE_SPLIT_BF16):
        with engine.Batch(engine=kind) as b:
            ids = [b.add_run(cfg, *data, freq) for cfg, data, freq in specs]
            b.run()
            every = b.fetch_all()
            assert len(every) == len(ids)
            for r in ids:
                one = b.fetch(r)
                for key in ("generation", "minimum_fitness", "best_index", "spectrum_length", "finished"):
                    assert every[r][key] == one[key], key
                assert np.array_equal(every[r]["dsf"], one["dsf"])
                assert np.array_equal(every[r]["frequency"], one["frequency"])
