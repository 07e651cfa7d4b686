"""Counter streams (DEAC_STREAMS_COUNTER): the batched forms' compact draw
layout, which replaces the reference's per-gene xoshiro256+ state table
(deac.cpp:1114-1135, 2 S P (M+1) states of 32 bytes) by SplitMix64 outputs at
positions computed from (generation, member, side, gene).

CPU: the oracle's draws are the SplitMix64 sequence of the reference's own
seeding generator (rng.hpp:10-15) at the stated positions, and the draws are
uniform and independent enough for the roles they play (crossover tests at a
rate CR, uniform mutant indices).  GPU: the plain engine with counter streams
equals the oracle's GPU order with counter streams bit for bit (trial fitness
of every member at every generation, final population, spectrum), and the
split engine equals the plain engine on the same runs."""
import numpy as np
import pytest

from deac_testlib import GPU_ORDER_COUNTER, config0_data, config1_data, make_isf, uniform_grid

GAMMA = 0x9E3779B97F4A7C15
MASK = (1 << 64) - 1


def _splitmix_sequence(state, n):
    """The reference's seeding generator, step by step."""
    out = []
    for _ in range(n):
        state = (state + GAMMA) & MASK
        z = state
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & MASK
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & MASK
        out.append(z ^ (z >> 31))
    return out


def test_stream_draws_are_the_splitmix_sequence(oracle):
    for key in (0, 1, 1407513601, 0xDEADBEEFCAFEF00D, MASK):
        seq = _splitmix_sequence(key, 40)
        assert [oracle.stream_draw(key, k) for k in range(40)] == seq
    # random access far into the stream: position n is key + (n+1) gamma mixed
    key, pos = 12345, (1 << 40) + 17
    assert oracle.stream_draw(key, pos) == _splitmix_sequence((key + pos * GAMMA) & MASK, 1)[0]


def test_stream_keys_follow_the_population_seed(oracle):
    seed = 1407513600 + 7
    seq = _splitmix_sequence(seed, 4)
    assert oracle.stream_keys(seed) == (seq[2], seq[3])


def test_crossover_draws_are_uniform_and_independent(oracle):
    """20,000 consecutive crossover positions of one generation: the mean of
    the uniforms, a 16-bin chi-square, the pass rate of a CR = 0.9 test and
    the lag-1 correlation lie within their 5-sigma bands."""
    kx, _ = oracle.stream_keys(1407513600 + 3)
    n = 20000
    u = np.array([(oracle.stream_draw(kx, 5 * n + k) >> 11) * 2.0 ** -53 for k in range(n)])
    assert abs(u.mean() - 0.5) < 5 * np.sqrt(1 / 12 / n)
    counts = np.histogram(u, bins=16, range=(0.0, 1.0))[0]
    chi2 = ((counts - n / 16) ** 2 / (n / 16)).sum()
    assert chi2 < 15 + 5 * np.sqrt(30)
    rate = (u < 0.9).mean()
    assert abs(rate - 0.9) < 5 * np.sqrt(0.09 / n)
    assert abs(np.corrcoef(u[:-1], u[1:])[0, 1]) < 5 / np.sqrt(n)


def test_mutant_draws_are_uniform(oracle):
    """The mutant-index draws (position 8 on of each member's jDE span) of
    P = 8: x % P is uniform over the members."""
    _, kj = oracle.stream_keys(1407513600 + 5)
    n = 8000
    r = np.array([oracle.stream_draw(kj, (1 << 16) * k + 8) % 8 for k in range(n)])
    counts = np.bincount(r, minlength=8)
    chi2 = ((counts - n / 8) ** 2 / (n / 8)).sum()
    assert chi2 < 7 + 5 * np.sqrt(14)


# ---------------------------------------------------------------------- GPU

CASES = {
    # name: (data, M, omega_max, generations, overrides)
    "standard-normalize": ("cfg0", 64, 64.0, 400, dict(spectra_type="bfull", normalize=True)),
    "hyperbolic": ("cfg0", 96, 64.0, 300, dict(model="hyperbolic", spectra_type="bfull")),
    "bosonic": ("cfg0", 64, 64.0, 300, dict(bosonic=True)),
    "signed-weights": ("cfg0", 64, 64.0, 300, dict(spectra_type="bfull", allow_negative_weight=True)),
    "odd-population": ("odd", 64, 20.0, 300, dict(spectra_type="bfull", population_size=13, temperature=0.5)),
    "moments": ("cfg0", 48, 64.0, 300, dict(spectra_type="ffull", first_moment=2.0, third_moment=50.0,
                                           third_moment_error=2.0)),
    "cfg1-shape": ("cfg1", 4096, 512.0, 80, dict(spectra_type="bfull", normalize=True)),
    "stop": ("cfg0", 64, 64.0, 20000, dict(spectra_type="bfull", stop_minimum_fitness=5e4)),
}


def _data(kind, seed=2):
    if kind == "cfg0":
        return config0_data(seed)
    if kind == "cfg1":
        return config1_data(seed)
    return make_isf(50, 0.5, [(0.6, 3.0, 1.0), (0.4, 9.0, 2.0)], 1e-3, seed)


def _run(engine, kind, cfg, data, freq, n, trace):
    with engine.Batch(engine=kind, streams="counter") as b:
        r = b.add_run(cfg, *data, freq)
        if trace:
            b.enable_trace(r, n)
        b.run()
        out = b.fetch(r)
        out.update(b.fetch_state(r))
        if trace:
            out["trace"] = b.fetch_trace(r, n)
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(CASES))
def test_counter_streams_plain_matches_oracle_and_split_matches_plain(engine, oracle, name):
    kind, m, omax, n, over = CASES[name]
    kw = dict(temperature=1.35, population_size=8, number_of_generations=n, seed=13, stop_minimum_fitness=1.0,
              track_stats=True)
    kw.update(over)
    cfg = engine.make_config(**kw)
    data = _data(kind)
    freq = uniform_grid(m, omax)
    ref = oracle.run(cfg, *data, freq, order=GPU_ORDER_COUNTER, trace=min(n, 2000), state=True)
    plain = _run(engine, engine.ENGINE_PLAIN_FP64, cfg, data, freq, min(n, 2000), True)
    assert plain["generation"] == ref["generation"]
    assert plain["minimum_fitness"] == ref["minimum_fitness"]
    rows = ref["trace"].shape[0]
    bad = np.nonzero(~np.all(plain["trace"][:rows] == ref["trace"], axis=1))[0]
    assert bad.size == 0, f"trial fitness differs first at generation {bad[0]}"
    assert np.array_equal(plain["dsf"], ref["dsf"])
    assert np.array_equal(plain["population"], ref["population"])
    assert np.array_equal(plain["fitness"], ref["fitness"])
    for k in ("stats_mean", "stats_minimum", "stats_squared_mean"):
        assert np.array_equal(plain[k], ref[k]), k
    if m % 32:
        return  # the split engine needs M a multiple of 32
    split = _run(engine, engine.ENGINE_SPLIT_BF16, cfg, data, freq, n, False)
    for k in ("generation", "minimum_fitness", "best_index"):
        assert split[k] == plain[k], k
    for k in ("dsf", "population", "fitness", "crossover", "weights"):
        assert np.array_equal(split[k], plain[k]), k


@pytest.mark.gpu
def test_counter_streams_ragged_batch(engine, oracle):
    """A ragged batch (models, sides, sizes, stops) on counter streams: every
    run equals its own oracle run, in the plain and the split engine.  In the
    split engine the runs of at most 64 members take the slice path (items of
    64/P chunks: P = 13 on M = 96 is one short item of three chunks, P = 5 on
    M = 416 is two items, the second short) and the run of 100 members the
    per-member part path, in the same generations."""
    specs = []
    for k, (over, m) in enumerate([(dict(spectra_type="bfull", population_size=8), 64),
                                   (dict(model="hyperbolic", spectra_type="bfull", population_size=32), 128),
                                   (dict(bosonic=True, population_size=13), 96),
                                   (dict(model="normalization", spectra_type="bfull", population_size=64,
                                         normalize=True), 256),
                                   (dict(spectra_type="bfull", population_size=8, stop_minimum_fitness=1e5), 64),
                                   (dict(spectra_type="bfull", population_size=100), 160),
                                   (dict(bosonic=True, population_size=5, allow_negative_weight=True), 416),
                                   (dict(spectra_type="bfull", population_size=4), 32)]):
        kw = dict(temperature=1.35, number_of_generations=300, seed=40 + k, stop_minimum_fitness=1.0)
        kw.update(over)
        specs.append((engine.make_config(**kw), config0_data(40 + k), uniform_grid(m, 64.0)))
    for kind in (engine.ENGINE_PLAIN_FP64, engine.ENGINE_SPLIT_BF16):
        with engine.Batch(engine=kind, streams="counter") as b:
            ids = [b.add_run(cfg, *data, freq) for cfg, data, freq in specs]
            b.run()
            for r, (cfg, data, freq) in zip(ids, specs):
                ref = oracle.run(cfg, *data, freq, order=GPU_ORDER_COUNTER, state=True)
                got = b.fetch(r)
                got.update(b.fetch_state(r))
                assert got["generation"] == ref["generation"], (kind, r)
                assert got["minimum_fitness"] == ref["minimum_fitness"], (kind, r)
                assert np.array_equal(got["dsf"], ref["dsf"]), (kind, r)
                assert np.array_equal(got["population"], ref["population"]), (kind, r)


@pytest.mark.gpu
def test_counter_streams_rejected_when_positions_overflow(engine):
    """Positions must stay below 2^62: N P S M beyond it is refused at once
    (checked on the host, no GPU needed)."""
    lib = engine.load_library()
    import ctypes
    h = ctypes.c_void_p()
    rc = lib.deac_batch_create(0, None, engine.ENGINE_PLAIN_FP64, ctypes.byref(h))
    assert rc == 0, lib.deac_last_error().decode()
    try:
        assert lib.deac_batch_set_streams(h, 1) == 0
        cfg = engine.make_config(temperature=1.35, spectra_type="bfull", population_size=1 << 20,
                                 number_of_generations=1 << 40)
        tau, isf, err = config0_data(1)
        freq = uniform_grid(1 << 10, 64.0)
        rc = lib.deac_batch_add_run(h, ctypes.byref(cfg), *(x.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
                                                             for x in (tau, isf, err)), len(tau),
                                    freq.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), len(freq), None)
        assert rc != 0
        assert "counter streams" in lib.deac_last_error().decode()
    finally:
        lib.deac_batch_destroy(h)
