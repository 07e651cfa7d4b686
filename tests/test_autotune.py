"""deac_batch_autotune: the split engine's launch shapes (trial parts per
CTA, contraction CTAs per wave of SMs) chosen by timing real generations of
the batch.  On counter streams the runs of at most 64 members take the
trial-slice path, which has no parts-per-CTA choice; the run of 96 members
here keeps the part path, so both shapes are tuned.  Shapes change no
result: a tuned batch ends exactly as the plain engine on the same runs and
generations; a second batch of the same mix takes the cached choice without
timing."""
import numpy as np
import pytest

from deac_testlib import config0_data, uniform_grid

pytestmark = pytest.mark.gpu


def _specs(engine):
    specs = []
    for k, (m, p) in enumerate([(1024, 8), (2048, 16), (1024, 32), (4096, 8), (1024, 96)]):
        cfg = engine.make_config(temperature=1.35, spectra_type="bfull", population_size=p,
                                 number_of_generations=400, seed=60 + k, normalize=(k % 2 == 1))
        specs.append((cfg, config0_data(60 + k), uniform_grid(m, 64.0)))
    return specs


def test_autotune_keeps_results_and_caches_the_choice(engine):
    specs = _specs(engine)
    with engine.Batch(engine=engine.ENGINE_SPLIT_BF16, streams="counter") as b:
        ids = [b.add_run(cfg, *data, freq) for cfg, data, freq in specs]
        b.setup()
        rep = b.autotune(16)
        assert rep["candidates"] == 12 and rep["from_cache"] == 0
        assert rep["parts_per_cta"] in (1, 2, 4, 8) and rep["split_waves"] in (1, 2, 4)
        assert 0 < rep["ms_per_generation"] <= rep["ms_per_generation_default"]
        b.launch(40)  # 12 x 16 + 40 generations in all
        b.sync()
        split = [b.fetch(r) for r in ids]
    with engine.Batch(engine=engine.ENGINE_PLAIN_FP64, streams="counter") as b:
        ids = [b.add_run(cfg, *data, freq) for cfg, data, freq in specs]
        b.setup()
        b.launch(12 * 16 + 40)
        b.sync()
        plain = [b.fetch(r) for r in ids]
    for x, y in zip(split, plain):
        assert x["generation"] == y["generation"]
        assert x["minimum_fitness"] == y["minimum_fitness"]
        assert np.array_equal(x["dsf"], y["dsf"])
    with engine.Batch(engine=engine.ENGINE_SPLIT_BF16, streams="counter") as b:
        for cfg, data, freq in specs:
            b.add_run(cfg, *data, freq)
        b.setup()
        again = b.autotune(16)
        assert again["from_cache"] == 1 and again["candidates"] == 0
        assert (again["parts_per_cta"], again["split_waves"]) == (rep["parts_per_cta"], rep["split_waves"])


def test_autotune_sliced_batch_tunes_the_contraction_only(engine):
    """Every run on the slice path: only the contraction's CTAs per wave are
    timed, and the tuned batch still ends as the plain engine."""
    specs = _specs(engine)[:4]
    with engine.Batch(engine=engine.ENGINE_SPLIT_BF16, streams="counter") as b:
        ids = [b.add_run(cfg, *data, freq) for cfg, data, freq in specs]
        b.setup()
        rep = b.autotune(8)
        assert rep["candidates"] == 3 and rep["split_waves"] in (1, 2, 4)
        b.launch(10)  # 3 x 8 + 10 generations in all
        b.sync()
        split = [b.fetch(r) for r in ids]
    with engine.Batch(engine=engine.ENGINE_PLAIN_FP64, streams="counter") as b:
        ids = [b.add_run(cfg, *data, freq) for cfg, data, freq in specs]
        b.setup()
        b.launch(3 * 8 + 10)
        b.sync()
        plain = [b.fetch(r) for r in ids]
    for x, y in zip(split, plain):
        assert x["minimum_fitness"] == y["minimum_fitness"]
        assert np.array_equal(x["dsf"], y["dsf"])


def test_autotune_plain_engine_has_nothing_to_tune(engine):
    cfg, data, freq = _specs(engine)[0]
    with engine.Batch(engine=engine.ENGINE_PLAIN_FP64) as b:
        b.add_run(cfg, *data, freq)
        b.setup()
        rep = b.autotune(4)
        assert rep["candidates"] == 0 and rep["parts_per_cta"] == 0
