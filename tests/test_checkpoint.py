"""Checkpoint and resume (the state the reference's --save_state names,
deac.cpp:2004-2007): a run checkpointed after some generations and restored
into a fresh batch ends exactly as the same run never interrupted -- the same
generation count, minimum fitness, spectrum, statistics and final
population, fitness, CR and F."""
import numpy as np
import pytest

from deac_testlib import config0_data, uniform_grid

pytestmark = pytest.mark.gpu


def _cfg(engine, **over):
    kw = dict(temperature=1.35, spectra_type="bfull", population_size=8, number_of_generations=400, seed=21,
              stop_minimum_fitness=0.0, track_stats=True, normalize=True)
    kw.update(over)
    return engine.make_config(**kw)


def _inputs():
    tau, isf, err = config0_data(2)
    return tau, isf, err, uniform_grid(64, 64.0)


def _same(a, b):
    for k in ("generation", "minimum_fitness"):
        assert a[k] == b[k], k
    for k in ("dsf", "frequency", "stats_mean", "stats_minimum", "stats_squared_mean"):
        if k in a:
            assert np.array_equal(a[k], b[k]), k


@pytest.mark.parametrize("after", [16, 112])
def test_resumed_run_equals_uninterrupted_run(engine, after):
    cfg = _cfg(engine)
    data = _inputs()
    with engine.Batch() as b:
        r = b.add_run(cfg, *data)
        b.run()
        want, want_state = b.fetch(r), b.fetch_state(r)
    with engine.Batch() as b:
        r = b.add_run(cfg, *data)
        b.setup()
        b.launch(after)
        assert b.sync() == 0  # still running at the checkpoint
        block = b.checkpoint(r)
    with engine.Batch() as b:
        r = b.add_run(cfg, *data)
        b.setup()
        b.restore(r, block)
        b.run()
        got, got_state = b.fetch(r), b.fetch_state(r)
    _same(got, want)
    for k in want_state:
        assert np.array_equal(got_state[k], want_state[k]), k


def test_restore_refuses_another_configuration(engine):
    data = _inputs()
    with engine.Batch() as b:
        r = b.add_run(_cfg(engine), *data)
        b.setup()
        block = b.checkpoint(r)
    with engine.Batch() as b:
        r = b.add_run(_cfg(engine, population_size=12), *data)
        b.setup()
        with pytest.raises(engine.DeacError, match="different configuration"):
            b.restore(r, block)
        with pytest.raises(engine.DeacError, match="too short"):
            b.restore(r, block[:16])


@pytest.mark.parametrize("change", ["seed", "isf", "temperature"])
def test_restore_refuses_a_run_with_other_inputs(engine, change):
    """Same sizes and flags, other seed, data or temperature: refused."""
    tau, isf, err, freq = _inputs()
    with engine.Batch() as b:
        r = b.add_run(_cfg(engine), tau, isf, err, freq)
        b.setup()
        block = b.checkpoint(r)
    over, data = {}, (tau, isf, err, freq)
    if change == "seed":
        over = dict(seed=22)
    elif change == "temperature":
        over = dict(temperature=1.4)
    else:
        isf2 = isf.copy()
        isf2[5] *= 1.0 + 1e-12
        data = (tau, isf2, err, freq)
    with engine.Batch() as b:
        r = b.add_run(_cfg(engine, **over), *data)
        b.setup()
        with pytest.raises(engine.DeacError, match="other inputs"):
            b.restore(r, block)


@pytest.mark.parametrize("engine_from,engine_to,after,stats", [
    ("split", "split", 16, True), ("split", "split", 112, False), ("plain", "split", 48, False),
    ("plain", "split", 112, True)])
def test_split_engine_checkpoints(engine, engine_from, engine_to, after, stats):
    """A split-engine run checkpointed and restored into a new split batch,
    and a plain-engine checkpoint continued by the split engine, end exactly
    as the plain run never interrupted (the split engine's decisions are the
    FP64 ones).  Without statistics most decisions are the intervals'."""
    kinds = {"plain": engine.ENGINE_PLAIN_FP64, "split": engine.ENGINE_SPLIT_BF16}
    cfg = _cfg(engine, track_stats=stats)
    data = _inputs()
    with engine.Batch() as b:
        r = b.add_run(cfg, *data)
        b.run()
        want, want_state = b.fetch(r), b.fetch_state(r)
    with engine.Batch(engine=kinds[engine_from]) as b:
        r = b.add_run(cfg, *data)
        b.setup()
        b.launch(after)
        assert b.sync() == 0
        block = b.checkpoint(r)
    with engine.Batch(engine=kinds[engine_to]) as b:
        r = b.add_run(cfg, *data)
        b.setup()
        b.restore(r, block)
        b.run()
        got, got_state = b.fetch(r), b.fetch_state(r)
    _same(got, want)
    for k in want_state:
        assert np.array_equal(got_state[k], want_state[k]), k


def test_split_checkpoint_refused_by_the_plain_engine(engine):
    data = _inputs()
    with engine.Batch(engine=engine.ENGINE_SPLIT_BF16) as b:
        r = b.add_run(_cfg(engine), *data)
        b.setup()
        b.launch(16)
        block = b.checkpoint(r)
    with engine.Batch() as b:
        r = b.add_run(_cfg(engine), *data)
        b.setup()
        with pytest.raises(engine.DeacError, match="continues only in the split engine"):
            b.restore(r, block)
