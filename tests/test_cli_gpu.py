"""deac.e on the GPU, end to end through the files: an isf.bin in, the
reference's dsf/frequency/stats .bin files and log out.  The outputs must
equal the GPU-order oracle's (the same spectrum, frequency axis, generation
and statistics), and `--engine split` must write byte-identical .bin files
and the same log."""
import filecmp

import numpy as np
import pytest

from deac_testlib import (GPU_ORDER, cli_args, config0_data, output_prefix, read_outputs, run_exe, uniform_grid,
                          write_doubles)

pytestmark = pytest.mark.gpu

CASES = {
    "standard-bfull": dict(spectra_type="bfull"),
    "normalize-stats": dict(spectra_type="bfull", normalize=True, track_stats=True),
    "bosonic": dict(bosonic=True),
}


def _run(engine, tmp_path, cfg, data, m, omax, extra, tag):
    isf_file = tmp_path / "isf.bin"
    tau, isf, err = data
    write_doubles(isf_file, list(tau) + list(isf) + list(err))
    save = tmp_path / tag
    args = cli_args(cfg, isf_file, save, genome_size=m, omega_max=omax, uuid="t")
    if cfg.bosonic:
        args = ["--bosonic"] + args
    r = run_exe(engine.EXE_PATH, list(extra) + args, tmp_path)
    assert r.returncode == 0, r.stdout
    return save, read_outputs(save, output_prefix(cfg), "t", track_stats=bool(cfg.track_stats))


@pytest.mark.parametrize("name", sorted(CASES))
def test_deac_exe_matches_oracle_and_engines_agree(engine, oracle, tmp_path, name):
    kw = dict(temperature=1.35, population_size=8, number_of_generations=400, seed=11, stop_minimum_fitness=1.0)
    kw.update(CASES[name])
    cfg = engine.make_config(**kw)
    data = config0_data(2)
    m, omax = 64, 64.0
    save_plain, out = _run(engine, tmp_path, cfg, data, m, omax, [], "plain")
    ref = oracle.run(cfg, *data, uniform_grid(m, omax), order=GPU_ORDER)
    assert out["generation"] == ref["generation"]
    assert np.array_equal(out["dsf"], ref["dsf"])
    assert np.array_equal(out["frequency"], ref["frequency"])
    assert float(out["minimum_fitness_text"]) == pytest.approx(ref["minimum_fitness"], rel=1e-5)
    if cfg.track_stats:
        for k in ("stats_mean", "stats_minimum", "stats_squared_mean"):
            assert np.array_equal(out[k], ref[k]), k
    save_split, _ = _run(engine, tmp_path, cfg, data, m, omax, ["--engine", "split"], "split")
    plain_files = sorted(p.name for p in save_plain.iterdir())
    assert plain_files == sorted(p.name for p in save_split.iterdir())
    for f in plain_files:
        if f.endswith(".dat"):  # the log names the files with their directory
            a = (save_plain / f).read_text().replace(str(save_plain), "DIR")
            b = (save_split / f).read_text().replace(str(save_split), "DIR")
            assert a == b, f
        else:
            assert filecmp.cmp(save_plain / f, save_split / f, shallow=False), f


def test_seed_range_matches_single_seed_runs_and_the_average(engine, oracle, tmp_path):
    """`--number_of_seeds 3 --seed 9` runs seeds 9, 10 and 11 in one batch:
    each seed's files equal the oracle's run of that seed, and the average
    file equals the reference's averaging of those dsf files, which sums them
    in the sorted order of their names ("10", "11", "9") and divides by 3
    (tools/plot_simple_average_deac_results.py:10-27)."""
    cfg = engine.make_config(temperature=1.35, population_size=8, number_of_generations=300, seed=9,
                             stop_minimum_fitness=1.0, spectra_type="bfull", normalize=True)
    data = config0_data(3)
    m, omax = 64, 64.0
    isf_file = tmp_path / "isf.bin"
    tau, isf, err = data
    write_doubles(isf_file, list(tau) + list(isf) + list(err))
    save = tmp_path / "seeds"
    avg_file = tmp_path / "average.bin"
    args = cli_args(cfg, isf_file, save, genome_size=m, omega_max=omax)
    r = run_exe(engine.EXE_PATH, ["--number_of_seeds", "3", "--average_file", avg_file] + args, tmp_path)
    assert r.returncode == 0, r.stdout
    prefix = output_prefix(cfg)
    dsfs = {}
    for seed in (9, 10, 11):
        out = read_outputs(save, prefix, str(seed))
        cfg.seed = seed
        ref = oracle.run(cfg, *data, uniform_grid(m, omax), order=GPU_ORDER)
        assert out["generation"] == ref["generation"], seed
        assert np.array_equal(out["dsf"], ref["dsf"]), seed
        assert np.array_equal(out["frequency"], ref["frequency"]), seed
        assert f"seed: {seed}\n" in out["log"]
        dsfs[str(seed)] = out["dsf"]
    keys = sorted(dsfs)
    avg = dsfs[keys[0]].copy()
    for k in keys[1:]:
        avg += dsfs[k]
    avg /= len(keys)
    assert np.array_equal(np.fromfile(avg_file, dtype=np.float64), avg)
