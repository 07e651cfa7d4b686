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


# The reference's own smoke test runs deac.e four times on a four-timeslice
# negative ISF (tau 0..0.6, F -1..-0.61, sigma 0.05) with -T 1.0 -P 8 -M 8
# --omega_max 4.0 and the default spectra type spfsf, checking the output
# sizes and the log (test/deac_smoke_test.py:84-177).  The same runs here,
# on the GPU, must also equal the oracle's runs.
SMOKE_TAU = [0.0, 0.2, 0.4, 0.6]
SMOKE_ISF = [-1.0, -0.85, -0.72, -0.61]
SMOKE_ERR = [0.05, 0.05, 0.05, 0.05]
SMOKE_RUNS = {
    # case: (seed, generations, extra flags, config overrides)
    "default": (1, 2, [], {}),
    "normalize": (2, 2, ["--normalize"], dict(normalize=True)),
    "first_moment": (3, 2, ["--first_moment", "0.5"], dict(first_moment=0.5)),
    "track_stats": (4, 3, ["--track_stats"], dict(track_stats=True)),
}


@pytest.mark.parametrize("case", sorted(SMOKE_RUNS))
def test_reference_smoke_runs_on_the_gpu(engine, oracle, tmp_path, case):
    seed, n, extra, over = SMOKE_RUNS[case]
    isf_file = tmp_path / "tiny-isf.bin"
    write_doubles(isf_file, SMOKE_TAU + SMOKE_ISF + SMOKE_ERR)
    save = tmp_path / "results"
    args = ["-T", "1.0", "-N", str(n), "-P", "8", "-M", "8", "--omega_max", "4.0", "--save_directory", str(save),
            "--seed", str(seed)] + extra + [str(isf_file)]
    r = run_exe(engine.EXE_PATH, args, tmp_path)
    assert r.returncode == 0, r.stdout
    assert "minimum_fitness:" in r.stdout
    prefix = "deac-spfsf"
    for kind in ("dsf", "frequency"):
        assert (save / f"{prefix}_{kind}_{seed}.bin").stat().st_size == (2 * 8 - 1) * 8
    out = read_outputs(save, prefix, str(seed), track_stats=case == "track_stats")
    assert "minimum_fitness:" in out["log"]
    if case == "track_stats":
        for k in ("mean", "minimum", "squared-mean"):
            assert (save / f"{prefix}_stats_fitness-{k}_{seed}.bin").stat().st_size == 3 * 8
        assert 'fitness_mean_filename: ""' not in out["log"]
    cfg = engine.make_config(temperature=1.0, number_of_generations=n, population_size=8, seed=seed, **over)
    ref = oracle.run(cfg, np.array(SMOKE_TAU), np.array(SMOKE_ISF), np.array(SMOKE_ERR), uniform_grid(8, 4.0),
                     order=GPU_ORDER)
    assert out["generation"] == ref["generation"]
    assert np.array_equal(out["dsf"], ref["dsf"])
    assert np.array_equal(out["frequency"], ref["frequency"])
    if case == "track_stats":
        for k in ("stats_mean", "stats_minimum", "stats_squared_mean"):
            assert np.array_equal(out[k], ref[k]), k


def test_frequency_file_run_on_the_gpu(engine, oracle, tmp_path):
    """deac.e with a non-uniform --frequency_file grid (the reference's
    backend-parity scenario, test/deac_parity_test.py:45-73, run to 300
    generations instead of stopping at once), and a denser non-uniform grid
    of 96 points: every output equals the oracle's."""
    tau, isf, err = config0_data(4)
    isf_file = tmp_path / "isf.bin"
    write_doubles(isf_file, list(tau) + list(isf) + list(err))
    grids = {"four": np.array([0.0, 0.7, 1.8, 3.0]),
             "dense": 64.0 * (np.arange(96, dtype=np.float64) / 95.0) ** 1.5}
    for tag, grid in grids.items():
        freq_file = tmp_path / f"freq_{tag}.bin"
        write_doubles(freq_file, list(grid))
        cfg = engine.make_config(temperature=1.35, population_size=8, number_of_generations=300, seed=17,
                                 stop_minimum_fitness=1.0, spectra_type="bfull", track_stats=True)
        save = tmp_path / tag
        args = cli_args(cfg, isf_file, save, frequency_file=freq_file, uuid="17")
        r = run_exe(engine.EXE_PATH, args, tmp_path)
        assert r.returncode == 0, r.stdout
        out = read_outputs(save, output_prefix(cfg), "17", track_stats=True)
        ref = oracle.run(cfg, tau, isf, err, grid, order=GPU_ORDER)
        assert out["generation"] == ref["generation"], tag
        assert np.array_equal(out["dsf"], ref["dsf"]), tag
        assert np.array_equal(out["frequency"], ref["frequency"]), tag
        for k in ("stats_mean", "stats_minimum", "stats_squared_mean"):
            assert np.array_equal(out[k], ref[k]), (tag, k)
