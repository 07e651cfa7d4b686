"""deac.e front end: help, spectra-type check and the input-validation
failures, which all happen before the GPU is touched.  Cases follow the
reference's smoke test (test/deac_smoke_test.py:9-34, 180-259): each must
exit with status 1 and print the reference's message."""
import struct

import pytest

from deac_testlib import run_exe, write_doubles


def _fixture(path, tau=(0.0, 0.2, 0.4, 0.6), isf=(-1.0, -0.85, -0.72, -0.61), err=(0.05,) * 4):
    write_doubles(path, list(tau) + list(isf) + list(err))


def _cmd(tmp_path, fixture, n="2", p="8", m="8", omega="4.0", extra=()):
    return ["-T", "1.0", "-N", n, "-P", p, "-M", m, "--omega_max", omega,
            "--save_directory", str(tmp_path / "results"), "--seed", "7", *extra, str(fixture)]


def test_help(engine, tmp_path):
    r = run_exe(engine.EXE_PATH, ["--help"], tmp_path)
    assert r.returncode == 0 and "Usage: deac-cpp" in r.stdout


def test_bad_spectra_type(engine, tmp_path):
    _fixture(tmp_path / "isf.bin")
    r = run_exe(engine.EXE_PATH, ["-T", "1.0", "--spectra_type", "invalid", str(tmp_path / "isf.bin")], tmp_path)
    assert r.returncode == 1 and "Please choose spectra_type" in r.stdout


def test_missing_positional(engine, tmp_path):
    r = run_exe(engine.EXE_PATH, ["-T", "1.0"], tmp_path)
    assert r.returncode == 1 and "isf_file" in r.stdout


def _case(name, d):
    f = d / "invalid-isf.bin"
    ff = d / "frequency.bin"
    opts, extra = {}, ()
    if name == "bad_isf_byte_length":
        f.write_bytes(b"not-a-double")
        msg = "does not contain a whole number of doubles"
    elif name == "empty_isf":
        f.write_bytes(b"")
        msg = "is empty"
    elif name == "uneven_isf_arrays":
        write_doubles(f, [0.0, 0.2, -1.0, 0.05])
        msg = "ISF input file must contain tau, isf, and error arrays of equal length"
    elif name == "too_few_timeslices":
        _fixture(f, (0.0,), (-1.0,), (0.05,))
        msg = "ISF input file must contain at least two timeslices"
    elif name == "nonfinite_isf":
        _fixture(f, isf=(-1.0, float("nan"), -0.72, -0.61))
        msg = "ISF input file contains non-finite values"
    elif name == "positive_isf_single_particle":
        _fixture(f, isf=(1.0, 0.85, 0.72, 0.61))
        msg = "positive ISF values are not supported for single-particle spectra"
    elif name == "nonpositive_error":
        _fixture(f, err=(0.05, 0.0, 0.05, 0.05))
        msg = "ISF input errors must be positive"
    elif name == "bad_third_moment_error":
        _fixture(f)
        extra = ("--third_moment", "1.0", "--third_moment_error", "0.0")
        msg = "third_moment_error must be positive when third_moment is used"
    elif name == "too_few_generations":
        _fixture(f)
        opts = {"n": "1"}
        msg = "number_of_generations must be at least 2"
    elif name == "too_small_population":
        _fixture(f)
        opts = {"p": "3"}
        msg = "population_size must be at least 4"
    elif name == "too_small_genome":
        _fixture(f)
        opts = {"m": "1"}
        msg = "genome_size must be at least 2"
    elif name == "bad_omega_max":
        _fixture(f)
        opts = {"omega": "0.0"}
        msg = "omega_max must be positive"
    elif name == "short_frequency_file":
        _fixture(f)
        write_doubles(ff, [0.0])
        extra = ("--frequency_file", str(ff))
        msg = "frequency_file must contain at least two frequencies"
    elif name == "nonfinite_frequency":
        _fixture(f)
        write_doubles(ff, [0.0, float("inf")])
        extra = ("--frequency_file", str(ff))
        msg = "frequencies must be finite and non-negative"
    elif name == "negative_frequency":
        _fixture(f)
        write_doubles(ff, [0.0, -1.0])
        extra = ("--frequency_file", str(ff))
        msg = "frequencies must be finite and non-negative"
    elif name == "unsorted_frequency":
        _fixture(f)
        write_doubles(ff, [0.0, 2.0, 1.0])
        extra = ("--frequency_file", str(ff))
        msg = "frequencies must be sorted in non-decreasing order"
    elif name == "missing_file":
        f = d / "does-not-exist.bin"
        msg = "File error:"
    else:
        raise KeyError(name)
    return f, opts, extra, msg


CASES = ["bad_isf_byte_length", "empty_isf", "uneven_isf_arrays", "too_few_timeslices", "nonfinite_isf",
         "positive_isf_single_particle", "nonpositive_error", "bad_third_moment_error", "too_few_generations",
         "too_small_population", "too_small_genome", "bad_omega_max", "short_frequency_file",
         "nonfinite_frequency", "negative_frequency", "unsorted_frequency", "missing_file"]


@pytest.mark.parametrize("name", CASES)
def test_validation(engine, tmp_path, name):
    f, opts, extra, msg = _case(name, tmp_path)
    r = run_exe(engine.EXE_PATH, _cmd(tmp_path, f, extra=extra, **opts), tmp_path)
    assert r.returncode == 1, r.stdout
    assert msg in r.stdout


def test_zero_temperature_two_sided_rejected(engine, tmp_path):
    _fixture(tmp_path / "isf.bin")
    r = run_exe(engine.EXE_PATH, ["--zero_temperature", "--spectra_type", "bfull", str(tmp_path / "isf.bin")],
                tmp_path)
    assert r.returncode == 1 and "--bosonic" in r.stdout


@pytest.mark.parametrize("extra,msg", [
    (("--number_of_seeds", "0"), "number_of_seeds must be at least 1"),
    (("--number_of_seeds", "2", "--uuid", "run"), "uuid cannot be combined with number_of_seeds > 1"),
    (("--number_of_seeds", "2", "--average_file", "no-such-dir/avg.bin"), "average_file directory does not exist"),
    (("--first_moment_formula", "mixed"), "--first_moment_formula must be gpu or cpu"),
    (("--streams", "table"), "--streams must be reference or counter"),
    (("--engine", "fast"), "--engine must be plain or split"),
])
def test_seed_range_validation(engine, tmp_path, extra, msg):
    _fixture(tmp_path / "isf.bin")
    r = run_exe(engine.EXE_PATH, _cmd(tmp_path, tmp_path / "isf.bin", extra=extra), tmp_path)
    assert r.returncode == 1, r.stdout
    assert msg in r.stdout
