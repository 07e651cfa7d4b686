"""The npz -> bin converter of the ISF input (the reference's
tools/convert_isf_data.py:11-19): float32 or float64 arrays ``tau``, ``isf``,
``error`` become one float64 block (3, n_tau), which deac.e's loader reads
back as the three arrays."""
import numpy as np
import pytest

from deac_testlib import read_doubles, run_exe
from deac_gb300.convert_isf_data import convert_isf_npz, main


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_convert_writes_three_float64_rows(tmp_path, dtype):
    rng = np.random.default_rng(5)
    tau = np.linspace(0.0, 0.74, 38).astype(dtype)
    isf = (-np.exp(-tau.astype(np.float64)) + 1e-3 * rng.standard_normal(38)).astype(dtype)
    err = np.full(38, 2e-3, dtype=dtype)
    np.savez(tmp_path / "isf.npz", tau=tau, isf=isf, error=err)
    assert main([str(tmp_path / "isf.npz"), str(tmp_path / "isf.bin")]) == 0
    got = read_doubles(tmp_path / "isf.bin")
    want = np.concatenate([tau.astype(np.float64), isf.astype(np.float64), err.astype(np.float64)])
    assert got.dtype == np.float64 and np.array_equal(got, want)
    assert (tmp_path / "isf.bin").stat().st_size == 3 * 38 * 8


def test_convert_rejects_ragged_arrays(tmp_path):
    np.savez(tmp_path / "bad.npz", tau=np.zeros(4), isf=np.zeros(5), error=np.ones(4))
    with pytest.raises(ValueError):
        convert_isf_npz(tmp_path / "bad.npz", tmp_path / "bad.bin")
    assert not (tmp_path / "bad.bin").exists()


def test_converted_file_passes_deac_input_checks(engine, tmp_path):
    """deac.e reads the converted file and gets past every input check: a
    validation failure that comes after the ISF checks (too few generations)
    is the one it reports."""
    tau = np.array([0.0, 0.2, 0.4, 0.6], dtype=np.float32)
    np.savez(tmp_path / "isf.npz", tau=tau, isf=-np.exp(-tau), error=np.full(4, 0.05, dtype=np.float32))
    convert_isf_npz(tmp_path / "isf.npz", tmp_path / "isf.bin")
    r = run_exe(engine.EXE_PATH, ["-T", "1.0", "-N", "1", "--save_directory", str(tmp_path / "out"),
                                  str(tmp_path / "isf.bin")], tmp_path)
    assert r.returncode == 1 and "number_of_generations must be at least 2" in r.stdout, r.stdout
