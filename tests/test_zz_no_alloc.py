"""deac_population_fitness_noalloc: the fitness pass for callers that cannot
allocate device memory (their process's framework or pool allocator owns the
GPU's memory, or a cudaFree would stall their other streams).  It takes the
caller's device buffers and keeps its own scratch in a static device array.

Its values must equal the batch engine's fitness (deac_batch_fetch_state) for
the same population, bit for bit like every other engine test, on calls made
one after the other -- each call finds the previous call's data in the shared
scratch and must not depend on it.  This file is collected last."""
import ctypes

import numpy as np
import pytest

from deac_testlib import config0_data, make_isf, uniform_grid

DEAC_E_INVALID = -1


def _batch_states(engine, cfg, data, freq, generations_later):
    """Population and fitness after set-up and after `generations_later`
    more generations, from the batch engine."""
    with engine.Batch(engine=engine.ENGINE_PLAIN_FP64) as b:
        r = b.add_run(cfg, *data, freq)
        b.setup()
        first = b.fetch_state(r)
        b.launch(generations_later)
        b.sync()
        second = b.fetch_state(r)
    return first, second


def _noalloc(engine, torch, sides, pop, k_pos, k_neg, isf, err):
    lib = engine.load_library()
    dev = torch.device("cuda", 0)
    d_pop = torch.from_numpy(np.ascontiguousarray(pop)).to(dev)
    d_kp = torch.from_numpy(np.ascontiguousarray(k_pos)).to(dev)
    d_kn = torch.from_numpy(np.ascontiguousarray(k_neg)).to(dev) if sides == 2 else None
    d_isf = torch.from_numpy(np.ascontiguousarray(isf)).to(dev)
    d_err = torch.from_numpy(np.ascontiguousarray(err)).to(dev)
    p, m = pop.shape[1], pop.shape[2]
    d_fit = torch.full((p,), float("nan"), dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)
    rc = lib.deac_population_fitness_noalloc(0, stream.cuda_stream, sides, d_pop.data_ptr(), p, m, d_kp.data_ptr(),
                                             d_kn.data_ptr() if d_kn is not None else None, d_isf.data_ptr(),
                                             d_err.data_ptr(), len(isf), d_fit.data_ptr())
    assert rc == 0, lib.deac_last_error().decode()
    stream.synchronize()
    return d_fit.cpu().numpy()


@pytest.mark.gpu
def test_noalloc_fitness_equals_batch_fitness_on_consecutive_calls(engine, oracle):
    torch = pytest.importorskip("torch")
    # two-sided run, then a one-sided run of other sizes: four calls in a row
    tau, isf, err = config0_data(1)
    freq = uniform_grid(64, 64.0)
    cfg = engine.make_config(temperature=1.35, spectra_type="bfull", population_size=24,
                             number_of_generations=1000, seed=3, stop_minimum_fitness=0.0)
    first, later = _batch_states(engine, cfg, (tau, isf, err), freq, 200)
    k_pos, k_neg = oracle.kernel_matrix(cfg, tau, freq)
    for state in (first, later):
        fit = _noalloc(engine, torch, 2, state["population"], k_pos, k_neg, isf, err)
        np.testing.assert_array_equal(fit, state["fitness"])

    data = make_isf(50, 0.5, [(0.6, 3.0, 1.0), (0.4, 9.0, 2.0)], 1e-3, 7)
    freq1 = uniform_grid(96, 20.0)
    cfg1 = engine.make_config(temperature=0.5, bosonic=True, population_size=13, number_of_generations=1000, seed=8,
                              stop_minimum_fitness=0.0)
    first, later = _batch_states(engine, cfg1, data, freq1, 150)
    k_pos1, _ = oracle.kernel_matrix(cfg1, data[0], freq1)
    for state in (first, later):
        fit = _noalloc(engine, torch, 1, state["population"], k_pos1, None, data[1], data[2])
        np.testing.assert_array_equal(fit, state["fitness"])


@pytest.mark.gpu
def test_noalloc_fitness_near_the_scratch_limit(engine, oracle):
    """A population x timeslice model ISF of 16,384,000 bytes (P = 4000,
    N_tau = 512), with its work list and buffer indices 16,646,656 of the
    16 MiB static scratch: two calls in a row, each equal to the batch
    engine's fitness of the same population."""
    torch = pytest.importorskip("torch")
    p, nt, m = 4000, 512, 1024
    tau, isf, err = make_isf(nt, 1.35, [(0.7, 5.0, 1.0), (0.3, 20.0, 3.0)], 1e-4, 5)
    freq = uniform_grid(m, 64.0)
    cfg = engine.make_config(temperature=1.35, spectra_type="bfull", population_size=p,
                             number_of_generations=100, seed=11, stop_minimum_fitness=0.0)
    first, later = _batch_states(engine, cfg, (tau, isf, err), freq, 2)
    k_pos, k_neg = oracle.kernel_matrix(cfg, tau, freq)
    for state in (first, later):
        fit = _noalloc(engine, torch, 2, state["population"], k_pos, k_neg, isf, err)
        np.testing.assert_array_equal(fit, state["fitness"])


@pytest.mark.parametrize("case,message", [
    ("sides", "sides must be 1 or 2"),
    ("empty", "must be positive"),
    ("null", "null device pointer"),
    ("misaligned", "16-byte aligned"),
    ("too-large", "static scratch"),
])
def test_noalloc_rejects_bad_arguments(engine, case, message):
    """Checked before any CUDA call.  Device -1 keeps every one of these calls
    off any GPU even if a check were missing (that would fail as 'no CUDA
    device' instead)."""
    lib = engine.load_library()
    a = 1 << 20  # stand-in addresses: never dereferenced
    args = dict(sides=2, pop=a, p=8, m=64, kp=a, kn=a, isf=a, err=a, nt=64, fit=a)
    if case == "sides":
        args["sides"] = 3
    elif case == "empty":
        args["p"] = 0
    elif case == "null":
        args["kn"] = None
    elif case == "misaligned":
        args["pop"] = a + 8
    elif case == "too-large":
        args["p"], args["nt"] = 4096, 1024  # 32 MiB of model ISF
    rc = lib.deac_population_fitness_noalloc(-1, None, args["sides"], args["pop"], args["p"], args["m"], args["kp"],
                                             args["kn"], args["isf"], args["err"], args["nt"], args["fit"])
    assert rc == DEAC_E_INVALID
    assert message in lib.deac_last_error().decode()
