"""The exact parallel FMA chain of the row-sum kernels (deac_chain.cuh) must
equal the plain one-step-at-a-time chain bit for bit: on the CPU through its
host form (tests/chain_check.cpp), on the GPU through the warp form against
the device's own sequential fma."""
import ctypes
import subprocess

import numpy as np
import pytest

from deac_testlib import REPO


def test_host_chain_matches_sequential_fma(tmp_path):
    exe = tmp_path / "chain_check"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I", str(REPO / "deac-cpp_gb300" / "csrc"),
                    str(REPO / "tests" / "chain_check.cpp"), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe), "6000"], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.startswith("ok")


def test_prng_table_jump_powers_match_the_jump_chain(tmp_path):
    # the per-gene PRNG states come from GF(2) matrix powers of the jump
    # (rng_table_kernel), the initial populations' draws from powers of one
    # step (population_kernel); on the host they must equal the chain of
    # jumps and the sequence of draws
    exe = tmp_path / "rng_jump_check"
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", str(REPO / "deac-cpp_gb300" / "csrc"),
                    str(REPO / "tests" / "rng_jump_check.cpp"), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe), "70000"], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.startswith("ok")


def _chains(kind, n, count, rng):
    x = np.empty((count, n))
    w = np.empty((count, n))
    start = np.zeros(count)
    k = np.arange(n)
    for c in range(count):
        u, v = rng.random(n), rng.random(n)
        if kind == 0:  # normalisation-like
            a, b = u, np.full(n, 0.125)
            b[0] = b[-1] = 0.0625
        elif kind == 1:  # few significant bits
            a = np.ldexp(rng.integers(0, 64, n).astype(float), rng.integers(-4, 4, n))
            b = np.ldexp(rng.integers(1, 17, n).astype(float), rng.integers(-3, 3, n))
            a[rng.random(n) < 0.25] *= -1
        elif kind == 2:  # signed terms: cancellation and sign flips
            a, b = u - 0.5, np.ldexp(1.0, rng.integers(-20, 20, n))
        elif kind == 3:  # exponentially decaying weights
            a, b = 3.0 * u, np.exp(-0.37 * k)
        elif kind == 4:  # zeros, subnormals, huge and tiny terms
            a, b = u.copy(), v.copy()
            a[rng.random(n) < 0.14] = 0.0
            b[rng.random(n) < 0.09] = np.ldexp(1.0, -1060)
            a[rng.random(n) < 0.08] *= 2.0 ** 300
            b[rng.random(n) < 0.06] *= 2.0 ** -300
            a[rng.random(n) < 0.2] *= -1
        elif kind == 5:  # sums landing on binade edges
            a = np.ldexp(1.0, rng.integers(-6, 6, n)) * np.where(rng.random(n) < 0.33, -1.0, 1.0)
            b = 1.0 + np.ldexp(rng.integers(0, 4, n).astype(float), -52)
            start[c] = -np.ldexp(1.0, int(rng.integers(0, 10))) if c % 2 else 0.0
        elif kind == 6:  # integers near 2^53: ties to even
            a = rng.integers(0, 5, n).astype(float)
            b = np.where(rng.random(n) < 0.5, 0.5, 1.5)
            start[c] = 2.0 ** 53 - float(rng.integers(0, 64))
        elif kind == 8:  # positive, few significant bits: ties inside predicted binades
            a = np.ldexp(rng.integers(1, 65, n).astype(float), rng.integers(-4, 4, n))
            b = np.ldexp(rng.integers(1, 17, n).astype(float), rng.integers(-3, 3, n))
        elif kind == 9:  # a peak after tiny first steps: terms far beyond the first states' grid
            centre, width = rng.uniform(n / 8, n / 2), max(2.0, n / 16)
            a = np.exp(-((k - centre) / width) ** 2) * (1.0 + 0.3 * u)
            b = np.full(n, 0.125)
        elif kind == 10:  # positive with rare spikes of 2^10 .. 2^60
            a = u.copy()
            spikes = rng.random(n) < 0.01
            a[spikes] *= np.ldexp(1.0, rng.integers(10, 61, int(spikes.sum())))
            b = np.full(n, 0.125)
        else:  # random sign and scale
            a = (u - 0.5) * np.ldexp(1.0, rng.integers(-30, 30, n))
            b = (v - 0.25) * np.ldexp(1.0, rng.integers(-30, 30, n))
        x[c], w[c] = a, b
    return x, w, start


@pytest.mark.gpu
@pytest.mark.parametrize("n", [1, 7, 256, 257, 4096, 5000, 12288])
def test_warp_chain_matches_sequential_fma(engine, n):
    lib = engine.load_debug_library()
    fn = lib.deac_debug_fma_chains
    dp = ctypes.POINTER(ctypes.c_double)
    fn.restype = ctypes.c_int
    fn.argtypes = [dp, dp, ctypes.c_uint64, dp, ctypes.c_uint32, dp, dp]
    rng = np.random.default_rng(n)
    for kind in range(11):
        x, w, start = _chains(kind, n, 48, rng)
        fast = np.zeros(len(start))
        plain = np.zeros(len(start))
        p = lambda a: a.ctypes.data_as(dp)
        rc = fn(p(x), p(w), n, p(start), len(start), p(fast), p(plain))
        assert rc == 0, lib.deac_debug_last_error().decode()
        same = (fast.view(np.uint64) == plain.view(np.uint64)) | (np.isnan(fast) & np.isnan(plain))
        assert same.all(), (kind, np.flatnonzero(~same)[:5], fast[~same][:3], plain[~same][:3])
