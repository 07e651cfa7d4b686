"""Synthetic inputs of the benchmark configurations.

There is no public dataset for this path; the recipe itself is the
benchmark: S(omega) is a Gaussian mixture, F(tau) its two-sided
detailed-balance transform sum_w [e^{-tau w} + e^{-(beta-tau) w}] S(w) dw on
a fine grid, sigma(tau) = rel * F(tau), and F_data = F + sigma * N(0,1) drawn
with numpy.random.default_rng(seed).
"""
from __future__ import annotations

import numpy as np


def gaussian(w, mean, sd):
    return np.exp(-0.5 * ((w - mean) / sd) ** 2) / (sd * np.sqrt(2 * np.pi))


def make_isf(n_tau, temperature, peaks, rel_error=1e-4, seed=1, omega_max_data=None,
             n_omega_data=20001, tau_max=None):
    """(tau, F_data, sigma) for peaks = [(weight, mean, sd), ...]; tau uniform
    on [0, tau_max] (default beta = 1/T)."""
    beta = 1.0 / temperature
    if omega_max_data is None:
        omega_max_data = max(m + 8 * s for _, m, s in peaks)
    w = np.linspace(0.0, omega_max_data, n_omega_data)
    dw = w[1] - w[0]
    s = sum(a * gaussian(w, m, sd) for a, m, sd in peaks)
    tau = np.linspace(0.0, beta if tau_max is None else tau_max, n_tau)
    kern = np.exp(-np.outer(tau, w)) + np.exp(-np.outer(beta - tau, w))
    f = kern @ (s * dw)
    sigma = rel_error * np.abs(f)
    rng = np.random.default_rng(seed)
    f_data = f + sigma * rng.standard_normal(n_tau)
    return tau, f_data, sigma


TWO_PEAKS = [(0.7, 5.0, 1.0), (0.3, 20.0, 3.0)]
THREE_PEAKS = [(0.5, 3.0, 0.5), (0.3, 40.0, 5.0), (0.2, 200.0, 30.0)]


def config0_data(seed=1):
    """Plain FP64 single run: T=1.35, N_tau=64 on [0, beta],
    S = 0.7 N(5,1) + 0.3 N(20,3), sigma = 1e-4 F."""
    return make_isf(64, 1.35, TWO_PEAKS, 1e-4, seed)


def config1_data(seed=1, temperature=1.35):
    """The reference's production scale: the same recipe with N_tau = 128."""
    return make_isf(128, temperature, TWO_PEAKS, 1e-4, seed)


def config2_data(seed=1, temperature=1.35):
    """Precision-form single run: N_tau = 256, three peaks at 3, 40, 200
    (sd 0.5, 5, 30; weights 0.5, 0.3, 0.2), sigma = 1e-5 F."""
    return make_isf(256, temperature, THREE_PEAKS, 1e-5, seed, omega_max_data=512.0, n_omega_data=40001)


def uniform_grid(m, omega_max):
    """deac.e's frequency grid, i * (omega_max / (M - 1)) (deac.cpp:2123-2126)."""
    d = omega_max / (m - 1)
    return np.array([i * d for i in range(m)], dtype=np.float64)


# ---- batched configurations: many independent runs, each drawn from its seed

MODELS = ("standard", "hyperbolic", "normalization")


def _noisy(f, rel_error, rng):
    sigma = rel_error * np.abs(f)
    return f + sigma * rng.standard_normal(len(f)), sigma


def config3_runs(n_runs=1024, first_seed=1, n_tau=128, omega_max=64.0):
    """The batching form's runs: seeds first_seed .. first_seed + n_runs - 1;
    from each run's seed (numpy default_rng) its genome size M from {1024,
    4096, 16384}, population from {8, 32, 64}, temperature from {0.5, 1.35,
    3.0} and model from {standard, hyperbolic, normalization}, each uniform;
    N_tau = 128 and the single-run recipe at its temperature (0.7 N(5,1) +
    0.3 N(20,3), sigma = 1e-4 F, noise from the seed); genome on [0, 64] as
    in the single-run configuration.  Returns a list of dicts (seed, model,
    temperature, population_size, genome_size, tau, isf, err, frequency)."""
    w = np.linspace(0.0, max(m + 8 * s for _, m, s in TWO_PEAKS), 20001)
    s = sum(a * gaussian(w, m, sd) for a, m, sd in TWO_PEAKS) * (w[1] - w[0])
    clean, grids = {}, {}
    runs = []
    for k in range(n_runs):
        seed = first_seed + k
        rng = np.random.default_rng(seed)
        m = int(rng.choice([1024, 4096, 16384]))
        p = int(rng.choice([8, 32, 64]))
        t = float(rng.choice([0.5, 1.35, 3.0]))
        model = MODELS[int(rng.integers(3))]
        if t not in clean:
            beta = 1.0 / t
            tau = np.linspace(0.0, beta, n_tau)
            clean[t] = (tau, (np.exp(-np.outer(tau, w)) + np.exp(-np.outer(beta - tau, w))) @ s)
        if m not in grids:
            grids[m] = uniform_grid(m, omega_max)
        tau, f = clean[t]
        isf, err = _noisy(f, 1e-4, rng)
        runs.append(dict(seed=seed, model=model, temperature=t, population_size=p, genome_size=m, tau=tau,
                         isf=isf, err=err, frequency=grids[m]))
    return runs


def config4_runs(n_runs=4096, first_seed=1, n_tau=512, genome_size=16384, omega_max=1024.0, temperature=1.35,
                 n_omega_data=20001, omega_max_data=1500.0):
    """The batched split-precision runs at full size: each run's S(omega) a
    mixture of 1-4 Gaussians (count uniform, centres U[1, 800], sd U[0.5, 50],
    Dirichlet(1) weights) drawn from its seed; N_tau = 512 on [0, beta],
    sigma = 1e-5 F, genome M = 16384 on [0, 1024], T = 1.35 (the
    configuration names none).  Every run shares tau, the genome grid and so
    the kernel matrix.  Returns (tau, frequency, [(seed, isf, err), ...])."""
    beta = 1.0 / temperature
    tau = np.linspace(0.0, beta, n_tau)
    w = np.linspace(0.0, omega_max_data, n_omega_data)
    dw = w[1] - w[0]
    kern = np.exp(-np.outer(tau, w)) + np.exp(-np.outer(beta - tau, w))
    out = []
    block = 256
    for k0 in range(0, n_runs, block):
        seeds = range(first_seed + k0, first_seed + min(n_runs, k0 + block))
        rngs = [np.random.default_rng(sd) for sd in seeds]
        smat = np.zeros((len(w), len(rngs)))
        for c, rng in enumerate(rngs):
            n = int(rng.integers(1, 5))
            centres = rng.uniform(1.0, 800.0, n)
            sds = rng.uniform(0.5, 50.0, n)
            weights = rng.dirichlet(np.ones(n))
            smat[:, c] = sum(a * gaussian(w, m, sd) for a, m, sd in zip(weights, centres, sds)) * dw
        f = kern @ smat
        for c, (sd, rng) in enumerate(zip(seeds, rngs)):
            isf, err = _noisy(f[:, c], 1e-5, rng)
            out.append((sd, isf, err))
    return tau, uniform_grid(genome_size, omega_max), out
