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
