// deac_model.cpp -- see deac_model.hpp.  Compiled with -ffp-contract=off:
// none of these expressions is fused in the reference either.
#include "deac_model.hpp"

#include <cmath>

namespace deac {

namespace {

bool fermionic(int spectra_type) {
    return spectra_type == DEAC_SPECTRA_SPFSF || spectra_type == DEAC_SPECTRA_FFULL;
}

// trapezoid weight of grid point j (deac.cpp:351-358)
double trapezoid(const double* g, uint64_t n, uint64_t j) {
    if (j == 0) return 0.5 * (g[j + 1] - g[j]);
    if (j == n - 1) return 0.5 * (g[j] - g[j - 1]);
    return 0.5 * (g[j + 1] - g[j - 1]);
}

}  // namespace

std::string check_config(const deac_config& c) {
    if (c.model < DEAC_MODEL_STANDARD || c.model > DEAC_MODEL_NORMALIZATION)
        return "model must be standard, hyperbolic or normalization";
    if (c.bosonic) {
        if (c.spectra_type != DEAC_SPECTRA_BDSF)
            return "Please choose spectra_type from the following options: bdsf";
    } else {
        if (c.spectra_type < DEAC_SPECTRA_SPBSF || c.spectra_type > DEAC_SPECTRA_FFULL)
            return "Please choose spectra_type from the following options: spbsf, spfsf, bfull, ffull";
        if (c.zero_temperature)
            return "zero temperature requires the one-sided (bosonic) genome";
    }
    if (!c.zero_temperature && (!std::isfinite(c.temperature) || c.temperature <= 0.0))
        return "temperature must be positive for non-ZeroT builds";
    if (c.number_of_generations < 2) return "number_of_generations must be at least 2";
    if (c.population_size < 4) return "population_size must be at least 4";
    if (!std::isfinite(c.first_moment)) return "first_moment must be finite";
    if (!std::isfinite(c.third_moment)) return "third_moment must be finite";
    if (c.third_moment >= 0.0 && (!std::isfinite(c.third_moment_error) || c.third_moment_error <= 0.0))
        return "third_moment_error must be positive when third_moment is used";
    if (c.first_moment_formula != DEAC_FIRST_MOMENT_GPU && c.first_moment_formula != DEAC_FIRST_MOMENT_CPU)
        return "first_moment_formula must be gpu or cpu";
    return std::string();
}

// Rows [i0, i1) of the kernel matrix (deac.cpp:310-401) into o.k_pos /
// o.k_neg, sized nt * m by the caller; o.beta and o.periodicity set.
void kernel_rows(const deac_config& c, Model& o, const double* tau, const double* freq, uint64_t m, uint64_t i0,
                 uint64_t i1) {
    const bool two = o.sides == 2;
    const double beta = o.beta, per = o.periodicity;
    for (uint64_t i = i0; i < i1; ++i) {
        const double t = tau[i];
        for (uint64_t j = 0; j < m; ++j) {
            const double f = freq[j];
            const double df = trapezoid(freq, m, j);
            const uint64_t idx = i * m + j;
            if (c.zero_temperature) {
                o.k_pos[idx] = df * std::exp(-t * f);
            } else if (c.model == DEAC_MODEL_HYPERBOLIC) {
                if (!two) {
                    const double half_beta_minus_tau = 0.5 * beta - t;
                    o.k_pos[idx] = df * std::cosh(half_beta_minus_tau * f);
                } else {
                    const double shifted_up = -0.5 * beta - t;   // tau + beta
                    const double shifted_down = 1.5 * beta - t;  // tau - beta
                    o.k_pos[idx] = per * df * std::exp(shifted_up * f) / 2;
                    o.k_neg[idx] = per * df * std::exp(-shifted_down * f) / 2;
                }
            } else if (c.model == DEAC_MODEL_STANDARD) {
                if (!two) {
                    const double beta_minus_tau = beta - t;
                    o.k_pos[idx] = df * (std::exp(-beta_minus_tau * f) + std::exp(-t * f));
                } else {
                    const double tau_minus_beta = t - beta;
                    o.k_pos[idx] = df * std::exp(-t * f);
                    o.k_neg[idx] = per * df * std::exp(tau_minus_beta * f);
                }
            } else {
                if (!two) {
                    const double beta_minus_tau = beta - t;
                    const double num = std::exp(-beta_minus_tau * f) + std::exp(-t * f);
                    const double den = 1.0 + std::exp(-beta * f);
                    o.k_pos[idx] = df * (num / den);
                } else {
                    const double tau_minus_beta = t - beta;
                    const double num = std::exp(-t * f);
                    const double den = 1.0 + std::exp(-beta * f);
                    o.k_pos[idx] = df * (num / den);
                    const double e = std::exp(tau_minus_beta * f);
                    const double den_n = 1.0 + std::exp(-beta * f);
                    o.k_neg[idx] = per * df * (e - e / den_n);
                }
            }
        }
    }

}

void build_model(const deac_config& c, const double* tau, const double* isf,
                 const double* err, uint64_t nt, const double* freq, uint64_t m,
                 Model& o, bool with_kernel) {
    o = Model();
    o.sides = c.bosonic ? 1 : 2;
    const bool two = o.sides == 2;
    if (!c.zero_temperature) {
        o.beta = 1.0 / c.temperature;
        o.periodicity = fermionic(c.spectra_type) ? -1.0 : 1.0;
    }
    o.zeroth_moment = isf[0];
    o.use_first_moment = c.first_moment >= 0.0;
    o.use_third_moment = c.third_moment >= 0.0;
    // the negative first moment exists only for the one-sided genome and is
    // switched off at zero temperature (deac.cpp:234-239, 868-924)
    o.use_negative_first_moment = c.use_negative_first_moment && c.bosonic && !c.zero_temperature;
    const double beta = o.beta, per = o.periodicity;

    // kernel matrix, deac.cpp:310-401
    if (with_kernel) {
        o.k_pos.assign(nt * m, 0.0);
        if (two) o.k_neg.assign(nt * m, 0.0);
        kernel_rows(c, o, tau, freq, m, 0, nt);
    }

    // normalisation terms, deac.cpp:493-538
    if (c.normalize) {
        o.norm_pos.assign(m, 0.0);
        if (two) o.norm_neg.assign(m, 0.0);
        for (uint64_t j = 0; j < m; ++j) {
            const double f = freq[j];
            const double df = trapezoid(freq, m, j);
            if (c.zero_temperature) {
                o.norm_pos[j] = df;
                if (two) o.norm_neg[j] = df;
            } else if (c.model == DEAC_MODEL_HYPERBOLIC) {
                if (!two) {
                    o.norm_pos[j] = df * std::cosh(0.5 * beta * f);
                } else {
                    o.norm_pos[j] = 0.5 * df / std::exp(-0.5 * beta * f);
                    o.norm_neg[j] = 0.5 * df * std::exp(-0.5 * beta * f);
                }
            } else if (c.model == DEAC_MODEL_STANDARD) {
                if (!two) {
                    o.norm_pos[j] = df * (1.0 + std::exp(-beta * f));
                } else {
                    o.norm_pos[j] = df;
                    o.norm_neg[j] = df;
                }
            } else {
                if (!two) {
                    o.norm_pos[j] = df;
                } else {
                    o.norm_pos[j] = df * (1.0 / (1.0 + std::exp(-beta * f)));
                    const double e = std::exp(-beta * f);
                    o.norm_neg[j] = df * (e / (1.0 + e));
                }
            }
        }
    }

    // first / third moment terms, deac.cpp:630-675, 720-784.  The third
    // moment term is df * pow(f,3) * f, i.e. the fourth power, as released.
    auto moments = [&](bool third, std::vector<double>& tp, std::vector<double>& tn) {
        tp.assign(m, 0.0);
        if (two) tn.assign(m, 0.0);
        for (uint64_t j = 0; j < m; ++j) {
            const double f = freq[j];
            const double df = trapezoid(freq, m, j);
            // a = df*f (first) or df*pow(f,3)*f (third), evaluated left to right
            const double f3 = third ? std::pow(f, 3) : 0.0;
            auto lead = [&](double coeff_df) { return third ? coeff_df * f3 * f : coeff_df * f; };
            if (c.zero_temperature) {
                tp[j] = lead(df);
                if (two) tn[j] = lead(-df);
            } else if (c.model == DEAC_MODEL_HYPERBOLIC) {
                if (!two) {
                    tp[j] = lead(df) * std::sinh(0.5 * beta * f);
                } else {
                    tp[j] = lead(0.5 * df) / std::exp(-0.5 * beta * f);
                    tn[j] = lead(-0.5 * df) * std::exp(-0.5 * beta * f);
                }
            } else if (c.model == DEAC_MODEL_STANDARD) {
                if (!two) {
                    tp[j] = lead(df) * (1.0 - std::exp(-beta * f));
                } else {
                    tp[j] = lead(df);
                    tn[j] = lead(-df);
                }
            } else {
                if (!two) {
                    tp[j] = lead(df) * std::tanh(0.5 * beta * f);
                } else {
                    tp[j] = lead(df) * (1.0 / (1.0 + std::exp(-beta * f)));
                    const double e = std::exp(-beta * f);
                    tn[j] = lead(-df) * (e / (1.0 + e));
                }
            }
        }
    };
    if (o.use_first_moment) moments(false, o.first_pos, o.first_neg);
    if (o.use_third_moment) moments(true, o.third_pos, o.third_neg);

    // negative first moment, deac.cpp:878-894: the target is a plain running
    // sum, and its error keeps only the last timeslice's term because the
    // reference assigns where it means to accumulate (deac.cpp:890).
    if (o.use_negative_first_moment) {
        o.tau_weight.assign(nt, 0.0);
        double target = 0.0, err2 = 0.0;
        for (uint64_t j = 0; j < nt; ++j) {
            const double dt = trapezoid(tau, nt, j);
            o.tau_weight[j] = dt;
            target = target + isf[j] * dt;
            err2 = (err[j] * err[j]) * (dt * dt);
        }
        o.negative_first_moment = target;
        o.negative_first_moment_error = std::sqrt(err2);
    }
}

void best_spectrum(const deac_config& c, const Model& o, const double* freq, uint64_t m,
                   const double* xpos, const double* xneg, double* dsf, double* fout) {
    const bool two = o.sides == 2;
    const double beta = o.beta;
    const int st = c.spectra_type;
    const double two_pi = 2.0 * 3.14159265358979323846;
    for (uint64_t i = 0; i < m; ++i) {
        const double f = freq[i];
        const double xp = xpos[i];
        const double xn = two ? xneg[i] : 0.0;
        double p, n = 0.0;
        if (c.zero_temperature) {
            p = xp;
            n = xn;
        } else if (c.model == DEAC_MODEL_HYPERBOLIC) {
            if (!two) {
                p = 0.5 * xp * std::exp(0.5 * beta * f);
            } else if (st == DEAC_SPECTRA_SPBSF) {
                p = -two_pi * xp * std::sinh(beta * f / 2);
                n = two_pi * xn * std::sinh(beta * f / 2);
            } else if (st == DEAC_SPECTRA_SPFSF) {
                p = -two_pi * xp * std::cosh(beta * f / 2);
                n = -two_pi * xn * std::cosh(beta * f / 2);
            } else {
                p = 0.5 * xp * std::exp(0.5 * beta * f);
                n = 0.5 * xn * std::exp(-0.5 * beta * f);
            }
        } else if (c.model == DEAC_MODEL_STANDARD) {
            if (!two) {
                p = xp;
            } else if (st == DEAC_SPECTRA_SPBSF) {
                p = -two_pi * xp * (1.0 - std::exp(-beta * f));
                n = -two_pi * xn * (1.0 - std::exp(beta * f));
            } else if (st == DEAC_SPECTRA_SPFSF) {
                p = -two_pi * xp * (1.0 + std::exp(-beta * f));
                n = -two_pi * xn * (1.0 + std::exp(beta * f));
            } else {
                p = xp;
                n = xn;
            }
        } else {
            if (!two) {
                p = xp / (1.0 + std::exp(-beta * f));
            } else if (st == DEAC_SPECTRA_SPBSF) {
                p = -two_pi * xp * std::tanh(0.5 * beta * f);
                n = two_pi * xn * std::tanh(0.5 * beta * f);
            } else if (st == DEAC_SPECTRA_SPFSF) {
                p = -two_pi * xp;
                n = -two_pi * xn;
            } else {
                p = xp / (1.0 + std::exp(-beta * f));
                n = xn / (1.0 + std::exp(beta * f));
            }
        }
        if (!two) {
            fout[i] = f;
            dsf[i] = p;
        } else {
            // -omega_max .. omega_max; at i = 0 both indices coincide and the
            // negative side is written last (centre frequency -0.0)
            const uint64_t ip = m + i - 1, in = m - i - 1;
            fout[ip] = f;
            fout[in] = -f;
            dsf[ip] = p;
            dsf[in] = n;
        }
    }
}

double sequential_mean(const double* f, uint64_t n) {
    double s = 0.0;
    for (uint64_t i = 0; i < n; ++i) s += f[i];
    return s / n;
}

double sequential_squared_mean(const double* f, uint64_t n) {
    double s = 0.0;
    for (uint64_t i = 0; i < n; ++i) s = s + f[i] * f[i];
    return s / n;
}

}  // namespace deac
