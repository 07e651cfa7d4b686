// deac_model.hpp -- host-side construction of everything the generation
// loop reads but never changes: the kernel matrix K(tau, omega), the
// normalisation and moment terms, and the transform of the best genome into
// the reported spectrum.  All of it is built in FP64 on the host with the
// C library's exp/cosh/sinh/tanh/pow, in the same operation order as the
// reference (deac.cpp:310-401, 478-538, 605-675, 720-784, 868-924,
// 1594-1675), so that the values are bit-identical to the reference's.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "deac_gb300.h"

namespace deac {

struct Model {
    int sides = 2;             // 2 two-sided, 1 one-sided genome
    double beta = 0.0;         // 1/T (unused at zero temperature)
    double periodicity = 1.0;  // -1 for the fermionic spectra types
    double zeroth_moment = 0.0;
    std::vector<double> k_pos, k_neg;            // [Nt][M]
    std::vector<double> norm_pos, norm_neg;      // [M]
    std::vector<double> first_pos, first_neg;    // [M]
    std::vector<double> third_pos, third_neg;    // [M]
    std::vector<double> tau_weight;              // [Nt] negative-first-moment terms
    double negative_first_moment = 0.0;
    double negative_first_moment_error = 0.0;
    bool use_first_moment = false;
    bool use_third_moment = false;
    bool use_negative_first_moment = false;
};

// Check a configuration the way the reference front end does before it calls
// deac() (deac.cpp:2093-2106, 2143-2153), plus the variant rules of this
// engine.  Returns an empty string when valid, else the reference message.
std::string check_config(const deac_config& cfg);

// Build every constant term for one run.
void build_model(const deac_config& cfg, const double* tau, const double* isf,
                 const double* isf_error, uint64_t nt, const double* freq,
                 uint64_t m, Model& out, bool with_kernel = true);
// Rows [i0, i1) of the kernel matrix into out.k_pos / out.k_neg (sized nt * m
// by the caller; out.sides, beta and periodicity set, as build_model leaves
// them): with_kernel = false and this, row blocks on several threads, give
// build_model's matrix.
void kernel_rows(const deac_config& cfg, Model& out, const double* tau, const double* freq, uint64_t m,
                 uint64_t i0, uint64_t i1);

// Best genome -> reported spectrum and frequency axis (deac.cpp:1594-1675).
// xpos/xneg are the M genes of the best member (xneg ignored when one-sided).
void best_spectrum(const deac_config& cfg, const Model& model, const double* freq,
                   uint64_t m, const double* xpos, const double* xneg, double* dsf,
                   double* frequency_out);

// Host-side sequential statistics used for the final stats entry
// (deac.cpp:169-183, 1677-1685).
double sequential_mean(const double* f, uint64_t n);
double sequential_squared_mean(const double* f, uint64_t n);

}  // namespace deac
