/*
 * deac_oracle.c -- CPU oracle of the DEAC per-generation loop.
 *
 * TEST INFRASTRUCTURE.  This file is the checker that the GPU engine is
 * compared against and the CPU baseline that bench.py times; the product
 * never links or calls it.  It restates, in plain C, the algorithm of
 * nscottnichols/deac-cpp 2.0.0-rc1 (all citations are paths inside that
 * project), written from the reference's source as a specification:
 *
 *  - PRNG: src/deac/include/rng.hpp:10-131 (splitmix64 seeding with the
 *    32-bit-half packing quirk, xoshiro256+, the 2^128 jump, to_double2).
 *  - kernel matrix, normalisation and moment terms: deac.cpp:310-401,
 *    478-538, 605-675, 720-784, 868-924 for every model variant.
 *  - the generation loop: deac.cpp:1137-1574, in one of two orders:
 *
 *    GPU order (the engine's target) follows the USE_GPU branches and the
 *    kernels of src/deac/src/deac_gpu.cu: one xoshiro state per (member,
 *    gene, side) taken from a table of jump()-separated states
 *    (deac.cpp:1114-1135), per-kernel state offsets (deac.cpp:1170-1174,
 *    1219-1222), two k-ascending FMA chains per contraction output added at
 *    the end (deac_gpu.cu:277-315, two calls deac.cpp:1378-1382), the
 *    1024-slot pairwise-tree chi^2 (deac_gpu.cu:417-448) and fitness
 *    statistics (deac_gpu.cu:458-512), the GPU first-moment formula with
 *    first_moment_error = 1.0 (deac.cpp:623, deac_gpu.cu:450-456).
 *    Two defects of the reference CUDA build are NOT reproduced:
 *      * gpu_get_minimum accumulates into an uninitialised buffer
 *        (deac_gpu.cu:402); here the minimum is the minimum, as in the
 *        reference HIP and SYCL backends, so the stop criterion works;
 *      * gpu_deac_gemv with beta=1 lets every x-block add its row sum into y
 *        (deac_gpu.cu:345-374), so --normalize and the moment terms get a
 *        nondeterministic multiple of the negative-side sum once M > 32.
 *        Here y = fma(alpha, s_neg, alpha*s_pos), the single-block value,
 *        where s is the k-ascending FMA chain every block computes.
 *
 *    CPU order follows the #else branches (deac.cpp:437-446, 1180-1241,
 *    1261-1311, 1539-1571): one PRNG stream, member-major draws, one FMA
 *    chain over the positive then the negative side, sequential chi^2, the
 *    CPU first-moment formula, and no normalisation inside the loop (the
 *    reference only normalises the initial population on the CPU,
 *    deac.cpp:1343-1363).  This order exists to pin the oracle against the
 *    unmodified reference CPU build.
 *
 * Floating point: the reference is compiled with FMA contraction (nvcc
 * default; g++ -O3 -march=native in GNU mode).  Every a*b+c that the
 * reference build fuses is written here as an explicit fma(), and this file
 * is compiled with -ffp-contract=off so that nothing else is fused.  On the
 * host side g++ fuses the accumulations that go through memory (the
 * matrix_multiply_* loops, deac.cpp:102-118) and straight-line updates, but
 * not loops that carry their accumulator in a register: chi^2
 * (deac.cpp:120-126), squared_mean (deac.cpp:177-183), the
 * negative-first-moment target (deac.cpp:888), and the inlined
 * matrix_multiply_* sites whose destination it keeps in a register (the
 * normalisation of the initial population, the one-sided contraction inside
 * the loop, the one-sided row sums, the negative-first-moment and the
 * third-moment sums).
 * This map was established by comparing against the reference CPU build
 * (g++ 13, -O3 -march=native, x86-64) bit for bit, stats arrays included;
 * another host compiler may fuse differently.  nvcc fuses every a*b+c of
 * the device code.
 */
#include "deac_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------ PRNG */

/* splitmix64, rng.hpp:10-15 */
static uint64_t splitmix64_next(uint64_t* s) {
    uint64_t r = (*s += 0x9E3779B97f4A7C15ULL);
    r = (r ^ (r >> 30)) * 0xBF58476D1CE4E5B9ULL;
    r = (r ^ (r >> 27)) * 0x94D049BB133111EBULL;
    return r ^ (r >> 31);
}

static uint64_t rotl64(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

/* xoshiro256+, rng.hpp:25-38 */
uint64_t deac_oracle_rng_next(uint64_t s[4]) {
    const uint64_t result = s[0] + s[3];
    const uint64_t t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = rotl64(s[3], 45);
    return result;
}

/* xoshiro256p_init, rng.hpp:46-59: each 64-bit splitmix output fills two
 * state words with its low and high 32-bit halves. */
void deac_oracle_rng_init(uint64_t seed, uint64_t s[4]) {
    uint64_t sm = seed;
    uint64_t a = splitmix64_next(&sm);
    s[0] = (uint32_t)a;
    s[1] = (uint32_t)(a >> 32);
    uint64_t b = splitmix64_next(&sm);
    s[2] = (uint32_t)b;
    s[3] = (uint32_t)(b >> 32);
}

/* 2^128-step jump, rng.hpp:64-87 (published xoshiro256 jump polynomial). */
void deac_oracle_rng_jump(uint64_t s[4]) {
    static const uint64_t JUMP[4] = {0x180ec6d33cfd0abaULL, 0xd5a61266f0c9392cULL,
                                     0xa9582618e03fc9aaULL, 0x39abdc4529b1661cULL};
    uint64_t a = 0, b = 0, c = 0, d = 0;
    for (int i = 0; i < 4; i++) {
        for (int bit = 0; bit < 64; bit++) {
            if (JUMP[i] & (1ULL << bit)) {
                a ^= s[0];
                b ^= s[1];
                c ^= s[2];
                d ^= s[3];
            }
            deac_oracle_rng_next(s);
        }
    }
    s[0] = a;
    s[1] = b;
    s[2] = c;
    s[3] = d;
}

/* (x >> 11) * 2^-53, rng.hpp:129-131 and every inline use in deac.cpp */
static double u01(uint64_t x) { return (double)(x >> 11) * 0x1.0p-53; }

/* --------------------------------------------------------------- helpers */

/* trapezoid weight of frequency j, deac.cpp:351-358 */
static double trapezoid(const double* f, uint64_t n, uint64_t j) {
    if (j == 0) return 0.5 * (f[j + 1] - f[j]);
    if (j == n - 1) return 0.5 * (f[j] - f[j - 1]);
    return 0.5 * (f[j + 1] - f[j - 1]);
}

/* k-ascending FMA chain starting from `acc` (gpu_matmul / gpu_deac_gemv
 * inner loops, deac_gpu.cu:302-304, 359-363; CPU matrix_multiply_*,
 * deac.cpp:102-118). */
static double chain(const double* a, const double* b, uint64_t n, double acc) {
    for (uint64_t k = 0; k < n; k++) acc = fma(a[k], b[k], acc);
    return acc;
}

/* the same sum with separate multiply and add roundings (the reference
 * host build at the call sites listed in the file header) */
static double chain_unfused(const double* a, const double* b, uint64_t n, double acc) {
    for (uint64_t k = 0; k < n; k++) acc = acc + a[k] * b[k];
    return acc;
}

static uint64_t pow2_ceil(uint64_t n) {
    uint64_t w = 1;
    while (w < n) w <<= 1;
    return w;
}

/* Pairwise tree of the reference block reductions (deac_gpu.cu:431-442,
 * gpu_reduce_add deac_gpu.cu:63-129 with GPU_BLOCK_SIZE=1024): slot t holds
 * the values t, t+1024, ... summed in order; levels s = 512..1 add slot t+s
 * into slot t.  Slots past the data hold +0.0, so levels wider than the
 * data change nothing and the tree starts at pow2_ceil(min(n,1024))/2. */
static double tree_sum(double* slots, uint64_t width) {
    for (uint64_t s = width / 2; s > 0; s >>= 1)
        for (uint64_t t = 0; t < s; t++) slots[t] += slots[t + s];
    return slots[0];
}

/* ----------------------------------------------------------------- model */

typedef struct {
    const deac_config* c;
    int order;
    int S;                 /* sides: 2 two-sided, 1 one-sided */
    uint64_t P, M, Nt, N;
    double beta, periodicity;
    const double *tau, *isf, *err, *freq;
    double *Kp, *Kn;        /* [Nt][M] */
    double *np_, *nn_;      /* normalisation terms [M] */
    double *fmp, *fmn;      /* first-moment terms [M] */
    double *tmp_, *tmn;     /* third-moment terms [M] */
    double *dt;             /* negative-first-moment terms [Nt] */
    double nfm_target, nfm_error;
    int use_fm, use_tm, use_nfm;
    double zeroth;
    /* state */
    double *pop_old[2], *pop_new[2];            /* [P][M] per side */
    double *cr_old[2], *cr_new[2], *w_old[2], *w_new[2];
    double *fit_old, *fit_new, *E, *slots;
    uint64_t *states;       /* GPU order: table of xoshiro states, 4 words each */
    uint64_t key_crossover, key_jde; /* GPU order with counter streams */
    uint64_t rng[4];        /* host stream */
    uint64_t *mutant;       /* 3*P */
    unsigned char *mask[2]; /* [P][M] */
} oracle_t;

static int is_fermionic(int spectra_type) {
    return spectra_type == DEAC_SPECTRA_SPFSF || spectra_type == DEAC_SPECTRA_FFULL;
}

/* K(tau, omega) for both sides, deac.cpp:310-401 */
static void build_kernel(oracle_t* o) {
    const deac_config* c = o->c;
    const double beta = o->beta, per = o->periodicity;
    for (uint64_t i = 0; i < o->Nt; i++) {
        const double t = o->tau[i];
        for (uint64_t j = 0; j < o->M; j++) {
            const double f = o->freq[j];
            const double df = trapezoid(o->freq, o->M, j);
            const uint64_t idx = i * o->M + j;
            if (c->zero_temperature) {
                /* deac.cpp:392-399 (one-sided; two-sided ZeroT does not build) */
                o->Kp[idx] = df * exp(-t * f);
            } else if (c->model == DEAC_MODEL_HYPERBOLIC) {
                if (o->S == 1) {
                    const double bo2mt = 0.5 * beta - t;
                    o->Kp[idx] = df * cosh(bo2mt * f);
                } else {
                    const double bo2mtp = -0.5 * beta - t;
                    const double bo2mtn = 1.5 * beta - t;
                    o->Kp[idx] = per * df * exp(bo2mtp * f) / 2;
                    o->Kn[idx] = per * df * exp(-bo2mtn * f) / 2;
                }
            } else if (c->model == DEAC_MODEL_STANDARD) {
                if (o->S == 1) {
                    const double bmt = beta - t;
                    o->Kp[idx] = df * (exp(-bmt * f) + exp(-t * f));
                } else {
                    const double tmb = t - beta;
                    o->Kp[idx] = df * exp(-t * f);
                    o->Kn[idx] = per * df * exp(tmb * f);
                }
            } else { /* normalization model */
                if (o->S == 1) {
                    const double bmt = beta - t;
                    const double num = exp(-bmt * f) + exp(-t * f);
                    const double den = 1.0 + exp(-beta * f);
                    o->Kp[idx] = df * (num / den);
                } else {
                    const double tmb = t - beta;
                    const double num = exp(-t * f);
                    const double den = 1.0 + exp(-beta * f);
                    o->Kp[idx] = df * (num / den);
                    const double e = exp(tmb * f);
                    const double dn = 1.0 + exp(-beta * f);
                    o->Kn[idx] = per * df * (e - e / dn);
                }
            }
        }
    }
}

/* normalisation terms, deac.cpp:493-538 */
static void build_normalization_terms(oracle_t* o) {
    const double beta = o->beta;
    for (uint64_t j = 0; j < o->M; j++) {
        const double f = o->freq[j];
        const double df = trapezoid(o->freq, o->M, j);
        if (o->c->zero_temperature) {
            o->np_[j] = df;
            if (o->S == 2) o->nn_[j] = df;
        } else if (o->c->model == DEAC_MODEL_HYPERBOLIC) {
            if (o->S == 1) {
                o->np_[j] = df * cosh(0.5 * beta * f);
            } else {
                o->np_[j] = 0.5 * df / exp(-0.5 * beta * f);
                o->nn_[j] = 0.5 * df * exp(-0.5 * beta * f);
            }
        } else if (o->c->model == DEAC_MODEL_STANDARD) {
            if (o->S == 1) {
                o->np_[j] = df * (1.0 + exp(-beta * f));
            } else {
                o->np_[j] = df;
                o->nn_[j] = df;
            }
        } else {
            if (o->S == 1) {
                o->np_[j] = df;
            } else {
                o->np_[j] = df * (1.0 / (1.0 + exp(-beta * f)));
                const double e = exp(-beta * f);
                o->nn_[j] = df * (e / (1.0 + e));
            }
        }
    }
}

/* first (power 1) and third (power 3, written pow(f,3)*f as in the
 * reference, deac.cpp:746-783) moment terms, deac.cpp:630-675 */
static void build_moment_terms(oracle_t* o, int third, double* tp, double* tn) {
    const double beta = o->beta;
    for (uint64_t j = 0; j < o->M; j++) {
        const double f = o->freq[j];
        const double df = trapezoid(o->freq, o->M, j);
        if (!third) {
            if (o->c->zero_temperature) {
                tp[j] = df * f;
                if (o->S == 2) tn[j] = -df * f;
            } else if (o->c->model == DEAC_MODEL_HYPERBOLIC) {
                if (o->S == 1) {
                    tp[j] = df * f * sinh(0.5 * beta * f);
                } else {
                    tp[j] = 0.5 * df * f / exp(-0.5 * beta * f);
                    tn[j] = -0.5 * df * f * exp(-0.5 * beta * f);
                }
            } else if (o->c->model == DEAC_MODEL_STANDARD) {
                if (o->S == 1) {
                    tp[j] = df * f * (1.0 - exp(-beta * f));
                } else {
                    tp[j] = df * f;
                    tn[j] = -df * f;
                }
            } else {
                if (o->S == 1) {
                    tp[j] = df * f * tanh(0.5 * beta * f);
                } else {
                    tp[j] = df * f * (1.0 / (1.0 + exp(-beta * f)));
                    const double e = exp(-beta * f);
                    tn[j] = -df * f * (e / (1.0 + e));
                }
            }
        } else {
            const double f3 = pow(f, 3);
            if (o->c->zero_temperature) {
                tp[j] = df * f3 * f;
                if (o->S == 2) tn[j] = -df * f3 * f;
            } else if (o->c->model == DEAC_MODEL_HYPERBOLIC) {
                if (o->S == 1) {
                    tp[j] = df * f3 * f * sinh(0.5 * beta * f);
                } else {
                    tp[j] = 0.5 * df * f3 * f / exp(-0.5 * beta * f);
                    tn[j] = -0.5 * df * f3 * f * exp(-0.5 * beta * f);
                }
            } else if (o->c->model == DEAC_MODEL_STANDARD) {
                if (o->S == 1) {
                    tp[j] = df * f3 * f * (1.0 - exp(-beta * f));
                } else {
                    tp[j] = df * f3 * f;
                    tn[j] = -df * f3 * f;
                }
            } else {
                if (o->S == 1) {
                    tp[j] = df * f3 * f * tanh(0.5 * beta * f);
                } else {
                    tp[j] = df * f3 * f * (1.0 / (1.0 + exp(-beta * f)));
                    const double e = exp(-beta * f);
                    tn[j] = -df * f3 * f * (e / (1.0 + e));
                }
            }
        }
    }
}

/* negative first moment (one-sided genome only), deac.cpp:878-894: the
 * target is sum_tau F*dt and its "error" keeps only the last term, because
 * the reference assigns instead of accumulating (deac.cpp:890). */
static void build_negative_first_moment(oracle_t* o) {
    double target = 0.0, errsq = 0.0;
    for (uint64_t j = 0; j < o->Nt; j++) {
        double dtj;
        if (j == 0) dtj = 0.5 * (o->tau[j + 1] - o->tau[j]);
        else if (j == o->Nt - 1) dtj = 0.5 * (o->tau[j] - o->tau[j - 1]);
        else dtj = 0.5 * (o->tau[j + 1] - o->tau[j - 1]);
        o->dt[j] = dtj;
        target = target + o->isf[j] * dtj;
        errsq = (o->err[j] * o->err[j]) * (dtj * dtj);
    }
    o->nfm_target = target;
    o->nfm_error = sqrt(errsq);
}

/* ------------------------------------------------------------ evaluation */

/* GPU-order gemv pair (deac_gpu.cu:345-374, called with beta=0 then beta=1):
 * y = fma(alpha, s_neg, alpha*s_pos). */
static double gemv_gpu(const oracle_t* o, uint64_t i, double* const pop[2],
                       const double* tp, const double* tn, double alpha) {
    double y = alpha * chain(pop[0] + i * o->M, tp, o->M, 0.0);
    if (o->S == 2) y = fma(alpha, chain(pop[1] + i * o->M, tn, o->M, 0.0), y);
    return y;
}

/* CPU-order row sum: one chain over the positive then the negative side
 * (matrix_multiply_MxN_by_Nx1 called twice into the same accumulator); the
 * one-sided build keeps its single call's accumulator in a register. */
static double gemv_cpu(const oracle_t* o, uint64_t i, double* const pop[2],
                       const double* tp, const double* tn) {
    double y = (o->S == 1) ? chain_unfused(pop[0] + i * o->M, tp, o->M, 0.0) : chain(pop[0] + i * o->M, tp, o->M, 0.0);
    if (o->S == 2) y = chain(pop[1] + i * o->M, tn, o->M, y);
    return y;
}

/* --normalize on the GPU path: gemv with alpha = 1/F(0), then
 * gpu_deac_dgmmDiv1D multiplies by the reciprocal (deac_gpu.cu:406-415). */
static void normalize_gpu(oracle_t* o, double* pop[2]) {
    const double alpha = 1.0 / o->zeroth;
    for (uint64_t i = 0; i < o->P; i++) {
        const double norm = gemv_gpu(o, i, pop, o->np_, o->nn_, alpha);
        const double r = 1.0 / norm;
        for (int s = 0; s < o->S; s++)
            for (uint64_t j = 0; j < o->M; j++) pop[s][i * o->M + j] *= r;
    }
}

/* --normalize of the initial population on the CPU path, deac.cpp:581-601
 * (its accumulator lives in a register in the reference build: unfused) */
static void normalize_cpu(oracle_t* o, double* pop[2]) {
    for (uint64_t i = 0; i < o->P; i++) {
        double norm = chain_unfused(pop[0] + i * o->M, o->np_, o->M, 0.0);
        if (o->S == 2) norm = chain_unfused(pop[1] + i * o->M, o->nn_, o->M, norm);
        for (uint64_t j = 0; j < o->M; j++) {
            pop[0][i * o->M + j] *= o->zeroth / norm;
            if (o->S == 2) pop[1][i * o->M + j] *= o->zeroth / norm;
        }
    }
}

/* model ISF of member i and its fitness (contraction, moments, chi^2).
 * `setup` marks the evaluation of the initial population (deac.cpp:857),
 * as opposed to the one inside the loop (deac.cpp:1386). */
static double fitness_of(oracle_t* o, uint64_t i, double* pop[2], int setup) {
    const uint64_t M = o->M, Nt = o->Nt;
    double* E = o->E + i * Nt;
    for (uint64_t t = 0; t < Nt; t++) {
        if (o->order == DEAC_ORACLE_GPU_ORDER) {
            /* two gpu_matmul calls: C = 1*c_pos + 0*C, then C = 1*c_neg + 1*C */
            double e = chain(pop[0] + i * M, o->Kp + t * M, M, 0.0);
            if (o->S == 2) e = chain(pop[1] + i * M, o->Kn + t * M, M, 0.0) + e;
            E[t] = e;
        } else {
            /* one continued chain (deac.cpp:857-865, 1386-1394).  The
             * one-sided build fuses it at the set-up site and carries it in a
             * register, unfused, inside the loop */
            double e;
            if (o->S == 2) e = chain(o->Kn + t * M, pop[1] + i * M, M, chain(o->Kp + t * M, pop[0] + i * M, M, 0.0));
            else if (setup)
                e = chain(o->Kp + t * M, pop[0] + i * M, M, 0.0);
            else e = chain_unfused(o->Kp + t * M, pop[0] + i * M, M, 0.0);
            E[t] = e;
        }
    }
    double fit;
    if (o->order == DEAC_ORACLE_GPU_ORDER) {
        const uint64_t lanes = Nt < 1024 ? Nt : 1024;
        const uint64_t width = pow2_ceil(lanes);
        for (uint64_t s = 0; s < width; s++) o->slots[s] = 0.0;
        for (uint64_t t = 0; t < Nt; t++) {
            const double term = (o->isf[t] - E[t]) / o->err[t];
            o->slots[t % 1024] = fma(term, term, o->slots[t % 1024]);
        }
        fit = tree_sum(o->slots, width) / (double)Nt;
    } else {
        /* reduced_chi_square_statistic, deac.cpp:120-126: the register
         * accumulator of this loop is not fused by the reference build */
        double chi = 0.0;
        for (uint64_t t = 0; t < Nt; t++) {
            const double term = (o->isf[t] - E[t]) / o->err[t];
            chi = chi + term * term;
        }
        fit = chi / (double)Nt;
    }
    if (o->use_nfm) {
        /* negative first moment from the model ISF (deac.cpp:1410-1414) */
        const double m = (o->order == DEAC_ORACLE_GPU_ORDER) ? chain(E, o->dt, Nt, 0.0)
                                                             : chain_unfused(E, o->dt, Nt, 0.0);
        const double term = (o->nfm_target - m) / o->nfm_error;
        fit = fma(term, term, fit);
    }
    if (o->use_fm) {
        if (o->order == DEAC_ORACLE_GPU_ORDER && o->c->first_moment_formula == DEAC_FIRST_MOMENT_CPU) {
            /* the CPU build's term on the GPU order's moment */
            const double m = gemv_gpu(o, i, pop, o->fmp, o->fmn, 1.0);
            const double d = m - o->c->first_moment;
            fit = fit + (d * d) / o->c->first_moment; /* deac.cpp:969 */
        } else if (o->order == DEAC_ORACLE_GPU_ORDER) {
            const double m = gemv_gpu(o, i, pop, o->fmp, o->fmn, 1.0);
            const double term = (o->c->first_moment - m) / 1.0; /* deac.cpp:623 */
            fit = fma(term, term, fit);
        } else {
            const double m = gemv_cpu(o, i, pop, o->fmp, o->fmn);
            const double d = m - o->c->first_moment;
            fit = fit + (d * d) / o->c->first_moment; /* deac.cpp:969 */
        }
    }
    if (o->use_tm) {
        double m;
        if (o->order == DEAC_ORACLE_GPU_ORDER) {
            m = gemv_gpu(o, i, pop, o->tmp_, o->tmn, 1.0);
        } else {
            m = chain_unfused(pop[0] + i * o->M, o->tmp_, o->M, 0.0);
            if (o->S == 2) m = chain_unfused(pop[1] + i * o->M, o->tmn, o->M, m);
        }
        const double term = (o->c->third_moment - m) / o->c->third_moment_error;
        fit = fma(term, term, fit);
    }
    return fit;
}

/* GPU-order fitness mean / mean of squares (deac_gpu.cu:458-512) */
static double stat_tree(oracle_t* o, const double* f, int squared) {
    const uint64_t P = o->P;
    const uint64_t lanes = P < 1024 ? P : 1024;
    const uint64_t width = pow2_ceil(lanes);
    for (uint64_t s = 0; s < width; s++) o->slots[s] = 0.0;
    for (uint64_t s = 0; s < lanes; s++) o->slots[s] = squared ? f[s] * f[s] : f[s];
    for (uint64_t s = 1024; s < P; s++) {
        if (squared) o->slots[s % 1024] = fma(f[s], f[s], o->slots[s % 1024]);
        else o->slots[s % 1024] += f[s];
    }
    return tree_sum(o->slots, width) / (double)P;
}

/* deac.cpp:169-183 */
static double seq_mean(const double* f, uint64_t n) {
    double m = 0.0;
    for (uint64_t i = 0; i < n; i++) m += f[i];
    return m / n;
}
static double seq_squared_mean(const double* f, uint64_t n) {
    double m = 0.0;
    for (uint64_t i = 0; i < n; i++) m = m + f[i] * f[i];
    return m / n;
}
static double seq_min(const double* f, uint64_t n) {
    double m = f[0];
    for (uint64_t i = 0; i < n; i++)
        if (f[i] < m) m = f[i];
    return m;
}

/* rejection-sampled r1 != r2 != r3 != i (deac.cpp:200-216, deac_gpu.cu:608-626) */
static void mutant_indices(uint64_t* s, uint64_t* r, uint64_t i, uint64_t P) {
    r[0] = r[1] = r[2] = i;
    while (r[0] == i) r[0] = deac_oracle_rng_next(s) % P;
    while (r[1] == i || r[1] == r[0]) r[1] = deac_oracle_rng_next(s) % P;
    while (r[2] == i || r[2] == r[0] || r[2] == r[1]) r[2] = deac_oracle_rng_next(s) % P;
}

static double mutate(const oracle_t* o, double* const old, uint64_t j, const uint64_t* r, double F) {
    const uint64_t M = o->M;
    const double v = fma(F, old[r[1] * M + j] - old[r[2] * M + j], old[r[0] * M + j]);
    return o->c->allow_negative_weight ? v : fabs(v);
}

/* Counter streams (the engine's DEAC_STREAMS_COUNTER layout, which the
 * reference does not have): output `pos` of the SplitMix64 stream whose state
 * starts at `key` -- the (pos+1)-th splitmix64_next() from that state, in one
 * step (the state after n steps is key + n * gamma). */
uint64_t deac_oracle_stream_draw(uint64_t key, uint64_t pos) {
    uint64_t x = key + pos * 0x9E3779B97F4A7C15ULL;
    return splitmix64_next(&x);
}

/* A run's two stream keys: the third and fourth splitmix64 outputs of the
 * seed whose first two seed the population's xoshiro256+ (rng.hpp:46-59). */
void deac_oracle_stream_keys(uint64_t seed, uint64_t keys[2]) {
    uint64_t x = seed;
    splitmix64_next(&x);
    splitmix64_next(&x);
    keys[0] = splitmix64_next(&x);
    keys[1] = splitmix64_next(&x);
}

#define JDE_SPAN (1ULL << 16)

/* One generation's trial vectors in GPU order from counter streams: jDE step
 * n = ii of member i reads the jDE stream at JDE_SPAN (n P + i) + k (k = 4s:
 * CR test of side s, 4s+1 new CR, 4s+2 F test, 4s+3 new F, 8.. the mutant
 * draws); gene j of side s its crossover draw at ((n P + i) S + s) M + j.
 * Arithmetic as trials_gpu. */
static void trials_gpu_counter(oracle_t* o, uint64_t ii) {
    const uint64_t P = o->P, M = o->M, S = (uint64_t)o->S;
    const deac_config* c = o->c;
    for (uint64_t i = 0; i < P; i++) {
        const uint64_t pos0 = JDE_SPAN * (ii * P + i);
        for (uint64_t s = 0; s < S; s++) {
            if (u01(deac_oracle_stream_draw(o->key_jde, pos0 + 4 * s)) < c->self_adapting_crossover_probability)
                o->cr_new[s][i] = u01(deac_oracle_stream_draw(o->key_jde, pos0 + 4 * s + 1));
            else
                o->cr_new[s][i] = o->cr_old[s][i];
            if (u01(deac_oracle_stream_draw(o->key_jde, pos0 + 4 * s + 2)) <
                c->self_adapting_differential_weight_probability)
                o->w_new[s][i] = 2.0 * u01(deac_oracle_stream_draw(o->key_jde, pos0 + 4 * s + 3));
            else
                o->w_new[s][i] = o->w_old[s][i];
        }
        uint64_t k = 8, *r = o->mutant + 3 * i;
        r[0] = r[1] = r[2] = i;
        while (r[0] == i) r[0] = deac_oracle_stream_draw(o->key_jde, pos0 + k++) % P;
        while (r[1] == i || r[1] == r[0]) r[1] = deac_oracle_stream_draw(o->key_jde, pos0 + k++) % P;
        while (r[2] == i || r[2] == r[0] || r[2] == r[1]) r[2] = deac_oracle_stream_draw(o->key_jde, pos0 + k++) % P;
        for (uint64_t s = 0; s < S; s++)
            for (uint64_t j = 0; j < M; j++)
                o->mask[s][i * M + j] =
                    u01(deac_oracle_stream_draw(o->key_crossover, ((ii * P + i) * S + s) * M + j)) < o->cr_new[s][i];
    }
    for (uint64_t s = 0; s < S; s++)
        for (uint64_t i = 0; i < P; i++)
            for (uint64_t j = 0; j < M; j++)
                o->pop_new[s][i * M + j] = o->mask[s][i * M + j]
                                               ? mutate(o, o->pop_old[s], j, o->mutant + 3 * i, o->w_new[s][i])
                                               : o->pop_old[s][i * M + j];
    if (o->S == 2)
        for (uint64_t i = 0; i < P; i++) o->pop_new[1][i * M] = o->pop_new[0][i * M];
    if (c->normalize) normalize_gpu(o, o->pop_new);
}

/* One generation's trial vectors in GPU order (deac.cpp:1168-1259). */
static void trials_gpu(oracle_t* o) {
    const uint64_t P = o->P, M = o->M;
    const deac_config* c = o->c;
    /* jDE: CR on states [0,P) and [2P,3P), F on [P,2P) and [3P,4P) */
    for (int s = 0; s < o->S; s++) {
        for (uint64_t i = 0; i < P; i++) {
            uint64_t* st = o->states + 4 * (2 * P * s + i);
            if (u01(deac_oracle_rng_next(st)) < c->self_adapting_crossover_probability)
                o->cr_new[s][i] = u01(deac_oracle_rng_next(st));
            else
                o->cr_new[s][i] = o->cr_old[s][i];
        }
        for (uint64_t i = 0; i < P; i++) {
            uint64_t* st = o->states + 4 * (2 * P * s + P + i);
            if (u01(deac_oracle_rng_next(st)) < c->self_adapting_differential_weight_probability)
                o->w_new[s][i] = 2.0 * u01(deac_oracle_rng_next(st));
            else
                o->w_new[s][i] = o->w_old[s][i];
        }
    }
    /* mutant indices on states [0,P), crossover masks on [P + s*P*M, ...) with
     * the column-major element index j*P + i (deac_gpu.cu:635-643) */
    for (uint64_t i = 0; i < P; i++) mutant_indices(o->states + 4 * i, o->mutant + 3 * i, i, P);
    for (int s = 0; s < o->S; s++)
        for (uint64_t j = 0; j < M; j++)
            for (uint64_t i = 0; i < P; i++) {
                uint64_t* st = o->states + 4 * (P + (uint64_t)s * P * M + j * P + i);
                o->mask[s][i * M + j] = u01(deac_oracle_rng_next(st)) < o->cr_new[s][i];
            }
    for (int s = 0; s < o->S; s++)
        for (uint64_t i = 0; i < P; i++)
            for (uint64_t j = 0; j < M; j++)
                o->pop_new[s][i * M + j] = o->mask[s][i * M + j]
                                               ? mutate(o, o->pop_old[s], j, o->mutant + 3 * i, o->w_new[s][i])
                                               : o->pop_old[s][i * M + j];
    if (o->S == 2)
        for (uint64_t i = 0; i < P; i++) o->pop_new[1][i * M] = o->pop_new[0][i * M];
    if (c->normalize) normalize_gpu(o, o->pop_new);
}

/* One generation's trial vectors in CPU order (deac.cpp:1180-1311). */
static void trials_cpu(oracle_t* o) {
    const uint64_t P = o->P, M = o->M;
    const deac_config* c = o->c;
    for (uint64_t i = 0; i < P; i++) {
        for (int s = 0; s < o->S; s++) {
            if (u01(deac_oracle_rng_next(o->rng)) < c->self_adapting_crossover_probability)
                o->cr_new[s][i] = u01(deac_oracle_rng_next(o->rng));
            else
                o->cr_new[s][i] = o->cr_old[s][i];
            if (u01(deac_oracle_rng_next(o->rng)) < c->self_adapting_differential_weight_probability)
                o->w_new[s][i] = 2.0 * u01(deac_oracle_rng_next(o->rng));
            else
                o->w_new[s][i] = o->w_old[s][i];
        }
    }
    for (uint64_t i = 0; i < P; i++) {
        mutant_indices(o->rng, o->mutant + 3 * i, i, P);
        for (int s = 0; s < o->S; s++)
            for (uint64_t j = 0; j < M; j++)
                o->mask[s][i * M + j] = u01(deac_oracle_rng_next(o->rng)) < o->cr_new[s][i];
    }
    for (uint64_t i = 0; i < P; i++)
        for (uint64_t j = 0; j < M; j++) {
            for (int s = 0; s < o->S; s++)
                o->pop_new[s][i * M + j] = o->mask[s][i * M + j]
                                               ? mutate(o, o->pop_old[s], j, o->mutant + 3 * i, o->w_new[s][i])
                                               : o->pop_old[s][i * M + j];
            if (o->S == 2 && j == 0) o->pop_new[1][i * M] = o->pop_new[0][i * M];
        }
    /* the CPU build only normalises inside the loop when
     * SINGLE_PARTICLE_FERMIONIC_SPECTRAL_FUNCTION is defined (deac.cpp:1343-1363) */
}

/* best spectrum transform, deac.cpp:1603-1675 */
static void transform(const oracle_t* o, uint64_t best, double* dsf, double* freq) {
    const uint64_t M = o->M, P = o->P;
    const double beta = o->beta;
    const int st = o->c->spectra_type;
    const double twopi = 2.0 * 3.14159265358979323846;
    (void)P;
    for (uint64_t i = 0; i < M; i++) {
        const double f = o->freq[i];
        const double xp = o->pop_old[0][best * M + i];
        const double xn = o->S == 2 ? o->pop_old[1][best * M + i] : 0.0;
        double p, n = 0.0;
        if (o->c->zero_temperature) {
            p = xp;
            n = xn;
        } else if (o->c->model == DEAC_MODEL_HYPERBOLIC) {
            if (o->S == 1) {
                p = 0.5 * xp * exp(0.5 * beta * f);
            } else if (st == DEAC_SPECTRA_SPBSF) {
                p = -twopi * xp * sinh(beta * f / 2);
                n = twopi * xn * sinh(beta * f / 2);
            } else if (st == DEAC_SPECTRA_SPFSF) {
                p = -twopi * xp * cosh(beta * f / 2);
                n = -twopi * xn * cosh(beta * f / 2);
            } else {
                p = 0.5 * xp * exp(0.5 * beta * f);
                n = 0.5 * xn * exp(-0.5 * beta * f);
            }
        } else if (o->c->model == DEAC_MODEL_STANDARD) {
            if (o->S == 1) {
                p = xp;
            } else if (st == DEAC_SPECTRA_SPBSF) {
                p = -twopi * xp * (1.0 - exp(-beta * f));
                n = -twopi * xn * (1.0 - exp(beta * f));
            } else if (st == DEAC_SPECTRA_SPFSF) {
                p = -twopi * xp * (1.0 + exp(-beta * f));
                n = -twopi * xn * (1.0 + exp(beta * f));
            } else {
                p = xp;
                n = xn;
            }
        } else {
            if (o->S == 1) {
                p = xp / (1.0 + exp(-beta * f));
            } else if (st == DEAC_SPECTRA_SPBSF) {
                p = -twopi * xp * tanh(0.5 * beta * f);
                n = twopi * xn * tanh(0.5 * beta * f);
            } else if (st == DEAC_SPECTRA_SPFSF) {
                p = -twopi * xp;
                n = -twopi * xn;
            } else {
                p = xp / (1.0 + exp(-beta * f));
                n = xn / (1.0 + exp(beta * f));
            }
        }
        if (o->S == 1) {
            freq[i] = f;
            dsf[i] = p;
        } else {
            /* ascending -omega_max..omega_max; at i = 0 the negative-side
             * values overwrite the positive ones (centre frequency -0.0) */
            const uint64_t ip = M + i - 1, in = M - i - 1;
            freq[ip] = f;
            freq[in] = -f;
            dsf[ip] = p;
            dsf[in] = n;
        }
    }
}

static void oracle_free(oracle_t* o) {
    free(o->Kp); free(o->Kn); free(o->np_); free(o->nn_); free(o->fmp); free(o->fmn);
    free(o->tmp_); free(o->tmn); free(o->dt);
    for (int s = 0; s < 2; s++) {
        free(o->pop_old[s]); free(o->pop_new[s]); free(o->cr_old[s]); free(o->cr_new[s]);
        free(o->w_old[s]); free(o->w_new[s]); free(o->mask[s]);
    }
    free(o->fit_old); free(o->fit_new); free(o->E); free(o->slots); free(o->states); free(o->mutant);
}

int deac_oracle_kernel_matrix(const deac_config* cfg, const double* tau, uint64_t Nt,
                              const double* freq, uint64_t M, double* k_pos, double* k_neg) {
    oracle_t o;
    memset(&o, 0, sizeof o);
    o.c = cfg;
    o.S = cfg->bosonic ? 1 : 2;
    o.M = M;
    o.Nt = Nt;
    o.tau = tau;
    o.freq = freq;
    if (!cfg->zero_temperature) {
        o.beta = 1.0 / cfg->temperature;
        o.periodicity = is_fermionic(cfg->spectra_type) ? -1.0 : 1.0;
    }
    o.Kp = k_pos;
    o.Kn = k_neg;
    if (o.S == 2 && !k_neg) return -1;
    build_kernel(&o);
    return 0;
}

#define ALLOC(p, n) do { size_t n_ = (size_t)(n); (p) = calloc(n_ > 0 ? n_ : 1, sizeof(*(p))); if (!(p)) goto fail; } while (0)

int deac_oracle_run(const deac_config* c, int32_t order, const double* tau, const double* isf,
                    const double* err, uint64_t Nt, const double* freq, uint64_t M,
                    deac_oracle_out* out, double* best_dsf, double* best_frequency,
                    double* stats_mean, double* stats_minimum, double* stats_squared_mean,
                    double* population, double* fitness, double* trace, uint64_t trace_capacity) {
    oracle_t o;
    memset(&o, 0, sizeof o);
    /* GPU order with counter streams: the GPU order's arithmetic, its
     * per-generation draws from the streams */
    const int counter = order == DEAC_ORACLE_GPU_ORDER_COUNTER;
    if (counter) order = DEAC_ORACLE_GPU_ORDER;
    if (!c || Nt < 2 || M < 2 || c->population_size < 4 || c->number_of_generations < 2) return -1;
    if (c->zero_temperature && !c->bosonic) return -1;
    o.c = c;
    o.order = order;
    o.S = c->bosonic ? 1 : 2;
    o.P = c->population_size;
    o.M = M;
    o.Nt = Nt;
    o.N = c->number_of_generations;
    o.tau = tau;
    o.isf = isf;
    o.err = err;
    o.freq = freq;
    if (!c->zero_temperature) {
        o.beta = 1.0 / c->temperature;
        o.periodicity = is_fermionic(c->spectra_type) ? -1.0 : 1.0;
    }
    o.zeroth = isf[0];
    o.use_fm = c->first_moment >= 0.0;
    o.use_tm = c->third_moment >= 0.0;
    /* ZeroT disables the negative first moment (deac.cpp:234-239); it only
     * exists for the one-sided genome (deac.cpp:868-924) */
    o.use_nfm = c->use_negative_first_moment && c->bosonic && !c->zero_temperature;
    const uint64_t P = o.P;
    const int S = o.S;

    ALLOC(o.Kp, Nt * M);
    if (S == 2) ALLOC(o.Kn, Nt * M);
    ALLOC(o.np_, M); ALLOC(o.nn_, M); ALLOC(o.fmp, M); ALLOC(o.fmn, M);
    ALLOC(o.tmp_, M); ALLOC(o.tmn, M); ALLOC(o.dt, Nt);
    for (int s = 0; s < S; s++) {
        ALLOC(o.pop_old[s], P * M); ALLOC(o.pop_new[s], P * M);
        ALLOC(o.cr_old[s], P); ALLOC(o.cr_new[s], P); ALLOC(o.w_old[s], P); ALLOC(o.w_new[s], P);
        ALLOC(o.mask[s], P * M);
    }
    ALLOC(o.fit_old, P); ALLOC(o.fit_new, P); ALLOC(o.E, P * Nt); ALLOC(o.slots, 1024 + 1);
    ALLOC(o.mutant, 3 * P);

    build_kernel(&o);
    if (c->normalize) build_normalization_terms(&o);
    if (o.use_fm) build_moment_terms(&o, 0, o.fmp, o.fmn);
    if (o.use_tm) build_moment_terms(&o, 1, o.tmp_, o.tmn);
    if (o.use_nfm) build_negative_first_moment(&o);

    /* initial population: one host stream, member-major, positive then
     * negative draw per gene (deac.cpp:429-446, main seeds it at 2089-2091) */
    deac_oracle_rng_init(1407513600ULL + c->seed, o.rng);
    for (uint64_t i = 0; i < P; i++)
        for (uint64_t j = 0; j < M; j++)
            for (int s = 0; s < S; s++) {
                double v = u01(deac_oracle_rng_next(o.rng));
                if (c->allow_negative_weight) v -= 0.5;
                o.pop_old[s][i * M + j] = v;
            }
    if (S == 2)
        for (uint64_t i = 0; i < P; i++) o.pop_old[1][i * M] = o.pop_old[0][i * M];

    if (c->normalize) {
        if (order == DEAC_ORACLE_GPU_ORDER) normalize_gpu(&o, o.pop_old);
        else normalize_cpu(&o, o.pop_old);
    }
    for (uint64_t i = 0; i < P; i++) o.fit_old[i] = fitness_of(&o, i, o.pop_old, 1);
    for (int s = 0; s < S; s++)
        for (uint64_t i = 0; i < P; i++) {
            o.cr_old[s][i] = c->crossover_probability;
            o.w_old[s][i] = c->differential_weight;
        }

    if (counter) {
        uint64_t keys[2];
        deac_oracle_stream_keys(1407513600ULL + c->seed, keys);
        o.key_crossover = keys[0];
        o.key_jde = keys[1];
    } else if (order == DEAC_ORACLE_GPU_ORDER) {
        /* state k = jump^k(state after the initial draws); only the first
         * P + S*P*M of the S*P*(M+1) states of deac.cpp:1116-1126 are read */
        const uint64_t nstates = P + (uint64_t)S * P * M;
        ALLOC(o.states, 4 * nstates);
        for (uint64_t k = 0; k < nstates; k++) {
            memcpy(o.states + 4 * k, o.rng, sizeof o.rng);
            deac_oracle_rng_jump(o.rng);
        }
    }

    uint64_t generation = 0, executed = 0;
    double minimum_fitness = 0.0;
    for (uint64_t ii = 0; ii < o.N - 1; ii++) {
        generation = ii;
        minimum_fitness = seq_min(o.fit_old, P);
        if (c->track_stats) {
            if (order == DEAC_ORACLE_GPU_ORDER) {
                if (stats_mean) stats_mean[ii] = stat_tree(&o, o.fit_old, 0);
                if (stats_squared_mean) stats_squared_mean[ii] = stat_tree(&o, o.fit_old, 1);
            } else {
                if (stats_mean) stats_mean[ii] = seq_mean(o.fit_old, P);
                if (stats_squared_mean) stats_squared_mean[ii] = seq_squared_mean(o.fit_old, P);
            }
            if (stats_minimum) stats_minimum[ii] = minimum_fitness;
        }
        if (minimum_fitness <= c->stop_minimum_fitness) break;

        if (counter) trials_gpu_counter(&o, ii);
        else if (order == DEAC_ORACLE_GPU_ORDER) trials_gpu(&o);
        else trials_cpu(&o);
        for (uint64_t i = 0; i < P; i++) o.fit_new[i] = fitness_of(&o, i, o.pop_new, 0);
        if (trace && ii < trace_capacity) memcpy(trace + ii * P, o.fit_new, P * sizeof(double));
        /* greedy selection, ties accept (deac_gpu.cu:551-582, deac.cpp:1556-1571) */
        for (uint64_t i = 0; i < P; i++) {
            if (o.fit_new[i] <= o.fit_old[i]) {
                o.fit_old[i] = o.fit_new[i];
                for (int s = 0; s < S; s++) {
                    o.cr_old[s][i] = o.cr_new[s][i];
                    o.w_old[s][i] = o.w_new[s][i];
                    memcpy(o.pop_old[s] + i * M, o.pop_new[s] + i * M, M * sizeof(double));
                }
            }
        }
        executed++;
    }

    /* argmin_and_min: first index of the strict minimum (deac.cpp:146-158) */
    uint64_t best = 0;
    double fmin = o.fit_old[0];
    for (uint64_t i = 0; i < P; i++)
        if (o.fit_old[i] < fmin) {
            fmin = o.fit_old[i];
            best = i;
        }
    minimum_fitness = fmin;
    const uint64_t spec_len = S == 2 ? 2 * M - 1 : M;
    if (best_dsf && best_frequency) transform(&o, best, best_dsf, best_frequency);
    else if (best_dsf || best_frequency) {
        double* tmp_d = calloc(spec_len, sizeof(double));
        double* tmp_f = calloc(spec_len, sizeof(double));
        if (!tmp_d || !tmp_f) { free(tmp_d); free(tmp_f); goto fail; }
        transform(&o, best, tmp_d, tmp_f);
        if (best_dsf) memcpy(best_dsf, tmp_d, spec_len * sizeof(double));
        if (best_frequency) memcpy(best_frequency, tmp_f, spec_len * sizeof(double));
        free(tmp_d);
        free(tmp_f);
    }
    /* deac.cpp:1677-1685: when the loop ran out, report N-1 and fill the
     * last stats entry on the host with the sequential mean */
    if (generation == o.N - 2) {
        generation += 1;
        if (c->track_stats) {
            if (stats_mean) stats_mean[generation] = seq_mean(o.fit_old, P);
            if (stats_minimum) stats_minimum[generation] = minimum_fitness;
            if (stats_squared_mean) stats_squared_mean[generation] = seq_squared_mean(o.fit_old, P);
        }
    }
    if (out) {
        out->generation = generation;
        out->minimum_fitness = minimum_fitness;
        out->best_index = best;
        out->spectrum_length = spec_len;
        out->stats_length = c->track_stats ? generation + 1 : 0;
        out->generations_executed = executed;
    }
    if (population)
        for (int s = 0; s < S; s++) memcpy(population + (uint64_t)s * P * M, o.pop_old[s], P * M * sizeof(double));
    if (fitness) memcpy(fitness, o.fit_old, P * sizeof(double));
    oracle_free(&o);
    return 0;
fail:
    oracle_free(&o);
    return -1;
}
