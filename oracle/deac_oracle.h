/*
 * deac_oracle.h -- CPU oracle of the DEAC per-generation loop.
 *
 * TEST INFRASTRUCTURE.  Only tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline leg may load this code, and only as the checker or the timed
 * CPU baseline; the product (deac-cpp_gb300/) never calls it.
 */
#ifndef DEAC_ORACLE_H
#define DEAC_ORACLE_H

#include <stdint.h>
#include "deac_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Draw order and arithmetic order to follow.
 *  GPU: the reference's CUDA path (deac.cpp USE_GPU branches + deac_gpu.cu),
 *       with its two defects removed (see deac_oracle.c header).
 *  CPU: the reference's CPU path (deac.cpp #else branches), including its
 *       CPU-only formulas, so it can be compared with the reference CPU build. */
#define DEAC_ORACLE_GPU_ORDER 0
#define DEAC_ORACLE_CPU_ORDER 1
/* GPU order with the engine's counter streams (DEAC_STREAMS_COUNTER) in place
 * of the per-gene state table: the batched forms' draw layout. */
#define DEAC_ORACLE_GPU_ORDER_COUNTER 2

typedef struct deac_oracle_out {
    uint64_t generation;
    double minimum_fitness;
    uint64_t best_index;
    uint64_t spectrum_length;
    uint64_t stats_length;
    uint64_t generations_executed; /* loop iterations that reached selection */
} deac_oracle_out;

/* Run one reconstruction.  Output pointers may be NULL.
 *  best_dsf/best_frequency: spectrum_length doubles
 *  stats_*: number_of_generations doubles (stats_length are written)
 *  population: S*P*M doubles [side][member][gene] (final parents)
 *  fitness: P doubles (final parent fitness)
 *  trace_trial_fitness: trace_capacity*P doubles, trial fitness per
 *      executed generation (row g = generation g).
 * Returns 0, or -1 on an invalid configuration / allocation failure. */
int deac_oracle_run(const deac_config* cfg, int32_t order,
                    const double* imaginary_time, const double* isf,
                    const double* isf_error, uint64_t number_of_timeslices,
                    const double* frequency, uint64_t genome_size,
                    deac_oracle_out* out, double* best_dsf,
                    double* best_frequency, double* stats_mean,
                    double* stats_minimum, double* stats_squared_mean,
                    double* population, double* fitness,
                    double* trace_trial_fitness, uint64_t trace_capacity);

/* Kernel matrix rows as the reference builds them (deac.cpp:310-401):
 * k_pos/k_neg are [number_of_timeslices][genome_size]; k_neg may be NULL for
 * the one-sided genome. */
int deac_oracle_kernel_matrix(const deac_config* cfg,
                              const double* imaginary_time,
                              uint64_t number_of_timeslices,
                              const double* frequency, uint64_t genome_size,
                              double* k_pos, double* k_neg);

/* xoshiro256+ helpers (rng.hpp): state after xoshiro256p_init(seed), the
 * next output, and the 2^128 jump. */
void deac_oracle_rng_init(uint64_t seed, uint64_t state[4]);
uint64_t deac_oracle_rng_next(uint64_t state[4]);
void deac_oracle_rng_jump(uint64_t state[4]);

/* Counter streams: output `pos` of the SplitMix64 stream whose state starts
 * at key, and a run's two keys (crossover, jDE) from its seed. */
uint64_t deac_oracle_stream_draw(uint64_t key, uint64_t pos);
void deac_oracle_stream_keys(uint64_t seed, uint64_t keys[2]);

#ifdef __cplusplus
}
#endif

#endif
