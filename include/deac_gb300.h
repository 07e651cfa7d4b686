/*
 * deac_gb300.h -- C-ABI of the GB300-native DEAC engine.
 *
 * DEAC (differential evolution for analytic continuation) reconstructs a
 * spectrum S(omega) from imaginary-time correlation data F(tau) +- sigma(tau)
 * by self-adaptive differential evolution (jDE) over a population of
 * discretised spectra ("genomes").
 *
 * This header is the drop-in boundary for the per-generation loop of
 * nscottnichols/deac-cpp.  In the reference that loop is the C++ function
 *     void deac(xoshiro256p_state*, double* imaginary_time, double* isf,
 *               double* isf_error, double* frequency, ... 27 arguments)
 * (src/deac/src/deac.cpp:218-229), which drives 19 C++-linkage launchers
 * `gpu_*(cudaStream_t, ...)` (src/deac/include/deac_gpu.cuh:6-27).  The
 * reference selects the spectral model, zero temperature, the one-sided
 * (bosonic) genome and signed weights at compile time
 * (src/deac/CMakeLists.txt:18-35, 98-109, 227-232); here they are fields of
 * `deac_config`, so one library serves every variant.
 *
 * Conventions
 *  - plain C types only; every function returns 0 on success or a negative
 *    DEAC_E_* code, with a message available from deac_last_error()
 *    (the reference asserts on CUDA return codes instead, common_gpu.hpp:51);
 *  - host arrays are caller owned and only read/written during the call;
 *  - a batch owns its device memory; kernels run on the stream given to
 *    deac_batch_create (NULL = the legacy default stream);
 *  - one host thread per batch.
 */
#ifndef DEAC_GB300_H
#define DEAC_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- error codes ------------------------------------------------------- */
#define DEAC_OK 0
#define DEAC_E_INVALID (-1)   /* bad argument or configuration */
#define DEAC_E_CUDA (-2)      /* a CUDA runtime call failed */
#define DEAC_E_NOMEM (-3)     /* host or device allocation failed */
#define DEAC_E_STATE (-4)     /* call out of order (e.g. run before setup) */
#define DEAC_E_NODEVICE (-5)  /* no usable sm_103 device */

/* ---- variants ---------------------------------------------------------- */
/* DEAC_MODEL (src/deac/CMakeLists.txt:98-109) */
#define DEAC_MODEL_STANDARD 0
#define DEAC_MODEL_HYPERBOLIC 1
#define DEAC_MODEL_NORMALIZATION 2

/* --spectra_type (deac.cpp:2016-2023, 2040-2058).  BDSF is the only type of
 * the one-sided (bosonic) genome; the other four are two-sided. */
#define DEAC_SPECTRA_SPBSF 0
#define DEAC_SPECTRA_SPFSF 1
#define DEAC_SPECTRA_BFULL 2
#define DEAC_SPECTRA_FFULL 3
#define DEAC_SPECTRA_BDSF 4

/* Evaluation engines of a batch.
 *  PLAIN_FP64: every step in FP64 in the order of the reference CUDA path;
 *              bit-identical to the reference semantics (the default).
 *  SPLIT_BF16: the contraction of each trial is first evaluated on the
 *              tcgen05 tensor cores from exact BF16 digit slices, with a
 *              rigorous bound on its distance from the FP64 value; only
 *              decisions that bound leaves open are settled by the FP64
 *              chains.  Selection, generation count, minimum fitness and
 *              spectrum are identical to PLAIN_FP64.  Needs genome_size a
 *              multiple of 32.  First and third moment terms enter the
 *              interval decisions exactly; runs with the negative first
 *              moment or statistics are decided by the FP64 chains. */
#define DEAC_ENGINE_PLAIN_FP64 0
#define DEAC_ENGINE_SPLIT_BF16 1

/* Draw layouts of a batch (deac_batch_set_streams).
 *  REFERENCE: the reference's per-gene xoshiro256+ state table (deac.cpp:
 *             1114-1135): 2 S P (M+1) states of 32 bytes, each read and
 *             written by every draw; bit-identical to the reference's draws
 *             (the default).
 *  COUNTER:   the batched forms' compact layout: every per-generation draw
 *             is the SplitMix64 output at a position computed from
 *             (generation, member, side, gene), keyed by the run's seed; one
 *             8-byte jDE step count per member replaces the table.  Draws
 *             are statistically equivalent (uniform, independent positions of
 *             one stream) but not the reference's values; both engines draw
 *             the same values, so PLAIN_FP64 and SPLIT_BF16 still agree bit
 *             for bit.  The initial population is drawn as in REFERENCE. */
#define DEAC_STREAMS_REFERENCE 0
#define DEAC_STREAMS_COUNTER 1

/* The first-moment term of the fitness differs between the reference's
 * builds: the GPU build adds ((m - m_i) / 1.0)^2 (deac.cpp:623, 949;
 * deac_gpu.cu:450-456), the CPU build (m_i - m)^2 / m (deac.cpp:969). */
#define DEAC_FIRST_MOMENT_GPU 0
#define DEAC_FIRST_MOMENT_CPU 1

/* Everything the reference reads from its command line (deac.cpp:1926-2024)
 * plus the compile-time variant switches. */
typedef struct deac_config {
    int32_t model;                 /* DEAC_MODEL_* */
    int32_t zero_temperature;      /* ZeroT build type: K = df*exp(-tau*omega) */
    int32_t bosonic;               /* one-sided genome (detailed balance) */
    int32_t allow_negative_weight; /* no fabs() in the mutation */
    int32_t spectra_type;          /* DEAC_SPECTRA_* */
    int32_t normalize;             /* --normalize */
    int32_t use_negative_first_moment; /* --use_negative_first_moment */
    int32_t track_stats;           /* --track_stats */
    double temperature;            /* -T */
    double first_moment;           /* --first_moment (<0: unused) */
    double third_moment;           /* --third_moment (<0: unused) */
    double third_moment_error;     /* --third_moment_error */
    double crossover_probability;  /* -r, initial CR */
    double self_adapting_crossover_probability;           /* -u, tau_CR */
    double differential_weight;                           /* -F, initial F */
    double self_adapting_differential_weight_probability; /* -v, tau_F */
    double self_adapting_differential_weight_shift;       /* -l, accepted and unused, as in the reference */
    double self_adapting_differential_weight;             /* -m, accepted and unused, as in the reference */
    double stop_minimum_fitness;   /* --stop_minimum_fitness */
    uint64_t number_of_generations; /* -N */
    uint64_t population_size;       /* -P */
    uint64_t seed;                  /* --seed; the PRNG is seeded with 1407513600 + seed */
    int32_t first_moment_formula;   /* DEAC_FIRST_MOMENT_GPU (default) or DEAC_FIRST_MOMENT_CPU */
} deac_config;

/* Result of one run, as the reference reports it (deac.cpp:1592, 1677-1685,
 * 1760-1763). */
typedef struct deac_run_result {
    uint64_t generation;      /* the `generation:` value of the log */
    double minimum_fitness;   /* the `minimum_fitness:` value */
    uint64_t best_index;      /* first member with the minimum fitness */
    uint64_t spectrum_length; /* 2M-1 (two-sided) or M (one-sided) */
    uint64_t stats_length;    /* generation+1 when track_stats, else 0 */
    uint64_t population_size;
    uint64_t genome_size;
    uint64_t number_of_timeslices;
    int32_t sides;            /* 2 two-sided, 1 one-sided */
    int32_t finished;         /* 1 once the run stopped or used all generations */
} deac_run_result;

/* Fill `cfg` with the reference command-line defaults (deac.cpp:1927-2024):
 * T=0, N=100000, P=512, CR=0.9, tau_CR=0.1, F=0.9, tau_F=0.1, stop=1.0,
 * seed=0, standard model, two-sided, spectra_type spfsf. */
void deac_config_default(deac_config* cfg);

/* Validate a configuration against the checks the reference applies before
 * calling deac() (deac.cpp:2093-2106, 2143-2153) and the variant rules
 * (e.g. zero temperature needs the one-sided genome, as in the reference
 * where the two-sided ZeroT build does not compile).  Returns DEAC_OK or
 * DEAC_E_INVALID with the reference's message in deac_last_error(). */
int deac_config_check(const deac_config* cfg);

/* Message for the last failing call on this thread. */
const char* deac_last_error(void);

/* ---- batch engine: the deac() loop for one or many independent runs ----- */
typedef struct deac_batch deac_batch;

/* Create an empty batch on `device` that launches on `cuda_stream`
 * (a cudaStream_t; NULL for the default stream).  Replaces the stream and
 * buffer set-up of deac.cpp:256-301. */
int deac_batch_create(int device, void* cuda_stream, int32_t engine, deac_batch** out);

/* Add one run: the configuration plus the arrays main() hands to deac()
 * (deac.cpp:2184-2192): tau, F(tau), sigma(tau) of length
 * number_of_timeslices, and the frequency grid of length genome_size.
 * Writes the run's index to *run_index. */
int deac_batch_add_run(deac_batch* b, const deac_config* cfg,
                       const double* imaginary_time, const double* isf,
                       const double* isf_error, uint64_t number_of_timeslices,
                       const double* frequency, uint64_t genome_size,
                       uint32_t* run_index);

/* Build the kernel matrices and moment terms (deac.cpp:310-401, 478-827),
 * draw the initial populations and the per-gene PRNG state tables
 * (deac.cpp:418-458, 1114-1135), upload everything and evaluate the initial
 * fitness (deac.cpp:829-976).  Synchronous. */
int deac_batch_setup(deac_batch* b);

/* Enqueue `generations` generations of every unfinished run on the batch
 * stream and return without waiting (whole blocks of 16 as a captured CUDA
 * graph, the rest launched directly).  Runs that reach their stop fitness or
 * their generation limit stop on the device. */
int deac_batch_launch(deac_batch* b, uint64_t generations);

/* Wait for the stream, then report how many runs have finished. */
int deac_batch_sync(deac_batch* b, uint32_t* runs_finished);

/* setup (if not done) + launch/sync until every run has finished. */
int deac_batch_run(deac_batch* b);

/* Number of runs in the batch. */
int deac_batch_size(const deac_batch* b, uint32_t* runs);

/* Summary of run `run` (valid once it finished). */
int deac_batch_result(deac_batch* b, uint32_t run, deac_run_result* out);

/* Outputs of run `run`, as the reference writes them (deac.cpp:1594-1717):
 * best_dsf and best_frequency of spectrum_length doubles; the three stats
 * arrays of stats_length doubles (only with track_stats).  Any pointer may
 * be NULL. */
int deac_batch_fetch(deac_batch* b, uint32_t run, double* best_dsf,
                     double* best_frequency, double* stats_mean,
                     double* stats_minimum, double* stats_squared_mean);

/* Every run's summary and best spectrum in one call (the batch form of
 * deac_batch_result + deac_batch_fetch): results[r] for each run r, and the
 * spectra concatenated in run order -- run r's best_dsf and best_frequency
 * start at the sum of spectrum_length over the runs before it (size the
 * arrays with deac_batch_spectra_length).  The spectra are formed on host
 * threads.  Either array may be NULL. */
int deac_batch_fetch_all(deac_batch* b, deac_run_result* results, double* best_dsf,
                         double* best_frequency);
int deac_batch_spectra_length(deac_batch* b, uint64_t* doubles);

/* Current state of run `run`: population [side][member][gene] (S*P*M
 * doubles), fitness (P), crossover rates and differential weights
 * ([side][member], S*P each).  Any pointer may be NULL. */
int deac_batch_fetch_state(deac_batch* b, uint32_t run, double* population,
                           double* fitness, double* crossover_rates,
                           double* differential_weights);

/* Checkpoint of run `run` (after setup): the state the reference's
 * --save_state names (deac.cpp:2004-2007, declared there but never written)
 * -- the PRNG states, both parent buffers, fitness, crossover rates and
 * differential weights -- plus the generation counters, statistics and
 * trace, as one byte block.  A split-engine batch first makes every parent's
 * fitness exact and also saves the next generation's mutant indices and its
 * decision counts (its next jDE step is drawn when a selection becomes
 * final, a generation ahead of the plain engine).  With out == NULL only
 * *bytes (its size) is set; otherwise the block is written to out (capacity
 * bytes at least). */
int deac_batch_checkpoint(deac_batch* b, uint32_t run, void* out,
                          uint64_t capacity, uint64_t* bytes);

/* Resume from a checkpoint: after deac_batch_setup of a run added with the
 * same configuration and inputs, overwrite its state with the block, so that
 * the generations launched next continue the checkpointed run exactly (the
 * same results as a run never interrupted).  A plain-engine block restores
 * into either engine (the split engine draws the next jDE step on restore);
 * a split-engine block only into the split engine.  A block of another
 * configuration or other inputs, or with counters out of range, is refused
 * with DEAC_E_INVALID. */
int deac_batch_restore(deac_batch* b, uint32_t run, const void* in, uint64_t bytes);

/* Choose the draw layout (DEAC_STREAMS_*) of every run of the batch; before
 * deac_batch_setup.  No counterpart in the reference, which keeps one state
 * per gene (deac.cpp:1114-1135); the counter layout is what lets thousands
 * of runs at M = 16384 fit on one GPU. */
int deac_batch_set_streams(deac_batch* b, int32_t layout);

/* Record, for run `run`, the trial fitness of every member at every
 * generation up to `max_generations` (a test aid; call before setup). */
int deac_batch_enable_trace(deac_batch* b, uint32_t run, uint64_t max_generations);

/* Copy the recorded trace: trial_fitness[g*P + i] for generations
 * g < min(executed, max_generations). */
int deac_batch_fetch_trace(deac_batch* b, uint32_t run, double* trial_fitness,
                           uint64_t capacity);

/* Split engine: how the trials of run `run` were decided so far --
 * counts[0] equal to their parent (no gene changed), counts[1] settled by the
 * tensor-core estimate's interval, counts[2] settled by the exact FP64 value. */
int deac_batch_split_counts(deac_batch* b, uint32_t run, uint64_t counts[3]);

/* Launch shapes of the split engine that deac_batch_autotune chooses. */
typedef struct deac_tune_report {
    uint32_t parts_per_cta;   /* trial-part CTAs: consecutive 512-gene parts of one member */
    uint32_t split_waves;     /* tensor-core contraction: about split_waves x SMs CTAs */
    uint32_t candidates;      /* shapes timed (0: taken from this process's cache) */
    uint32_t from_cache;      /* 1 when a batch of the same mix was tuned before */
    double ms_per_generation;          /* the chosen shapes' */
    double ms_per_generation_default;  /* the default shapes' */
} deac_tune_report;

/* Choose the split engine's launch shapes for this batch's mix of runs:
 * after setup, time `generations` generations in each candidate shape (trial
 * parts per CTA 1, 2, 4, 8 x contraction CTAs 1, 2, 4 waves of the SMs) and
 * keep the fastest.  The timed generations are real generations of the runs
 * (shapes change no result, only speed).  The choice is cached per mix (run
 * sizes, sides and row sums) for the process: a later batch of the same mix
 * takes it without timing, and generations == 0 applies a cached choice
 * only.  No counterpart in the reference, whose block and stream sizes are
 * compile-time constants (src/deac/CMakeLists.txt:86-95).  The plain engine
 * has nothing to tune (report all zero). */
int deac_batch_autotune(deac_batch* b, uint64_t generations, deac_tune_report* out);

/* Bytes this batch has copied host -> device and device -> host so far
 * (set-up uploads, status reads, result and state fetches).  No counterpart
 * in the reference. */
int deac_batch_transfer_bytes(const deac_batch* b, uint64_t* host_to_device, uint64_t* device_to_host);

/* Kernel launches one generation of this batch makes (after set-up; the
 * same for every generation, whichever runs are still going).  No
 * counterpart in the reference. */
int deac_batch_generation_launches(const deac_batch* b, uint32_t* launches);

/* Device time of the kernels launched since timing was enabled, per kernel
 * kind, measured with CUDA events on the batch stream (ms): 0 trial kernel,
 * 1 contraction kernel (plain generation or the split engine's exact
 * passes), 2 normalisation row sums of the split engine's --normalize
 * runs, 3 tensor-core contraction, 4 partial-sum combine, interval decisions
 * and the normalisation of the kept trials.
 * While timing is enabled, generations are launched one by one instead of
 * as CUDA graphs. */
int deac_batch_enable_timing(deac_batch* b, int32_t enable);
int deac_batch_kernel_time(deac_batch* b, int32_t kind, double* ms, uint64_t* launches);

int deac_batch_destroy(deac_batch* b);

/* ---- one-call form of deac() ------------------------------------------- */
/* Run one reconstruction to completion and return its outputs: the drop-in
 * for deac() (deac.cpp:218-1923) minus the file writing, which the deac.e
 * front end does.  Output arrays as in deac_batch_fetch. */
int deac_reconstruct(const deac_config* cfg, const double* imaginary_time,
                     const double* isf, const double* isf_error,
                     uint64_t number_of_timeslices, const double* frequency,
                     uint64_t genome_size, deac_run_result* result,
                     double* best_dsf, double* best_frequency,
                     double* stats_mean, double* stats_minimum,
                     double* stats_squared_mean);

/* ---- fitness of a device-resident population, allocating nothing -------- */
/* No counterpart in the reference.
 *
 * For callers that cannot allocate device memory when they need fitness
 * values: a framework that reserves most of the GPU at start-up, or a pool
 * allocator that owns every buffer, makes a cudaMalloc from this library fail
 * although the caller already holds all inputs and outputs; and cudaFree
 * waits for the whole device, stalling the caller's other streams.
 *
 * Writes fitness[i] = (1/Nt) sum_t ((isf[t] - E[i,t]) / isf_error[t])^2 with
 * E = population x kernel^T (both sides), the reduced chi^2 without moment
 * terms, computed by the batch engine's contraction kernel in the same order,
 * so the values equal deac_batch_fetch_state's fitness for the same
 * population.  Every pointer is device memory of `device`:
 *   population  [sides][population_size][genome_size], 16-byte aligned;
 *   kernel_pos, kernel_neg  [number_of_timeslices][genome_size], 16-byte
 *               aligned (kernel_neg ignored when sides == 1);
 *   isf, isf_error  [number_of_timeslices];  fitness  [population_size].
 * Enqueued on `cuda_stream` (NULL: the legacy default stream); returns
 * without waiting.
 *
 * The kernel's scratch (run descriptor, work list and the population x
 * timeslice model-ISF matrix) lives in one static device array of
 * DEAC_NOALLOC_SCRATCH_BYTES that every GPU loading this library holds until
 * the process exits: population_size x number_of_timeslices x 8 bytes plus a
 * few KB must fit in it, and larger calls fail with DEAC_E_INVALID.  Every
 * call looks up the array's device address in the current context (so a
 * context made again after cudaDeviceReset is handled); the first call on a
 * device also raises the kernel's shared-memory limit, so make that first
 * call before any stream capture.  All calls on a device share the one array, which keeps the last
 * call's contents: calls that overlap on the GPU (different streams or host
 * threads) race and must be ordered by the caller. */
#define DEAC_NOALLOC_SCRATCH_BYTES (16u << 20)
int deac_population_fitness_noalloc(int device, void* cuda_stream, int32_t sides,
                                    const double* population, uint64_t population_size,
                                    uint64_t genome_size, const double* kernel_pos,
                                    const double* kernel_neg, const double* isf,
                                    const double* isf_error, uint64_t number_of_timeslices,
                                    double* fitness);

/* Library version string. */
const char* deac_version(void);

#ifdef __cplusplus
}
#endif

#endif /* DEAC_GB300_H */
