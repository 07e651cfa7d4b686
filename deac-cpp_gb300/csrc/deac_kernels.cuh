// deac_kernels.cuh -- device data layout and kernels of the plain FP64
// engine.  One generation of every run in a batch is two launches:
//
//   trial_kernel     one CTA per (run, member): jDE self-adaptation of CR and
//                    F, mutant indices, per-gene crossover draws, DE/rand/1
//                    mutation with fabs, zero-frequency matching, and the
//                    normalisation / moment row sums of the new trial.
//                    Replaces gpu_set_crossover_probabilities_new,
//                    gpu_set_differential_weights_new, gpu_set_mutant_indices,
//                    gpu_set_mutate_indices, gpu_set_population_new,
//                    gpu_match_population_zero, gpu_deac_gemv and
//                    gpu_deac_dgmmDiv1D (deac_gpu.cu:345-374, 406-415,
//                    514-549, 584-643).
//   contract_kernel  one CTA per (run, member tile, tau tile): the
//                    population x K contraction as order-exact FP64 FMA
//                    chains; the last CTA of each run then forms chi^2 with
//                    the reference's reduction tree, adds the moment terms,
//                    does greedy selection by swapping the member's buffer
//                    index, records statistics and sets the run's stop flag.
//                    Replaces gpu_matmul, gpu_deac_reduced_chi_squared,
//                    gpu_deac_add_scalar_reduced_chi_squared,
//                    gpu_set_rejection_indices, gpu_swap_control_parameters,
//                    gpu_swap_populations, gpu_get_minimum and
//                    gpu_set_fitness_(squared_)mean (deac_gpu.cu:277-315,
//                    376-404, 417-512, 551-582).
//
// Arithmetic is FP64 in the reference's order; the file is compiled with
// --fmad=false and every fused multiply-add of the reference is an explicit
// fma().  The selection step never copies a genome: each member owns two
// buffers and an index saying which one holds its parent.
#pragma once

#include <cstdint>

namespace deac {

enum : uint32_t {
    kNormalize = 1u << 0,
    kFirstMoment = 1u << 1,
    kThirdMoment = 1u << 2,
    kNegativeFirstMoment = 1u << 3,
    kSignedWeights = 1u << 4,
    kTrackStats = 1u << 5,
    kTrace = 1u << 6,
    kDeferNorm = 1u << 7,  // split engine: normalisation applied after the decisions
    kNonNegProducts = 1u << 8,  // every gene x kernel product is >= 0 (unsigned genes, K >= 0)
    kCounterStreams = 1u << 9,  // draws from counter streams (deac_rng.cuh), not the per-gene state table
    kFirstMomentCpu = 1u << 10,  // the first-moment term of the reference's CPU build, (m_i - m)^2 / m
};

// Per-run descriptor, resident in device memory.
struct RunDev {
    uint32_t P, M, Nt, S;
    uint32_t flags;
    uint32_t contract_ctas;  // CTAs of contract_kernel for this run
    uint32_t member_tile;    // members per contract CTA (power of two)
    uint32_t tau_tile;       // timeslices per contract CTA
    uint32_t chunk;          // genes per shared-memory stage of contract_kernel
    uint64_t N;              // number_of_generations
    double tau_cr, tau_f;    // self-adaptation probabilities
    uint64_t p_magic;        // floor((2^64 - 1) / P): x % P without a 64-bit division
    uint64_t tau_cr_thr, tau_f_thr;  // ceil(tau 2^53): draw < tau as an integer test
    double alpha;            // 1 / F(0), the normalisation scale
    double stop;             // stop_minimum_fitness
    double first_target, third_target, third_error;
    double negfirst_target, negfirst_error;
    const double* k_pos;     // [Nt][M]
    const double* k_neg;     // [Nt][M] (two-sided)
    const double* isf;       // [Nt]
    const double* err;       // [Nt]
    const double* tau_w;     // [Nt] negative-first-moment weights
    const double* norm_pos;  // [M]
    const double* norm_neg;
    const double* first_pos;
    const double* first_neg;
    const double* third_pos;
    const double* third_neg;
    double* pop;             // [2 buffers][S][P][M]
    uint8_t* cur;            // [P] buffer holding each member's parent
    uint64_t* rng;           // 4 words x n_states, word-major
    uint64_t n_states;       // P * (1 + S*M); P with counter streams (a jDE step count per member)
    uint64_t key_crossover;  // counter streams: the keys of the run's crossover and jDE streams
    uint64_t key_jde;
    double* cr;              // [old|new][S][P]
    double* fw;              // [old|new][S][P]
    double* fit_old;         // [P]
    double* fit_new;         // [P]
    double* model_isf;       // [P][Nt]
    double* model_isf2;      // [P][Nt] kModeRecheck: the trials' (model_isf holds the parents')
    double* moments;         // [P][2]: first, third (of the trials, in the split engine)
    double* pmoments;        // split engine: [P][2] of the parents (null in the plain engine)
    double* stats;           // [mean|minimum|squared mean][N]
    double* trace;           // [trace_cap][P]
    uint64_t trace_cap;
    // split engine only (null otherwise): see deac_split.cuh
    uint8_t* changed;        // [P] trial differs from its parent
    const uint8_t* recheck;  // [P] decision left to the exact FP64 value
    double* f_lo;            // [P] interval holding the parent's exact fitness
    double* f_hi;
    uint16_t* xdig;          // digit planes of the trials of the runs sharing K (deac_split.cuh)
    uint64_t xdig_unit;      // elements between units of 8 genes
    uint64_t xdig_side;      // elements between the sides
    uint32_t xdig_row0;      // row of member 0 among the group's rows
    int16_t* xexp;           // [P][M/32] their chunk scale exponents
    int32_t* xexp_max;       // [P] their maximum (raised per part, reset after the decisions)
    uint32_t* mutants;       // [P][3] mutant indices of this generation
    // split engine with --normalize (kDeferNorm): the trials stay raw until
    // the decisions; norm_kernel forms each trial's exact reciprocal norm
    double* recip;           // [P] 1/norm of each trial
    // split engine: the batch's list of exact-pass items (shared by all
    // runs; see exact_pass_kernel) and its length
    uint64_t* exact_list;
    uint32_t* exact_count;
    // split engine: the final exact evaluations (final_list_kernel) -- the
    // parents to evaluate, ascending, and the tiling of their contraction
    uint32_t* final_members;  // [P]
    uint32_t final_n, final_mt, final_tt, final_chunk, final_ctas;
    // status, owned by the kernels
    uint64_t ii;             // next generation index to execute
    uint64_t generation;     // generation reported when done
    uint32_t ticket;         // CTAs of contract_kernel done this launch
    int32_t done;
    int32_t exact_idle;      // split engine: this generation needs no exact pass
                             // (set by split_select_kernel, which then also did
                             // the generation's bookkeeping)
};

// Per-member PRNG slot layout.  The reference keeps one state per
// (member, gene, side) plus P extra states, in the order
//   state i                       CR(+) and mutant indices of member i
//   state P + s*P*M + j*P + i     crossover draw of gene j, side s, member i
// (deac.cpp:1116-1126, 1170-1174, 1219-1222).  Here member i owns the
// contiguous slots  base(i) + q,  base(i) = i*(1+S*M):
//   q = 0            reference state i
//   q = 1 + s*M + j  reference state P + s*P*M + j*P + i
// The jDE kernels of the reference use states P+i, 2P+i, 3P+i for F(+),
// CR(-), F(-); they are member i's slots q = 1, 2, 3.
__host__ __device__ inline uint64_t rng_slot(uint32_t P, uint32_t M, uint32_t S, uint64_t ref_state) {
    if (ref_state < P) return ref_state * (1ull + (uint64_t)S * M);
    const uint64_t m = ref_state - P;
    const uint64_t pm = (uint64_t)P * M;
    const uint64_t s = m / pm, rem = m % pm;
    const uint64_t j = rem / P, i = rem % P;
    return i * (1ull + (uint64_t)S * M) + 1 + s * M + j;
}

// contract_kernel: 128 threads (4 warps), one FMA chain per thread.
// Two-sided runs put the positive-side chain of a (member, timeslice) pair in
// lane l and the negative-side chain in lane l+16 of the same warp, so a CTA
// covers 64 pairs; one-sided runs cover 128.  Each SM sub-partition retires
// one FP64 warp-instruction per ~64 cycles, and a second CTA on the same SM
// lands its warps on the same sub-partitions, doubling the cost of a chain
// step.  The host therefore requests enough shared memory to keep one CTA
// per SM: 4 warps, one per sub-partition, ~80 cycles per dependent step.
constexpr int kContractThreads = 128;
constexpr uint32_t kContractMinSmemBytes = 116 * 1024;  // > half of an SM's 228 KB
__host__ __device__ inline uint32_t contract_pairs(uint32_t S) { return S == 2 ? 64u : 128u; }
// shared-memory row stride of a staged chunk (even, so rows stay 16-byte
// aligned; the 2-double pad spreads rows over the banks)
__host__ __device__ inline uint32_t stage_stride(uint32_t chunk) { return chunk + 2; }
__host__ __device__ inline uint64_t stage_doubles(uint32_t S, uint32_t mt, uint32_t tt, uint32_t chunk) {
    return (uint64_t)S * (mt + tt) * stage_stride(chunk);
}

constexpr int kTrialThreads = 512;
// row-sum chains of trial_kernel: a group of 8 warps per side, 16 steps per
// thread in a round (2048 steps)
constexpr int kChainWarps = 8;
constexpr int kChainSteps = 8;

struct Work {
    uint32_t run;
    uint32_t index;  // member (trial) or tile (contract)
};

// contract_kernel modes
enum ContractMode : int {
    kModeGeneration = 0,  // trials of every member, selection, next-generation bookkeeping
    kModeInit = 1,        // fitness of the initial population, bookkeeping of generation 0
    kModeParents = 2,     // split engine: exact fitness of undecided members' inexact parents
    kModeTrials = 3,      // split engine: exact fitness and selection of undecided trials, bookkeeping
    kModeFinal = 4,       // split engine: exact fitness of every inexact parent (finished runs too)
    kModeFinalBest = 6,   // split engine: the same for the parents that may hold the minimum (an
                          // interval reaching below every other parent's upper end)
    kModeRecheck = 5,     // split engine (exact_pass_kernel): kModeParents and kModeTrials items
                          // of a run, one CTA finishing both
};

// Programmatic dependent launch: a kernel launched with the programmatic
// stream-serialisation attribute may be scheduled while its predecessor on
// the stream still runs.  Every generation kernel calls this first: it blocks
// until the predecessor grid has completed with its memory visible, then
// lets the next grid be scheduled (which waits here in turn, so at most two
// grids overlap).  Without the attribute both instructions return at once.
__device__ __forceinline__ void grid_dependency_wait() {
    asm volatile("griddepcontrol.wait;\n" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory");
}

// Integer form of the crossover test  (x >> 11) * 2^-53 < cr
// (deac_gpu.cu:641): with m = x >> 11 < 2^53 and X = cr * 2^53 (exact),
// m < X  <=>  m < ceil(X).  Keeps the FP64 pipe free for the row-sum chain.
__device__ __forceinline__ uint64_t crossover_threshold(double cr) {
    if (!(cr > 0.0)) return 0;
    if (cr >= 1.0) return 1ull << 53;
    return (uint64_t)ceil(cr * 0x1.0p53);
}

// |v|: v with its sign bit cleared by an integer AND on the high word.  The
// AND is inline PTX so that the compiler cannot turn it back into an FP64
// absolute value, which GB300 runs on its narrow FP64 pipe.
__device__ __forceinline__ double abs_bits(double v) {
    uint32_t hi = (uint32_t)__double2hiint(v);
    asm("and.b32 %0, %0, 0x7FFFFFFF;" : "+r"(hi));
    return __hiloint2double((int)hi, __double2loint(v));
}

// The DE/rand/1 mutation v = a + F (b - c) (one rounding for b - c, one for
// the fused multiply-add: deac_gpu.cu:514-539) in lanes where `mutate` holds;
// v keeps its value elsewhere.  Predicated in PTX so that the FP64 pipe (a
// narrow one on GB300) sees only the mutating lanes of a warp, where the
// compiler would compute every lane and select.
__device__ __forceinline__ void mutate_gene(double& v, double a, double b, double c, double fw, bool mutate) {
    asm("{\n\t.reg .pred p;\n\tsetp.ne.u32 p, %4, 0;\n\t@p sub.rn.f64 %0, %2, %3;\n\t"
        "@p fma.rn.f64 %0, %5, %0, %1;\n\t}"
        : "+d"(v)
        : "d"(a), "d"(b), "d"(c), "r"((uint32_t)mutate), "d"(fw));
}

// Asynchronous L2 prefetch of the `count` elements at p, rounded out to the
// 16-byte units a bulk copy addresses and clipped at `end` (one past the
// buffer's last element), so that it never reaches beyond the buffer.
template <typename T>
__device__ __forceinline__ void prefetch_l2(const T* p, uint64_t count, const T* end) {
    const uint64_t a = reinterpret_cast<uint64_t>(p) & ~15ull;
    uint64_t e = (reinterpret_cast<uint64_t>(p + count) + 15u) & ~15ull;
    const uint64_t lim = reinterpret_cast<uint64_t>(end) & ~15ull;
    if (e > lim) e = lim;
    if (e > a)
        asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(a), "r"((uint32_t)(e - a)) : "memory");
}

__global__ void trial_kernel(RunDev* runs, const Work* work, int init_mode, int smem_doubles);
// The result snapshot of n runs packed into one buffer: the RunDev
// descriptors (as 8-byte words), then every run's parent fitness (offsets
// fit_off), then their parent buffers (same offsets), then (8-byte aligned)
// the genes of each run's best parent, both sides (offsets gene_off, in
// doubles), for one copy to the host.
__global__ void snapshot_kernel(const RunDev* runs, uint32_t n, const uint32_t* fit_off, const uint64_t* gene_off,
                                uint64_t* out);
// the PRNG table of a run: state k = J^k s for the generator state s after
// the initial draws, from the matrices J^(2^b) (jpow, 1024 words each), into
// slot rng_slot(P, M, S, k) of the word-major table of n states
__global__ void rng_table_kernel(uint64_t* rng, uint64_t n, const uint64_t* jpow, uint32_t bits, uint64_t s0,
                                 uint64_t s1, uint64_t s2, uint64_t s3, uint32_t P, uint32_t M, uint32_t S);
// split engine: jDE of every member (one thread each) after the initial
// population; each generation's raw trials in parts of kTrialPart genes per
// side, each with its BF16 digit slices, up to kPartsPerCta consecutive
// parts of one member per CTA
constexpr uint32_t kTrialPart = 512;
constexpr uint32_t kPartsPerCta = 4;
constexpr int kTrialPartThreads = 128;
struct PartWork {
    uint32_t run, member, part0, nparts;
};
__global__ void jde_kernel(RunDev* runs, const Work* work, uint32_t n);
__global__ void trial_part_kernel(RunDev* runs, const PartWork* work);
// the same for batches that draw from counter streams
__global__ void trial_part_counter_kernel(RunDev* runs, const PartWork* work);
// The initial populations (deac.cpp:418-458), each into its run's parent
// buffer 0: the stream seeded with 1407513600 + seed, member-major, a draw
// per side per gene, U[0,1) (-0.5 with signed weights), then each member's
// negative-side gene 0 := its positive-side gene 0.  Thread t makes draws
// [t 2^block_log2, (t+1) 2^block_log2) from the state J^(t 2^block_log2) s0,
// J the generator's step as a GF(2)-linear map (jstep: the matrices
// J^(2^b), 1024 words each).
constexpr uint32_t kPopBlockLog2 = 10;
constexpr int kPopThreads = 128;
struct PopRun {
    double* pop;          // the run's parent buffer 0
    uint64_t s[4];        // its stream's seeded state
    uint32_t P, M, S, signed_weights;
};
struct PopWork {
    uint32_t run;         // index into the PopRun list
    uint32_t t0;          // the CTA's first thread within the run
};
// one CTA (kPopThreads) per entry of `work`, every run of the batch in one launch
__global__ void population_kernel(const PopRun* runs, const PopWork* work, const uint64_t* jstep);
// split engine, generation 0: the BF16 digit slices of every member's
// initial parent (the trial planes' rows), parts as trial_part_kernel's
__global__ void parent_digits_kernel(RunDev* runs, const PartWork* work);
// split engine, runs that normalise (kDeferNorm) or have moment terms: the
// exact normalisation row sums of one raw trial per CTA (both sides), the
// reciprocal norm and the final `changed` flag, then its moment row sums
constexpr int kNormThreads = 2 * kChainWarps * 32;
constexpr uint32_t kNormStage = kChainWarps * 32 * kChainSteps;  // steps staged in shared memory at a time
constexpr uint32_t kNormSmemBytes = 2 * 2 * kNormStage * sizeof(double);  // dynamic shared memory of norm_kernel
__global__ void norm_kernel(RunDev* runs, const Work* work);
__global__ void contract_kernel(RunDev* runs, const Work* work, int mode);
// split engine: the exact pass over the items split_select_kernel listed
// (entry = run << 32 | pass << 31 | tile, pass 1 = the trials; count entries)
__global__ void exact_pass_kernel(RunDev* runs, const uint64_t* list, const uint32_t* count);
// The split engine's final exact evaluations (kModeFinal / kModeFinalBest):
// final_list_kernel (one warp per run) lists the parents to evaluate and
// appends the tiles of their contraction to `items` (run << 32 | tile);
// final_exact_kernel evaluates the listed tiles, packed so that every chain
// pair of a tile belongs to a listed parent.
constexpr uint32_t kFinalSmemBytes = 96 * 1024;
// The tiling of n listed members: mt members (a power of two, at least
// min_mt) times tt timeslices fill the CTA's chain pairs.  Few members in few
// tiles suit a batch-wide pass, where the FP64 pipe (charged per warp
// instruction) is the limit; the exact pass of a generation is bound by the
// latency of its chains instead, and takes min_mt = 8: fewer staged rows,
// longer stages, fewer stage waits along each chain.
__host__ __device__ inline void final_tiling(uint32_t n, uint32_t S, uint32_t Nt, uint32_t& mt, uint32_t& tt,
                                             uint32_t& chunk, uint32_t& ctas, uint32_t min_mt = 1) {
    const uint32_t pairs = contract_pairs(S);
    mt = 1;
    while (mt * 2 <= (n < pairs ? n : pairs)) mt *= 2;
    while (mt < min_mt && mt * 2 <= pairs) mt *= 2;
    tt = pairs / mt;
    const uint32_t rows = S * (mt + tt);
    uint32_t c = (kFinalSmemBytes / 8) / (2 * rows) - 2;
    c = (c < 128 ? c : 128) & ~1u;
    chunk = c > 8 ? c : 8;
    ctas = ((n + mt - 1) / mt) * ((Nt + tt - 1) / tt);
}
__global__ void final_list_kernel(RunDev* runs, int mode, uint64_t* items, uint32_t* count, uint32_t capacity,
                                  int* status);
__global__ void final_exact_kernel(RunDev* runs, const uint64_t* items, const uint32_t* count, int mode);
// members per packed tile of the exact pass, at least
constexpr uint32_t kExactMinMembers = 8;
// status value of a final item list that would have overflowed
constexpr int kStatusFinalList = 3;

}  // namespace deac
