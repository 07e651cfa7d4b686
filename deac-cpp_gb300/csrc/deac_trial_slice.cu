// deac_trial_slice.cu -- the split engine's raw trials and their BF16 digit
// planes for batches that draw from counter streams (trial_slice_kernel; see
// deac_split.cuh for the item layout and deac_rng.cuh for the streams).
//
// Per gene the arithmetic is trial_kernel's: the crossover test of gene j,
// side s of member i against CR(s) of its jDE step n (deac_gpu.cu:635-643,
// drawn at ((n P + i) S + s) M + j of the run's crossover stream), and the
// DE/rand/1 mutation a + F (b - c) of the three mutant parents
// (deac_gpu.cu:514-539) with |.| unless signed weights are allowed; then
// gpu_match_population_zero (deac_gpu.cu:541-549) for two-sided runs.  The
// digit planes are digitize_trial's, by the same per-unit code.
#include <cuda_runtime.h>

#include "deac_async.cuh"
#include "deac_kernels.cuh"
#include "deac_rng.cuh"
#include "deac_split.cuh"

namespace deac {

namespace {

constexpr uint32_t kNoItem = 0xFFFFFFFFu;

// A trial gene to global memory, kept in L1 (evict-last): the warp reads its
// trial genes back at once, in the digit layout.
__device__ __forceinline__ void st_keep_l1(double* p, double v) {
    asm volatile("st.global.L1::evict_last.f64 [%0], %1;" ::"l"(p), "d"(v) : "memory");
}

// The CTA's position in its item sequence: segment g, item `it` of it.
struct SliceCursor {
    uint32_t g, it;
};

// Advance `c` to the first live item at or after it (runs that are done are
// skipped).
__device__ __forceinline__ void slice_settle(SliceCursor& c, const SliceSeg* segs, uint32_t se, const RunDev* runs) {
    while (c.g < se && (c.it >= segs[c.g].item1 || runs[segs[c.g].run].done)) {
        ++c.g;
        if (c.g < se) c.it = segs[c.g].item0;
    }
}

// What the warps need of a staged item's run: this generation's CR / F
// thresholds and weights, mutant indices, jDE step and parent buffer of
// every member, and the run's fields (written by the warp that stages the
// item, only when the stage's table is of another run).
struct SliceTable {
    uint64_t thr[2][kSliceRows];
    double fw[2][kSliceRows];
    uint64_t step[kSliceRows];
    uint8_t mut[3][kSliceRows];
    uint8_t cur[kSliceRows];
    // the run's fields the warps use (a copy of its description)
    double* pop;
    uint16_t* xdig;
    int16_t* xexp;
    uint64_t key_x, xdig_unit, xdig_side;
    uint32_t P, S, M, xdig_row0, keep_sign;
    uint32_t run, item;  // item kNoItem: the CTA's items are exhausted
};

}  // namespace

__global__ void __launch_bounds__(kSliceThreads, 1)
    trial_slice_kernel(RunDev* runs, const SliceSeg* segs, const uint32_t* seg_start, int* status) {
    extern __shared__ __align__(128) double slice_s[];  // kSliceStages stages of kSliceStageDoubles
    __shared__ __align__(8) uint64_t s_full[kSliceStages];
    __shared__ SliceTable s_tab[kSliceStages];
    __shared__ uint32_t s_done[kSliceStages];   // warps done with the stage's item
    __shared__ uint32_t s_armed[kSliceStages];  // phases of the stage armed with copies
    __shared__ SliceCursor s_next;              // the next item to stage
    __shared__ int s_fail;

    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    const uint32_t se = seg_start[blockIdx.x + 1];
    if (tid == 0) {
        for (uint32_t q = 0; q < kSliceStages; ++q) {
            mbar_init(&s_full[q], 1);
            s_done[q] = 0;
            s_armed[q] = 0;
            s_tab[q].run = kNoItem;
        }
        mbar_init_fence();
        s_fail = 0;
    }
    __syncthreads();
    grid_dependency_wait();
    // the previous generation's exact pass is done with its item list (one
    // count for the whole batch)
    if (blockIdx.x == 0 && tid == 0) *runs[0].exact_count = 0;

    // (the whole warp) stage the next item into stage st: the run's table,
    // then one bulk copy per (member, side) of the item's parent rows; a
    // table of kNoItem, without copies, once the items are exhausted
    auto stage_next = [&](uint32_t st) {
        SliceCursor c = s_next;
        SliceTable& T = s_tab[st];
        if (c.g >= se) {
            if (lane == 0) {
                T.item = kNoItem;
                mbar_arrive(&s_full[st]);
            }
            __syncwarp();
            return;
        }
        const uint32_t run = segs[c.g].run;
        if (T.run != run) {
            const RunDev& R = runs[run];
            const uint32_t P = R.P, S = R.S;
            for (uint32_t m = lane; m < P; m += 32) {
                T.cur[m] = R.cur[m];
                for (uint32_t s = 0; s < S; ++s) {
                    T.thr[s][m] = crossover_threshold(R.cr[(uint64_t)S * P + s * P + m]);
                    T.fw[s][m] = R.fw[(uint64_t)S * P + s * P + m];
                }
                for (uint32_t q = 0; q < 3; ++q) T.mut[q][m] = (uint8_t)R.mutants[3 * m + q];
                T.step[m] = R.rng[m] - 1;  // the jDE step this trial's CR / F and mutants come from
            }
            if (lane == 0) {
                T.pop = R.pop;
                T.xdig = R.xdig;
                T.xexp = R.xexp;
                T.key_x = R.key_crossover;
                T.xdig_unit = R.xdig_unit;
                T.xdig_side = R.xdig_side;
                T.P = P;
                T.S = S;
                T.M = R.M;
                T.xdig_row0 = R.xdig_row0;
                T.keep_sign = (R.flags & kSignedWeights) != 0;
                T.run = run;
            }
        }
        if (lane == 0) T.item = c.it;
        __syncwarp();
        const uint32_t P = T.P, S = T.S, M = T.M;
        const uint32_t L = slice_chunks(P, S) * kChunk;
        const uint32_t j0 = c.it * L;
        const uint32_t len = M - j0 < L ? M - j0 : L;
        const uint64_t PM = (uint64_t)P * M;
        if (lane == 0) mbar_expect_tx(&s_full[st], P * S * len * (uint32_t)sizeof(double));
        __syncwarp();
        double* dst = slice_s + (uint64_t)st * kSliceStageDoubles;
        for (uint32_t q = lane; q < P * S; q += 32) {
            const uint32_t m = q / S, s = q - m * S;
            const double* src = T.pop + ((uint64_t)T.cur[m] * S + s) * PM + (uint64_t)m * M + j0;
            bulk_load(dst + (uint64_t)q * L, src, len * (uint32_t)sizeof(double), &s_full[st]);
        }
        ++c.it;
        slice_settle(c, segs, se, runs);
        if (lane == 0) {
            s_next = c;
            ++s_armed[st];
        }
        __syncwarp();
    };

    if (warp == 0) {
        SliceCursor c{seg_start[blockIdx.x], 0};
        if (c.g < se) c.it = segs[c.g].item0;
        slice_settle(c, segs, se, runs);
        if (lane == 0) s_next = c;
        __syncwarp();
        for (uint32_t st = 0; st < kSliceStages; ++st) stage_next(st);
    }

    // this warp's bookkeeping of its members in the current run: the largest
    // chunk exponent and whether a gene mutated, per lane, raised into the
    // run's arrays when the warp leaves the run
    // the stream's Weyl increment, and this lane's multiple of it
    constexpr uint64_t kGamma = 0x9E3779B97F4A7C15ull;
    const uint64_t lane_gamma = (uint64_t)lane * kGamma;
    uint32_t run = kNoItem, P = 0, S = 1;
    int lane_max = -2000;
    bool lane_mut = false;
    auto flush = [&]() {
        if (run == kNoItem) return;
        const uint32_t LR = 8 * S;  // lanes per member
        int m = lane_max;
        bool mut = lane_mut;
        for (uint32_t o = 1; o < LR; o <<= 1) {
            m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
            mut = __shfl_xor_sync(0xffffffffu, mut ? 1 : 0, o) != 0 || mut;
        }
        const uint32_t G = slice_groups(P, S);
        const uint32_t row = (warp % G) * slice_rows_per_warp(S) + lane / LR;
        if (warp < G * slice_chunks(P, S) && lane % LR == 0 && row < P && m > -2000) {
            RunDev& R = runs[run];
            atomicMax(R.xexp_max + row, m);
            if (mut) R.changed[row] = 1;
        }
        lane_max = -2000;
        lane_mut = false;
    };

    for (uint32_t k = 0;; ++k) {
        const uint32_t st = k % kSliceStages;
        if (!mbar_wait(&s_full[st], (k / kSliceStages) & 1u)) {
            if (lane == 0) s_fail = 1;
            break;
        }
        const SliceTable& T = s_tab[st];
        if (T.item == kNoItem) break;
        const uint32_t rn = T.run;
        if (rn != run) {
            flush();
            run = rn;
            P = T.P;
            S = T.S;
        }
        const uint32_t M = T.M;
        const uint32_t cpi = slice_chunks(P, S), L = cpi * kChunk;
        const uint32_t j0 = T.item * L;
        const uint32_t len = M - j0 < L ? M - j0 : L;
        const uint32_t nch = (len + kChunk - 1) / kChunk;
        const uint32_t G = slice_groups(P, S);
        if (warp < G * nch) {
            // ---- one chunk of one member group
            const uint32_t RW = slice_rows_per_warp(S), LR = 8 * S;
            const uint32_t c = warp / G;
            const uint32_t row0 = (warp - c * G) * RW;
            const uint32_t jc = c * kChunk;                             // the chunk's first gene in the item
            const uint32_t halves = len - jc < (uint32_t)kChunk ? 1u : 2u;  // 32-gene halves of the chunk
            const bool first_chunk = j0 + jc == 0;  // holds gene 0
            const double* par = slice_s + (uint64_t)st * kSliceStageDoubles;
            const uint64_t PM = (uint64_t)P * M;
            const uint64_t key_x = T.key_x;
            const bool keep_sign = T.keep_sign != 0;
            // formation, lane = gene: per member of the group, side and half,
            // 32 consecutive genes (conflict-free reads of the staged parents,
            // coalesced trial stores); the chunk's exponent and mutation flag
            // of the member this lane digitises below
            int my_e = -2000;
            bool my_mut = false;
            for (uint32_t mm = 0; mm < RW; ++mm) {
                const uint32_t row = row0 + mm;
                if (row >= P) break;
                const double* pa = par + (uint64_t)T.mut[0][row] * S * L;
                const double* pb = par + (uint64_t)T.mut[1][row] * S * L;
                const double* pc = par + (uint64_t)T.mut[2][row] * S * L;
                const double* px = par + (uint64_t)row * S * L;
                double* dst = T.pop + (uint64_t)(1u - T.cur[row]) * S * PM + (uint64_t)row * M + j0;
                const uint64_t pos0 = (T.step[row] * P + row) * S;
                uint32_t ef_max = 0;
                bool mt = false;
                double z = 0.0;  // side 0's gene 0 (lane 0 of the first half)
                // (both sides unrolled: their loads, draws and FMAs overlap)
#pragma unroll
                for (uint32_t s = 0; s < 2; ++s) {
                    if (s >= S) break;
                    const uint64_t thr = T.thr[s][row];
                    const double fw = T.fw[s][row];
                    // the draws of this side's chunk genes are consecutive
                    // stream outputs: the Weyl value of gene jc + 32 h + lane
                    // is w0 + (32 h + lane) gamma
                    const uint64_t w0 = key_x + ((pos0 + s) * M + j0 + jc + 1) * kGamma + lane_gamma;
                    // both 32-gene halves at once (independent loads, draws
                    // and FMAs in flight)
                    // (a 32-gene last chunk reads the stage's stale second
                    // half too: inside the staged row, and never used)
                    double x[2], a[2], b[2], cc[2];
#pragma unroll
                    for (uint32_t h = 0; h < 2; ++h) {
                        const uint32_t o = s * L + jc + h * 32 + lane;
                        x[h] = px[o];
                        a[h] = pa[o];
                        b[h] = pb[o];
                        cc[h] = pc[o];
                    }
#pragma unroll
                    for (uint32_t h = 0; h < 2; ++h) {
                        if (h >= halves) continue;
                        const uint32_t jl = jc + h * 32 + lane;
                        const bool mutate = (splitmix_mix(w0 + h * (32 * kGamma)) >> 11) < thr;
                        double v = x[h];
                        mutate_gene(v, a[h], b[h], cc[h], fw, mutate);
                        if (mutate) {
                            if (!keep_sign) v = abs_bits(v);
                            mt = true;
                        }
                        if (first_chunk && h == 0 && lane == 0) {
                            if (s == 0) z = v;
                            else v = z;  // gpu_match_population_zero
                        }
                        st_keep_l1(dst + (uint64_t)s * PM + jl, v);
                        // the exponent field of |v| (0: zero or subnormal)
                        ef_max = max(ef_max, ((uint32_t)__double2hiint(v) >> 20) & 0x7FFu);
                    }
                }
                ef_max = __reduce_max_sync(0xffffffffu, ef_max);
                const int em = ef_max == 0 ? -2000 : (int)ef_max - 1023;  // as exp_of
                mt = __any_sync(0xffffffffu, mt);
                if (lane / LR == mm) {
                    my_e = em;
                    my_mut = mt;
                }
            }
            // the warp's trial stores are visible to all its lanes (a
            // warp-wide barrier orders memory among its threads)
            __syncwarp();
            // digits, lane = (member, side, unit of 8 genes): the unit's
            // trial genes read back (from the caches) and sliced at the
            // chunk's scale
            const uint32_t row = row0 + lane / LR;
            const uint32_t s = (lane % LR) >> 3, u = lane & 7u;
            if (row < P && u < halves * 4) {
                const uint32_t jl = jc + u * 8;
                const double2* src = reinterpret_cast<const double2*>(
                    T.pop + ((uint64_t)(1u - T.cur[row]) * S + s) * PM + (uint64_t)row * M + j0 + jl);
                double v[8];
#pragma unroll
                for (uint32_t q = 0; q < 4; ++q) {
                    const double2 w = src[q];
                    v[2 * q] = w.x;
                    v[2 * q + 1] = w.y;
                }
                const int e = my_e <= -1500 ? -1000 : my_e + 1;  // scale 2^e > every |v| of the chunk
                store_unit_digits(v, e,
                                  T.xdig + xdig_row_offset(T.xdig_row0 + row) + s * T.xdig_side +
                                      (uint64_t)((j0 + jl) >> 3) * T.xdig_unit);
                if (s == 0 && u == 0) T.xexp[(uint64_t)row * split_chunks(M) + (j0 + jc) / kChunk] = (int16_t)e;
                lane_max = max(lane_max, e);
                lane_mut = lane_mut || my_mut;
            }
        }
        // the last warp done with the stage stages the item kSliceStages on
        __syncwarp();
        uint32_t last = 0;
        if (lane == 0) {
            __threadfence_block();
            last = atomicAdd(&s_done[st], 1u) == kSliceWarps - 1 ? 1u : 0u;
            if (last) {
                s_done[st] = 0;
                __threadfence_block();
            }
        }
        if (__shfl_sync(0xffffffffu, last, 0)) stage_next(st);
    }
    flush();
    __syncthreads();
    if (s_fail && tid == 0) {
        atomicCAS(status, 0, kStatusSliceWait);
        // the copies this CTA issued land before it exits (bounded waits on
        // each stage's latest armed phase)
        for (uint32_t q = 0; q < kSliceStages; ++q)
            if (s_armed[q]) mbar_wait(&s_full[q], (s_armed[q] - 1) & 1u);
    }
}

}  // namespace deac
