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
// every member (written by the warp that stages the item).
struct SliceTable {
    uint64_t thr[2][kSliceRows];
    double fw[2][kSliceRows];
    uint64_t step[kSliceRows];
    uint8_t mut[3][kSliceRows];
    uint8_t cur[kSliceRows];
    uint32_t run, item;  // run kNoItem: the CTA's items are exhausted
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
                T.run = kNoItem;
                mbar_arrive(&s_full[st]);
            }
            __syncwarp();
            return;
        }
        const uint32_t run = segs[c.g].run;
        const RunDev& R = runs[run];
        const uint32_t P = R.P, S = R.S, M = R.M;
        const uint32_t L = slice_chunks(P, S) * kChunk;
        const uint32_t j0 = c.it * L;
        const uint32_t len = M - j0 < L ? M - j0 : L;
        const uint64_t PM = (uint64_t)P * M;
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
            T.run = run;
            T.item = c.it;
        }
        __syncwarp();
        if (lane == 0) mbar_expect_tx(&s_full[st], P * S * len * (uint32_t)sizeof(double));
        __syncwarp();
        double* dst = slice_s + (uint64_t)st * kSliceStageDoubles;
        for (uint32_t q = lane; q < P * S; q += 32) {
            const uint32_t m = q / S, s = q - m * S;
            const double* src = R.pop + ((uint64_t)T.cur[m] * S + s) * PM + (uint64_t)m * M + j0;
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
        const uint32_t rn = T.run;
        if (rn == kNoItem) break;
        RunDev& R = runs[rn];
        if (rn != run) {
            flush();
            run = rn;
            P = R.P;
            S = R.S;
        }
        const uint32_t M = R.M;
        const uint32_t cpi = slice_chunks(P, S), L = cpi * kChunk;
        const uint32_t j0 = T.item * L;
        const uint32_t len = M - j0 < L ? M - j0 : L;
        const uint32_t nch = (len + kChunk - 1) / kChunk;
        const uint32_t G = slice_groups(P, S);
        if (warp < G * nch) {
            // ---- one chunk of one member group: lane = (member, side, unit)
            const uint32_t LR = 8 * S;
            const uint32_t c = warp / G;
            const uint32_t row = (warp - c * G) * slice_rows_per_warp(S) + lane / LR;
            const uint32_t s = (lane % LR) >> 3, u = lane & 7u;
            const uint32_t jl = c * kChunk + u * 8;  // the unit's first gene within the item
            const bool live = row < P && jl < len;
            const uint32_t rr = row < P ? row : 0;
            const double* par = slice_s + (uint64_t)st * kSliceStageDoubles;
            const uint64_t PM = (uint64_t)P * M;
            double v[8] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
            bool mutated = false;
            int e = -2000;
            if (live) {
                const double* px = par + ((uint64_t)rr * S + s) * L + jl;
                const double* pa = par + ((uint64_t)T.mut[0][rr] * S + s) * L + jl;
                const double* pb = par + ((uint64_t)T.mut[1][rr] * S + s) * L + jl;
                const double* pc = par + ((uint64_t)T.mut[2][rr] * S + s) * L + jl;
                const uint64_t thr = T.thr[s][rr];
                const double fw = T.fw[s][rr];
                const bool keep_sign = (R.flags & kSignedWeights) != 0;
                const uint64_t pos = ((T.step[rr] * P + rr) * S + s) * (uint64_t)M + j0 + jl;
                const uint64_t key_x = R.key_crossover;
#pragma unroll
                for (uint32_t h = 0; h < 4; ++h) {
                    const double2 x = reinterpret_cast<const double2*>(px)[h];
                    const double2 a = reinterpret_cast<const double2*>(pa)[h];
                    const double2 b = reinterpret_cast<const double2*>(pb)[h];
                    const double2 cc = reinterpret_cast<const double2*>(pc)[h];
#pragma unroll
                    for (uint32_t q = 0; q < 2; ++q) {
                        const uint32_t kk = 2 * h + q;
                        const bool mutate = (stream_draw(key_x, pos + kk) >> 11) < thr;
                        double w = q ? x.y : x.x;
                        if (mutate) {
                            w = fma(fw, (q ? b.y : b.x) - (q ? cc.y : cc.x), q ? a.y : a.x);
                            if (!keep_sign)
                                w = __longlong_as_double(__double_as_longlong(w) & 0x7FFFFFFFFFFFFFFFll);  // fabs
                            mutated = true;
                        }
                        v[kk] = w;
                    }
                }
            }
            // gpu_match_population_zero: side 1's gene 0 takes side 0's (held
            // by the member's first lane)
            const double z = __shfl_sync(0xffffffffu, v[0], lane & ~(LR - 1u));
            if (live && s == 1 && j0 + jl == 0) v[0] = z;
            if (live) {
                double* dst = R.pop + ((uint64_t)(1u - T.cur[rr]) * S + s) * PM + (uint64_t)rr * M + j0 + jl;
#pragma unroll
                for (uint32_t h = 0; h < 4; ++h)
                    reinterpret_cast<double2*>(dst)[h] = make_double2(v[2 * h], v[2 * h + 1]);
#pragma unroll
                for (uint32_t kk = 0; kk < 8; ++kk) e = max(e, exp_of(v[kk]));
            }
            for (uint32_t o = 1; o < LR; o <<= 1) e = max(e, __shfl_xor_sync(0xffffffffu, e, o));
            e = e <= -1500 ? -1000 : e + 1;  // scale 2^e > every |v| of the chunk
            if (live) {
                store_unit_digits(v, e,
                                  R.xdig + xdig_row_offset(R.xdig_row0 + rr) + s * R.xdig_side +
                                      (uint64_t)((j0 + jl) >> 3) * R.xdig_unit);
                if (s == 0 && u == 0) R.xexp[(uint64_t)rr * split_chunks(M) + (j0 + jl) / kChunk] = (int16_t)e;
                lane_max = max(lane_max, e);
                lane_mut = lane_mut || mutated;
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
