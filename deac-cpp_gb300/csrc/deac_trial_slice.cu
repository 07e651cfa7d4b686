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

// The CTA's position in its item sequence: segment g, item `it` of it.
struct SliceCursor {
    uint32_t g, it;
};

// Advance `c` to the first live item at or after it (runs that are done are
// skipped; every thread of the CTA walks the same sequence).
__device__ __forceinline__ void slice_settle(SliceCursor& c, const SliceSeg* segs, uint32_t se, const RunDev* runs) {
    while (c.g < se && (c.it >= segs[c.g].item1 || runs[segs[c.g].run].done)) {
        ++c.g;
        if (c.g < se) c.it = segs[c.g].item0;
    }
}

}  // namespace

__global__ void __launch_bounds__(kSliceThreads, 2)
    trial_slice_kernel(RunDev* runs, const SliceSeg* segs, const uint32_t* seg_start, int* status) {
    extern __shared__ __align__(128) double slice_s[];
    double* const stage0 = slice_s;  // two stages of kSliceStageDoubles
    double* const tri = slice_s + 2 * kSliceStageDoubles;
    int* const s_e = reinterpret_cast<int*>(tri + kSliceTrialDoubles);  // [member][chunk] scale exponents
    __shared__ __align__(8) uint64_t s_bar[2];
    __shared__ uint64_t s_thr[2][kSliceRows];
    __shared__ double s_fw[2][kSliceRows];
    __shared__ uint64_t s_step[kSliceRows];
    __shared__ uint8_t s_mut[3][kSliceRows];
    __shared__ uint8_t s_cur[kSliceRows];
    __shared__ uint8_t s_changed[kSliceRows];
    __shared__ int s_rowmax[kSliceRows];

    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    constexpr uint32_t kWarps = kSliceThreads / 32;
    const uint32_t sb = seg_start[blockIdx.x], se = seg_start[blockIdx.x + 1];
    if (tid == 0) {
        mbar_init(&s_bar[0], 1);
        mbar_init(&s_bar[1], 1);
        mbar_init_fence();
    }
    __syncthreads();
    grid_dependency_wait();
    // the previous generation's exact pass is done with its item list (one
    // count for the whole batch)
    if (blockIdx.x == 0 && tid == 0) *runs[0].exact_count = 0;

    // warp 0: the bulk copies of the item at `c` into stage `st` -- every
    // member's parent rows of the item, one copy per (member, side)
    auto issue = [&](const SliceCursor& c, uint32_t st) {
        const RunDev& R = runs[segs[c.g].run];
        const uint32_t P = R.P, S = R.S, M = R.M;
        const uint32_t Lst = slice_chunks(P) * kChunk;
        const uint32_t j0 = c.it * Lst;
        const uint32_t L = M - j0 < Lst ? M - j0 : Lst;
        const uint64_t PM = (uint64_t)P * M;
        uint64_t* bar = &s_bar[st];
        if (lane == 0) mbar_expect_tx(bar, P * S * L * (uint32_t)sizeof(double));
        __syncwarp();
        double* dst = stage0 + (uint64_t)st * kSliceStageDoubles;
        for (uint32_t q = lane; q < P * S; q += 32) {
            const uint32_t m = q / S, s = q - m * S;
            const double* src = R.pop + ((uint64_t)R.cur[m] * S + s) * PM + (uint64_t)m * M + j0;
            bulk_load(dst + (uint64_t)q * Lst, src, L * (uint32_t)sizeof(double), bar);
        }
    };

    SliceCursor c{sb, sb < se ? segs[sb].item0 : 0u};
    slice_settle(c, segs, se, runs);
    SliceCursor ic = c;  // the next item to stage (warp 0)
    uint32_t issued = 0;
    if (warp == 0)
        for (uint32_t st = 0; st < 2 && ic.g < se; ++st) {
            issue(ic, st);
            ++ic.it;
            slice_settle(ic, segs, se, runs);
            ++issued;
        }
    bool failed = false;
    uint32_t k = 0;           // items consumed
    uint32_t run = 0xFFFFFFFFu, P = 0;
    // the run's bookkeeping of this CTA's items: chunk maxima and changed
    // flags, raised into the run's arrays when the CTA leaves the run
    auto flush = [&]() {
        if (run != 0xFFFFFFFFu && tid < P) {
            RunDev& R = runs[run];
            if (s_changed[tid]) R.changed[tid] = 1;
            atomicMax(R.xexp_max + tid, s_rowmax[tid]);
        }
    };
    while (c.g < se) {
        const uint32_t rn = segs[c.g].run;
        RunDev& R = runs[rn];
        if (rn != run) {
            flush();
            run = rn;
            P = R.P;
            if (tid < kSliceRows) {
                s_changed[tid] = 0;
                s_rowmax[tid] = -2000;
                if (tid < P) {
                    // the member's CR / F and mutant indices of this
                    // generation's trial, its jDE step and parent buffer
                    const uint32_t S = R.S;
                    s_cur[tid] = R.cur[tid];
                    for (uint32_t s = 0; s < S; ++s) {
                        s_thr[s][tid] = crossover_threshold(R.cr[(uint64_t)S * P + s * P + tid]);
                        s_fw[s][tid] = R.fw[(uint64_t)S * P + s * P + tid];
                    }
                    for (uint32_t q = 0; q < 3; ++q) s_mut[q][tid] = (uint8_t)R.mutants[3 * tid + q];
                    s_step[tid] = R.rng[tid] - 1;
                }
            }
            __syncthreads();
        }
        const uint32_t S = R.S, M = R.M;
        const uint32_t cpi = slice_chunks(P), Lst = cpi * kChunk;
        const uint32_t j0 = c.it * Lst;
        const uint32_t L = M - j0 < Lst ? M - j0 : Lst;
        const uint32_t nch = L / kChunk;
        const uint64_t PM = (uint64_t)P * M;
        const uint32_t T = S * Lst + 2;  // trial row stride (doubles)
        const uint32_t st = k & 1u;
        const double* par = stage0 + (uint64_t)st * kSliceStageDoubles;
        const bool ok = mbar_wait(&s_bar[st], (k >> 1) & 1u);
        if (__syncthreads_or(!ok)) {
            failed = true;
            break;
        }
        // ---- the trial genes: one warp per (member, chunk), both sides
        {
            const uint64_t key_x = R.key_crossover;
            const bool keep_sign = (R.flags & kSignedWeights) != 0;
            for (uint32_t t = warp; t < P * nch; t += kWarps) {
                const uint32_t i = t / nch, ch = t - i * nch;
                const uint32_t jl = ch * kChunk + lane, j = j0 + jl;
                const double* pa = par + (uint64_t)s_mut[0][i] * S * Lst + jl;
                const double* pb = par + (uint64_t)s_mut[1][i] * S * Lst + jl;
                const double* pc = par + (uint64_t)s_mut[2][i] * S * Lst + jl;
                const double* px = par + (uint64_t)i * S * Lst + jl;
                double* dst = R.pop + ((uint64_t)(1u - s_cur[i]) * S) * PM + (uint64_t)i * M + j;
                double* trow = tri + (uint64_t)i * T + jl;
                const uint64_t pos0 = (s_step[i] * P + i) * S;
                bool mutated = false;
                int e = -2000;
                double v0 = 0.0;
                for (uint32_t s = 0; s < S; ++s) {
                    const uint32_t o = s * Lst;
                    const bool mutate = (stream_draw(key_x, (pos0 + s) * M + j) >> 11) < s_thr[s][i];
                    double v = px[o];
                    if (mutate) {
                        v = fma(s_fw[s][i], pb[o] - pc[o], pa[o]);
                        if (!keep_sign)
                            v = __longlong_as_double(__double_as_longlong(v) & 0x7FFFFFFFFFFFFFFFll);  // fabs
                        mutated = true;
                    }
                    if (s == 0) v0 = v;
                    else if (j == 0) v = v0;  // gpu_match_population_zero
                    dst[(uint64_t)s * PM] = v;
                    trow[o] = v;
                    e = max(e, exp_of(v));
                }
                e = __reduce_max_sync(0xffffffffu, e);
                mutated = __any_sync(0xffffffffu, mutated);
                if (lane == 0) {
                    s_e[i * cpi + ch] = e;
                    if (mutated) s_changed[i] = 1;
                }
            }
        }
        __syncthreads();
        // the stage is free: the item after next into it
        if (warp == 0 && ic.g < se) {
            issue(ic, st);
            ++ic.it;
            slice_settle(ic, segs, se, runs);
            ++issued;
        }
        // ---- the digit planes: one thread per (member, side, unit of 8
        // genes), consecutive threads on consecutive members
        {
            const uint32_t units = nch * 4;
            const uint64_t unit0 = j0 / 8;
            const uint32_t C = M / kChunk;
            for (uint32_t t = tid; t < S * units * P; t += kSliceThreads) {
                const uint32_t row = t % P, q = t / P;
                const uint32_t s = q / units, u = q - s * units;
                const double* src = tri + (uint64_t)row * T + s * Lst + u * 8;
                double v[8];
#pragma unroll
                for (uint32_t h = 0; h < 4; ++h) {
                    const double2 w = reinterpret_cast<const double2*>(src)[h];
                    v[2 * h] = w.x;
                    v[2 * h + 1] = w.y;
                }
                const uint32_t ch = u >> 2;
                int e = s_e[row * cpi + ch];
                e = e <= -1500 ? -1000 : e + 1;  // scale 2^e > every |v| of the chunk
                store_unit_digits(v, e,
                                  R.xdig + xdig_row_offset(R.xdig_row0 + row) + s * R.xdig_side +
                                      (unit0 + u) * R.xdig_unit);
                if (s == 0 && (u & 3u) == 0) {
                    R.xexp[(uint64_t)row * C + j0 / kChunk + ch] = (int16_t)e;
                    atomicMax(&s_rowmax[row], e);
                }
            }
        }
        __syncthreads();
        ++k;
        ++c.it;
        slice_settle(c, segs, se, runs);
    }
    if (!failed) {
        flush();
        return;
    }
    if (tid == 0) {
        atomicCAS(status, 0, kStatusSliceWait);
        // the copies this CTA issued land before it exits (bounded waits)
        for (uint32_t q = k; q < issued; ++q) mbar_wait(&s_bar[q & 1u], (q >> 1) & 1u);
    }
    __syncthreads();
}

}  // namespace deac
