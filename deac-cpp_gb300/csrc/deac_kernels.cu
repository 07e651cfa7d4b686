// deac_kernels.cu -- kernels of the plain FP64 engine (see deac_kernels.cuh).
// Compiled with --fmad=false: the only fused multiply-adds are the explicit
// fma() calls, placed where the reference's nvcc build fuses.
#include <cuda_runtime.h>

#include "deac_chain.cuh"
#include "deac_jde.cuh"
#include "deac_kernels.cuh"
#include "deac_rng.cuh"
#include "deac_split.cuh"

namespace deac {

namespace {

constexpr int kTreeSlots = 1024;   // GPU_BLOCK_SIZE of the reference reductions

__device__ __forceinline__ void store_state(const RunDev& R, uint64_t slot, const uint64_t s[4]) {
    const uint64_t n = R.n_states;
    R.rng[slot] = s[0];
    R.rng[n + slot] = s[1];
    R.rng[2 * n + slot] = s[2];
    R.rng[3 * n + slot] = s[3];
}


// k-ascending FMA chain continuing from `acc` (the inner loops of
// gpu_matmul and gpu_deac_gemv, deac_gpu.cu:302-304, 359-363).  Operands of
// the next 8 steps are loaded while the current 8 are fused, so a dependent
// DFMA (64 cycles on this part) never waits for memory.
__device__ __forceinline__ double chain(const double* x, const double* w, uint32_t n, double acc) {
    constexpr uint32_t U = 8;
    uint32_t k = 0;
    if (n >= U) {
        double xa[U], wa[U];
#pragma unroll
        for (uint32_t u = 0; u < U; ++u) {
            xa[u] = x[u];
            wa[u] = w[u];
        }
        for (k = U; k + U <= n; k += U) {
            double xb[U], wb[U];
#pragma unroll
            for (uint32_t u = 0; u < U; ++u) {
                xb[u] = x[k + u];
                wb[u] = w[k + u];
            }
#pragma unroll
            for (uint32_t u = 0; u < U; ++u) acc = fma(xa[u], wa[u], acc);
#pragma unroll
            for (uint32_t u = 0; u < U; ++u) {
                xa[u] = xb[u];
                wa[u] = wb[u];
            }
        }
#pragma unroll
        for (uint32_t u = 0; u < U; ++u) acc = fma(xa[u], wa[u], acc);
    }
    for (; k < n; ++k) acc = fma(x[k], w[k], acc);
    return acc;
}

__device__ __forceinline__ void cp_async16(double* dst, const double* src) {
    const uint32_t d = (uint32_t)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async8(double* dst, const double* src) {
    const uint32_t d = (uint32_t)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// Row sum of the gemv pair the reference issues for normalisation and
// moments: y = alpha*s_pos (beta = 0), then y = alpha*s_neg + 1*y, which
// nvcc fuses as fma(alpha, s_neg, y).  (The reference's multi-block gemv
// adds s_neg once per 32-gene block when M > 32, deac_gpu.cu:345-374; this
// is the value of the race-free single block.)
__device__ __forceinline__ double gemv_pair(double s_pos, double s_neg, double alpha, int two_sided) {
    double y = alpha * s_pos;
    if (two_sided) y = fma(alpha, s_neg, y);
    return y;
}

// Pairwise tree over `width` (a power of two <= 1024) slots in shared memory
// by one warp: levels s = width/2 .. 1 add slot t+s into slot t, as the
// reference's block reductions do (deac_gpu.cu:435-442, 63-129).  Levels
// s >= 32 go through shared memory, the rest through shuffles; both pair the
// same slots.  Returns the total on lane 0.
__device__ double warp_tree(double* slots, uint32_t width) {
    const uint32_t lane = threadIdx.x & 31u;
    for (uint32_t s = width >> 1; s >= 32; s >>= 1) {
        for (uint32_t t = lane; t < s; t += 32) slots[t] += slots[t + s];
        __syncwarp();
    }
    const uint32_t w = width < 32 ? width : 32;
    double v = lane < w ? slots[lane] : 0.0;
    for (uint32_t s = w >> 1; s > 0; s >>= 1) v += __shfl_down_sync(0xffffffffu, v, s);
    return v;
}

__device__ __forceinline__ uint32_t pow2_ceil(uint32_t n) {
    uint32_t w = 1;
    while (w < n) w <<= 1;
    return w;
}

// min of a shared double with v (a CAS loop: no native double atomicMin)
__device__ __forceinline__ void atomic_min_double_smem(double* p, double v) {
    unsigned long long* a = reinterpret_cast<unsigned long long*>(p);
    unsigned long long old = *a;
    while (v < __longlong_as_double((long long)old)) {
        const unsigned long long seen = atomicCAS(a, old, (unsigned long long)__double_as_longlong(v));
        if (seen == old) break;
        old = seen;
    }
}

}  // namespace

// ---------------------------------------------------------------- trial
// Dynamic shared memory: the member's S*M trial genes, then S*M weights of
// the row sum being formed (normalisation, first or third moment), when the
// batch's capacity `smem_doubles` allows; otherwise the chains read global
// memory (still k-ascending).
// jDE of member i (deac_gpu.cu:584-606): CR(+) on slot 0, F(+) slot 1,
// CR(-) slot 2, F(-) slot 3; then the mutant indices on slot 0
// (deac_gpu.cu:608-633), the launch order of deac.cpp:1168-1219.  Stores
// the new CR and F and the four slots' states; returns CR, F and the indices.
// jDE of member i with every result stored (deac_jde.cuh)
__device__ __forceinline__ void jde_member(RunDev& R, uint32_t i, double cr_new[2], double fw_new[2],
                                           uint32_t mut[3]) {
    uint64_t st[4][4];
    jde_load(R, i, st);
    double cr_old[2], fw_old[2];
#pragma unroll
    for (uint32_t s = 0; s < 2; ++s) {
        cr_old[s] = s < R.S ? R.cr[s * R.P + i] : 0.0;
        fw_old[s] = s < R.S ? R.fw[s * R.P + i] : 0.0;
    }
    jde_draw(R, i, st, cr_old, fw_old, cr_new, fw_new, mut);
    jde_store(R, i, st, cr_new, fw_new, mut, false);
}

__device__ __forceinline__ void trial_body(RunDev* runs, const Work* work, int init_mode, int smem_doubles) {
    extern __shared__ __align__(16) double trial_s[];
    __shared__ double s_fw[2], s_sum[4];
    __shared__ uint64_t s_thr[2];
    __shared__ uint32_t s_mut[3];
    __shared__ uint64_t s_step;
    __shared__ ChainScratch s_chain[2];

    const Work w = work[blockIdx.x];
    RunDev& R = runs[w.run];
    if (R.done) return;
    const uint32_t i = w.index;
    const uint32_t P = R.P, M = R.M, S = R.S;
    const uint64_t PM = (uint64_t)P * M;
    const uint64_t SM = (uint64_t)S * M;
    const uint32_t parent_buf = R.cur[i];
    const uint32_t dst_buf = init_mode ? parent_buf : 1u - parent_buf;
    double* dst = R.pop + ((uint64_t)dst_buf * S) * PM + (uint64_t)i * M;  // side s at + s*PM
    const bool in_smem = SM <= (uint64_t)smem_doubles;
    const bool terms_in_smem = 2 * SM <= (uint64_t)smem_doubles;
    double* terms_s = trial_s + SM;
    const uint64_t base = (uint64_t)i * (1ull + SM);

    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    const bool normalize = (R.flags & kNormalize) != 0;

    // weights of one row sum, staged next to the genes when they fit
    auto weights = [&](const double* wp, const double* wn, const double*& tp, const double*& tn) {
        if (terms_in_smem) {
            for (uint32_t k = threadIdx.x; k < M; k += blockDim.x) {
                terms_s[k] = wp[k];
                if (S == 2) terms_s[M + k] = wn[k];
            }
            tp = terms_s;
            tn = terms_s + M;
        } else {
            tp = wp;
            tn = wn;
        }
    };
    const double *norm_p = nullptr, *norm_n = nullptr;
    const bool row_sums_here = normalize && (init_mode || !(R.flags & kDeferNorm));
    if (row_sums_here) weights(R.norm_pos, R.norm_neg, norm_p, norm_n);

    const bool counter = (R.flags & kCounterStreams) != 0;
    if (!init_mode && threadIdx.x == 0) {
        double cr[2], fw[2];
        if (counter) s_step = R.rng[i];  // this trial's jDE step
        jde_member(R, i, cr, fw, s_mut);
#pragma unroll
        for (uint32_t s = 0; s < 2; ++s)
            if (s < S) {
                s_thr[s] = crossover_threshold(cr[s]);
                s_fw[s] = fw[s];
            }
    }
    __syncthreads();

    const double* gene_pos = in_smem ? trial_s : dst;
    const double* gene_neg = in_smem ? trial_s + M : dst + PM;
    // row-sum chains (normalisation and moments): warps 0-7 the positive
    // side, warps 8-15 the negative side, each group by the exact parallel
    // evaluation of the sequential FMA chain (deac_chain.cuh)
    const uint32_t chain_side = warp / kChainWarps;
    const bool chain_warp = chain_side < S;
    const double* chain_x = chain_side == 0 ? gene_pos : gene_neg;
    const double* chain_w = chain_side == 0 ? norm_p : norm_n;
    auto row_sum = [&](const double* wts) -> double {
        return group_fma_chain<kChainWarps, kChainSteps>(chain_x, wts, M, 0.0, chain_side * kChainWarps,
                                                         1 + (int)chain_side, s_chain[chain_side]);
    };

    if (!init_mode) {
        // crossover draw + DE/rand/1 mutation per gene (deac_gpu.cu:514-539,
        // 635-643), in chunks of kGeneChunk genes per side
        const uint32_t r0 = s_mut[0], r1 = s_mut[1], r2 = s_mut[2];
        const uint64_t buf = (uint64_t)S * PM;  // stride between the two buffers
        const double* pa = R.pop + (uint64_t)R.cur[r0] * buf + (uint64_t)r0 * M;
        const double* pb = R.pop + (uint64_t)R.cur[r1] * buf + (uint64_t)r1 * M;
        const double* pc = R.pop + (uint64_t)R.cur[r2] * buf + (uint64_t)r2 * M;
        const double* px = R.pop + (uint64_t)parent_buf * buf + (uint64_t)i * M;
        const bool keep_sign = (R.flags & kSignedWeights) != 0;
        const uint64_t n = R.n_states;
        // counter streams: gene j of side s draws position cpos + s*M + j
        const uint64_t cpos = counter ? (s_step * P + i) * SM : 0;
        const uint64_t key_x = R.key_crossover;
        constexpr uint32_t kGeneChunk = 256;
        const uint32_t nchunks = (M + kGeneChunk - 1) / kGeneChunk;

        // genes [c*kGeneChunk, ...) of both sides, by worker `wid` of `nt`
        bool mutated = false;
        auto produce = [&](uint32_t c, uint32_t wid, uint32_t nt) {
            const uint32_t j0 = c * kGeneChunk;
            const uint32_t len = min(kGeneChunk, M - j0);
            const uint32_t items = S * len;
            constexpr int H = 2;  // genes in flight per thread
            for (uint32_t e0 = wid; e0 < items; e0 += H * nt) {
                uint64_t st[H][4];
                double a[H], b[H], cc[H], x[H];
                uint32_t sd[H], jj[H];
                bool ok[H];
#pragma unroll
                for (int h = 0; h < H; ++h) {
                    const uint32_t e = e0 + (uint32_t)h * nt;
                    ok[h] = e < items;
                    const uint32_t ee = ok[h] ? e : e0;
                    sd[h] = ee / len;
                    jj[h] = j0 + (ee - sd[h] * len);
                    const uint64_t slot = base + 1 + (uint64_t)sd[h] * M + jj[h];
                    if (!counter) {
                        st[h][0] = R.rng[slot];
                        st[h][1] = R.rng[n + slot];
                        st[h][2] = R.rng[2 * n + slot];
                        st[h][3] = R.rng[3 * n + slot];
                    }
                    const uint64_t off = (uint64_t)sd[h] * PM + jj[h];
                    a[h] = pa[off];
                    b[h] = pb[off];
                    cc[h] = pc[off];
                    x[h] = px[off];
                }
#pragma unroll
                for (int h = 0; h < H; ++h) {
                    if (!ok[h]) continue;
                    bool mutate;
                    if (counter) {
                        mutate = (stream_draw(key_x, cpos + (uint64_t)sd[h] * M + jj[h]) >> 11) < s_thr[sd[h]];
                    } else {
                        mutate = (xoshiro_next(st[h][0], st[h][1], st[h][2], st[h][3]) >> 11) < s_thr[sd[h]];
                        store_state(R, base + 1 + (uint64_t)sd[h] * M + jj[h], st[h]);
                    }
                    double v = x[h];
                    mutate_gene(v, a[h], b[h], cc[h], s_fw[sd[h]], mutate);
                    if (mutate) {
                        if (!keep_sign) v = abs_bits(v);
                        mutated = true;
                    }
                    dst[(uint64_t)sd[h] * PM + jj[h]] = v;
                    if (in_smem) trial_s[(uint64_t)sd[h] * M + jj[h]] = v;
                }
            }
        };

        for (uint32_t c = 0; c < nchunks; ++c) produce(c, threadIdx.x, blockDim.x);
        __syncthreads();
        if (S == 2 && threadIdx.x == 0) {
            // gpu_match_population_zero (deac_gpu.cu:541-549)
            const double z = in_smem ? trial_s[0] : dst[0];
            dst[PM] = z;
            if (in_smem) trial_s[M] = z;
        }
        __syncthreads();
    } else if (in_smem) {
        for (uint64_t q = threadIdx.x; q < SM; q += blockDim.x) {
            const uint32_t s = (uint32_t)(q / M);
            trial_s[q] = dst[(uint64_t)s * PM + (q - (uint64_t)s * M)];
        }
        __syncthreads();
    }

    // split engine, kDeferNorm: the trial stays raw here (norm_kernel forms
    // its norm; split_select_kernel normalises it after the decision)
    if (row_sums_here) {
        // normalisation row sum and reciprocal scale
        // (deac_gpu.cu:345-374 with alpha = 1/F(0), then 406-415)
        if (chain_warp) {
            const double v = row_sum(chain_w);
            if (warp % kChainWarps == 0 && lane == 0) s_sum[chain_side] = v;
        }
        __syncthreads();
        const double norm = gemv_pair(s_sum[0], S == 2 ? s_sum[1] : 0.0, R.alpha, S == 2);
        const double recip = 1.0 / norm;
        for (uint64_t q = threadIdx.x; q < SM; q += blockDim.x) {
            const uint32_t s = (uint32_t)(q / M);
            const uint64_t g = (uint64_t)s * PM + (q - (uint64_t)s * M);
            const double v = (in_smem ? trial_s[q] : dst[g]) * recip;
            dst[g] = v;
            if (in_smem) trial_s[q] = v;
        }
        __syncthreads();
    }

    // moment row sums with alpha = 1 (deac.cpp:1418-1477)
    for (int which = 0; which < 2; ++which) {
        const uint32_t flag = which == 0 ? kFirstMoment : kThirdMoment;
        if (!(R.flags & flag)) continue;
        const double *tp, *tn;
        weights(which == 0 ? R.first_pos : R.third_pos, which == 0 ? R.first_neg : R.third_neg, tp, tn);
        __syncthreads();
        if (chain_warp) {
            const double v = row_sum(chain_side == 0 ? tp : tn);
            if (warp % kChainWarps == 0 && lane == 0) s_sum[chain_side] = v;
        }
        __syncthreads();
        if (threadIdx.x == 0) R.moments[2 * i + which] = gemv_pair(s_sum[0], S == 2 ? s_sum[1] : 0.0, 1.0, S == 2);
        __syncthreads();
    }

}

__global__ void __launch_bounds__(kTrialThreads)
trial_kernel(RunDev* runs, const Work* work, int init_mode, int smem_doubles) {
    trial_body(runs, work, init_mode, smem_doubles);
}

// -------------------------------------------------------------- snapshot
__global__ void snapshot_kernel(const RunDev* runs, uint32_t n, const uint32_t* fit_off, const uint64_t* gene_off,
                                uint64_t* out) {
    constexpr uint32_t W = sizeof(RunDev) / 8;
    static_assert(sizeof(RunDev) % 8 == 0, "RunDev is copied as 8-byte words");
    __shared__ uint32_t s_best;
    const uint32_t r = blockIdx.x;
    if (r >= n) return;
    const RunDev& R = runs[r];
    const uint64_t* src = reinterpret_cast<const uint64_t*>(&R);
    for (uint32_t k = threadIdx.x; k < W; k += blockDim.x) out[(uint64_t)r * W + k] = src[k];
    double* fit = reinterpret_cast<double*>(out + (uint64_t)n * W);
    const uint32_t total = fit_off[n];
    uint8_t* cur = reinterpret_cast<uint8_t*>(fit + total);
    double* genes = reinterpret_cast<double*>(out + (uint64_t)n * W + total + (total + 7) / 8);
    for (uint32_t i = threadIdx.x; i < R.P; i += blockDim.x) {
        fit[fit_off[r] + i] = R.fit_old[i];
        cur[fit_off[r] + i] = R.cur[i];
    }
    if (threadIdx.x == 0) {
        // the first member of the strict minimum (deac.cpp:146-158), as the
        // host's summary finds it in the same values
        uint32_t best = 0;
        double mn = R.fit_old[0];
        for (uint32_t i = 0; i < R.P; ++i)
            if (R.fit_old[i] < mn) {
                mn = R.fit_old[i];
                best = i;
            }
        s_best = best;
    }
    __syncthreads();
    const uint32_t best = s_best;
    const uint64_t PM = (uint64_t)R.P * R.M;
    const double* row = R.pop + (uint64_t)R.cur[best] * R.S * PM + (uint64_t)best * R.M;
    for (uint32_t k = threadIdx.x; k < R.S * R.M; k += blockDim.x) {
        const uint32_t sd = k / R.M, j = k - sd * R.M;
        genes[gene_off[r] + k] = row[(uint64_t)sd * PM + j];
    }
}

// ------------------------------------------------------ initial population
// (x >> 11) 2^-53 (the reference's uniform, rng.hpp:129-131) from integer
// operations: the 53-bit integer's leading bit gives the exponent, the bits
// below it the fraction -- exact, and off the narrow FP64 pipe.
__device__ __forceinline__ double unit_from_bits(uint64_t x) {
    const uint64_t m = x >> 11;
    if (m == 0) return 0.0;
    const int e = 63 - __clzll((long long)m);  // 0 .. 52
    const uint64_t frac = (m << (52 - e)) & 0xFFFFFFFFFFFFFull;
    return __longlong_as_double((long long)(((uint64_t)(e - 53 + 1023) << 52) | frac));
}

__global__ void __launch_bounds__(kPopThreads) population_kernel(const PopRun* runs, const PopWork* work,
                                                                const uint64_t* jstep) {
    const PopWork w = work[blockIdx.x];
    const PopRun R = runs[w.run];
    const uint32_t P = R.P, M = R.M, S = R.S;
    const uint64_t t = (uint64_t)w.t0 + threadIdx.x;
    const uint64_t n = (uint64_t)P * M * S;
    const uint64_t d0 = t << kPopBlockLog2;
    if (d0 >= n) return;
    uint64_t v[4] = {R.s[0], R.s[1], R.s[2], R.s[3]};
    for (uint32_t b = 0; (t >> b) != 0; ++b)
        if ((t >> b) & 1u) {
            uint64_t o[4];
            gf2_matvec(jstep + (uint64_t)(b + kPopBlockLog2) * 1024, v, o);
            v[0] = o[0];
            v[1] = o[1];
            v[2] = o[2];
            v[3] = o[3];
        }
    const uint64_t d1 = d0 + (1ull << kPopBlockLog2) < n ? d0 + (1ull << kPopBlockLog2) : n;
    const uint64_t PM = (uint64_t)P * M, MS = (uint64_t)M * S;
    double* const pop = R.pop;
    // draw d is gene j, side s of member i: d = (i M + j) S + s
    uint64_t i = d0 / MS;
    uint32_t j = (uint32_t)((d0 - i * MS) / S), s = (uint32_t)(d0 - i * MS - (uint64_t)j * S);
    double first = 0.0;  // the member's positive-side gene 0 (its draw and the next are one thread's: d0 is even)
    for (uint64_t d = d0; d < d1; ++d) {
        double x = unit_from_bits(xoshiro_next(v[0], v[1], v[2], v[3]));
        if (R.signed_weights) x -= 0.5;
        if (S == 2 && j == 0) {
            if (s == 0) first = x;
            else x = first;
        }
        pop[(uint64_t)s * PM + i * M + j] = x;
        if (++s == S) {
            s = 0;
            if (++j == M) {
                j = 0;
                ++i;
            }
        }
    }
}

// ------------------------------------------------------------ PRNG table
__global__ void rng_table_kernel(uint64_t* rng, uint64_t n, const uint64_t* jpow, uint32_t bits, uint64_t s0,
                                 uint64_t s1, uint64_t s2, uint64_t s3, uint32_t P, uint32_t M, uint32_t S) {
    // a thread forms kPerThread consecutive states: the first from the
    // matrices of its index's set bits, the others one jump (J = jpow[0]) on
    constexpr uint32_t kPerThread = 8;
    const uint64_t groups = (n + kPerThread - 1) / kPerThread;
    for (uint64_t g = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; g < groups;
         g += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t k0 = g * kPerThread;
        uint64_t v[4] = {s0, s1, s2, s3};
        for (uint32_t b = 0; b < bits; ++b)
            if ((k0 >> b) & 1u) {
                uint64_t o[4];
                gf2_matvec(jpow + (uint64_t)b * 1024, v, o);
                v[0] = o[0];
                v[1] = o[1];
                v[2] = o[2];
                v[3] = o[3];
            }
        for (uint32_t i = 0; i < kPerThread && k0 + i < n; ++i) {
            if (i > 0) {
                uint64_t o[4];
                gf2_matvec(jpow, v, o);
                v[0] = o[0];
                v[1] = o[1];
                v[2] = o[2];
                v[3] = o[3];
            }
            const uint64_t slot = rng_slot(P, M, S, k0 + i);
#pragma unroll
            for (int w = 0; w < 4; ++w) rng[(uint64_t)w * n + slot] = v[w];
        }
    }
}

// --------------------------------------------------------------- split trials
// Split engine: jDE and the mutant indices of every member, one thread each
// (work = the trial work list), once after the initial population; later
// generations draw them where each member's selection becomes final
// (split_select_kernel, or the exact trial pass of contract_kernel).
__global__ void __launch_bounds__(128) jde_kernel(RunDev* runs, const Work* work, uint32_t n) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const Work w = work[k];
    RunDev& R = runs[w.run];
    if (R.done) return;
    double cr[2], fw[2];
    uint32_t mut[3];
    jde_member(R, w.index, cr, fw, mut);
    for (int q = 0; q < 3; ++q) R.mutants[3 * w.index + q] = mut[q];
}

// Split engine: the raw trial of member i, genes [part*kTrialPart, ...) of
// both sides for each part of the CTA's range -- the crossover draw and
// DE/rand/1 mutation of each gene as in trial_kernel, then the part's BF16
// digit slices.  The member's CR / F, mutants and the run's parent buffers
// are read once for the range, and each part's rows are prefetched into L2
// while the part before it is formed.  Sets the trial's `changed` flag when a
// gene mutated and raises its maximum chunk exponent (split_select_kernel
// resets both after use).
// kCounter: the batch draws from counter streams (no per-gene states in
// registers, so more CTAs fit on an SM); otherwise from the state table.
template <bool kCounter>
__device__ __forceinline__ void trial_part_body(RunDev* runs, const PartWork* work) {
    extern __shared__ __align__(16) double part_s[];  // [S][len] the part's trial genes
    __shared__ double s_fw[2];
    __shared__ uint64_t s_thr[2];
    __shared__ uint32_t s_mut[3];
    __shared__ uint64_t s_step;
    __shared__ uint8_t s_cur[kTrialPartThreads];
    __shared__ int s_digit_max[kTrialPartThreads / 32];
    // Before the wait only the static run description is read, and the
    // first part's PRNG states are prefetched into L2 meanwhile (a hint:
    // their values are read after the wait).
    const PartWork wk = work[blockIdx.x];
    RunDev& R = runs[wk.run];
    const uint32_t i = wk.member;
    const uint32_t P = R.P, M = R.M, S = R.S;
    const uint64_t PM = (uint64_t)P * M;
    const uint64_t n = R.n_states;
    const uint64_t base = (uint64_t)i * (1ull + (uint64_t)S * M);
    const uint64_t buf = (uint64_t)S * PM;
    constexpr bool counter = kCounter;
    auto part_len = [&](uint32_t part) {
        const uint32_t j0 = part * kTrialPart;
        return M - j0 < kTrialPart ? M - j0 : kTrialPart;
    };
    auto prefetch_states = [&](uint32_t part) {
        if (!counter && threadIdx.x < 4 * S)
            prefetch_l2(R.rng + (threadIdx.x / S) * n + base + 1 + (uint64_t)(threadIdx.x % S) * M +
                            part * kTrialPart,
                        part_len(part), R.rng + 4 * n);
    };
    prefetch_states(wk.part0);
    grid_dependency_wait();
    // the previous generation's exact pass is done with its item list
    if (blockIdx.x == 0 && threadIdx.x == 0) *R.exact_count = 0;
    if (R.done) return;
    // one round trip: the member's CR / F and mutant indices, and the
    // parent buffer of every member of the run (of the mutants on demand
    // when the run has more members than the CTA has threads)
    const bool table = P <= kTrialPartThreads;
    if (table && threadIdx.x < P) s_cur[threadIdx.x] = R.cur[threadIdx.x];
    if (threadIdx.x < S) {
        const double cr = R.cr[(uint64_t)S * P + threadIdx.x * P + i];
        s_thr[threadIdx.x] = crossover_threshold(cr);
        s_fw[threadIdx.x] = R.fw[(uint64_t)S * P + threadIdx.x * P + i];
    } else if (threadIdx.x >= 32 && threadIdx.x < 35) {
        s_mut[threadIdx.x - 32] = R.mutants[3 * i + threadIdx.x - 32];
    } else if (counter && threadIdx.x == 64) {
        s_step = R.rng[i] - 1;  // the jDE step this trial's CR / F and mutants come from
    }
    __syncthreads();
    const uint32_t r0 = s_mut[0], r1 = s_mut[1], r2 = s_mut[2];
    auto cur = [&](uint32_t m) -> uint64_t { return table ? s_cur[m] : R.cur[m]; };
    const uint32_t parent_buf = (uint32_t)cur(i);
    double* dst = R.pop + ((uint64_t)(1u - parent_buf) * S) * PM + (uint64_t)i * M;
    const double* pa = R.pop + cur(r0) * buf + (uint64_t)r0 * M;
    const double* pb = R.pop + cur(r1) * buf + (uint64_t)r1 * M;
    const double* pc = R.pop + cur(r2) * buf + (uint64_t)r2 * M;
    const double* px = R.pop + (uint64_t)parent_buf * buf + (uint64_t)i * M;
    const bool keep_sign = (R.flags & kSignedWeights) != 0;
    const uint64_t key_x = R.key_crossover;
    const double* rows[4] = {pa, pb, pc, px};
    bool mutated = false;
    constexpr uint32_t H = 4;  // genes in flight per thread (one pass of a 512-gene side)
    for (uint32_t part = wk.part0; part < wk.part0 + wk.nparts; ++part) {
        const uint32_t j0 = part * kTrialPart;
        const uint32_t len = part_len(part);
        // into L2 while this part is formed: this part's second side, and
        // both sides of the next part (and its PRNG states)
        if (threadIdx.x < 4 * S) {
            const uint32_t q = threadIdx.x & 3u, sd = threadIdx.x >> 2;
            if (sd == 1) prefetch_l2(rows[q] + PM + j0, len, R.pop + 2 * buf);
            if (part + 1 < wk.part0 + wk.nparts)
                prefetch_l2(rows[q] + (uint64_t)sd * PM + j0 + kTrialPart, part_len(part + 1), R.pop + 2 * buf);
        }
        if (part + 1 < wk.part0 + wk.nparts) prefetch_states(part + 1);
        for (uint32_t s = 0; s < S; ++s) {
            uint64_t* st0 = R.rng + base + 1 + (uint64_t)s * M + j0;
            // counter streams: gene j0 + k of side s draws position cpos + k
            const uint64_t cpos = counter ? ((s_step * P + i) * S + s) * (uint64_t)M + j0 : 0;
            const uint64_t off = (uint64_t)s * PM + j0;
            const double *qa = pa + off, *qb = pb + off, *qc = pc + off, *qx = px + off;
            double* qd = dst + off;
            double* qs = part_s + s * len;
            const uint64_t thr = s_thr[s];
            const double fw = s_fw[s];
            for (uint32_t j = threadIdx.x; j < len; j += H * blockDim.x) {
                uint64_t st[H][4];
                double a[H], b[H], c[H], x[H];
#pragma unroll
                for (uint32_t h = 0; h < H; ++h) {
                    const uint32_t jj = j + h * blockDim.x;
                    const uint32_t k = jj < len ? jj : j;
                    if (!counter) {
                        st[h][0] = st0[k];
                        st[h][1] = st0[n + k];
                        st[h][2] = st0[2 * n + k];
                        st[h][3] = st0[3 * n + k];
                    }
                    a[h] = qa[k];
                    b[h] = qb[k];
                    c[h] = qc[k];
                    x[h] = qx[k];
                }
#pragma unroll
                for (uint32_t h = 0; h < H; ++h) {
                    const uint32_t jj = j + h * blockDim.x;
                    if (jj >= len) continue;
                    bool mutate;
                    if (counter) {
                        mutate = (stream_draw(key_x, cpos + jj) >> 11) < thr;
                    } else {
                        mutate = (xoshiro_next(st[h][0], st[h][1], st[h][2], st[h][3]) >> 11) < thr;
                        uint64_t* so = st0 + jj;
                        so[0] = st[h][0];
                        so[n] = st[h][1];
                        so[2 * n] = st[h][2];
                        so[3 * n] = st[h][3];
                    }
                    double v = x[h];
                    mutate_gene(v, a[h], b[h], c[h], fw, mutate);
                    if (mutate) {
                        if (!keep_sign) v = abs_bits(v);
                        mutated = true;
                    }
                    qd[jj] = v;
                    qs[part_slot(jj)] = v;
                }
            }
        }
        __syncthreads();
        if (S == 2 && j0 == 0 && threadIdx.x == 0) {
            // gpu_match_population_zero (deac_gpu.cu:541-549)
            dst[PM] = part_s[part_slot(0)];
            part_s[len + part_slot(0)] = part_s[part_slot(0)];
        }
        __syncthreads();
        // (ends with a barrier after its last read of part_s)
        digitize_trial(part_s, len, S, len,
                       R.xdig + xdig_row_offset(R.xdig_row0 + i) + (uint64_t)(j0 >> 3) * R.xdig_unit, R.xdig_unit,
                       R.xdig_side, R.xexp + (uint64_t)i * split_chunks(M) + j0 / kChunk,
                       R.xexp_max + i, s_digit_max);
    }
    if (__syncthreads_or(mutated) && threadIdx.x == 0) R.changed[i] = 1;
}

__global__ void __launch_bounds__(kTrialPartThreads, 4) trial_part_kernel(RunDev* runs, const PartWork* work) {
    trial_part_body<false>(runs, work);
}
__global__ void __launch_bounds__(kTrialPartThreads, 4) trial_part_counter_kernel(RunDev* runs,
                                                                                  const PartWork* work) {
    trial_part_body<true>(runs, work);
}

// Split engine, generation 0: the digit slices of member i's parent (the
// initial population, normalised in place by trial_kernel), parts [part0,
// part0 + nparts) of 512 genes per side, so that the tensor-core contraction
// can estimate the initial fitness.  Raises the member's maximum chunk
// exponent, which the generation-0 decision resets.
__global__ void __launch_bounds__(kTrialPartThreads) parent_digits_kernel(RunDev* runs, const PartWork* work) {
    extern __shared__ __align__(16) double part_s[];  // [S][len]
    __shared__ int s_digit_max[kTrialPartThreads / 32];
    const PartWork wk = work[blockIdx.x];
    RunDev& R = runs[wk.run];
    const uint32_t i = wk.member, M = R.M, S = R.S;
    const uint64_t PM = (uint64_t)R.P * M;
    const double* src = R.pop + (uint64_t)R.cur[i] * S * PM + (uint64_t)i * M;
    for (uint32_t part = wk.part0; part < wk.part0 + wk.nparts; ++part) {
        const uint32_t j0 = part * kTrialPart;
        const uint32_t len = M - j0 < kTrialPart ? M - j0 : kTrialPart;
        for (uint32_t s = 0; s < S; ++s)
            for (uint32_t j = threadIdx.x; j < len; j += blockDim.x)
                part_s[s * len + part_slot(j)] = src[(uint64_t)s * PM + j0 + j];
        __syncthreads();
        // (ends with a barrier after its last read of part_s)
        digitize_trial(part_s, len, S, len,
                       R.xdig + xdig_row_offset(R.xdig_row0 + i) + (uint64_t)(j0 >> 3) * R.xdig_unit, R.xdig_unit,
                       R.xdig_side, R.xexp + (uint64_t)i * split_chunks(M) + j0 / kChunk, R.xexp_max + i, s_digit_max);
    }
}

// ---------------------------------------------------------------- norm
// Split engine, runs that normalise (kDeferNorm) or have moment terms: one
// CTA per raw trial forms its exact row sums (warps 0-7 the positive side,
// 8-15 the negative side, staged kNormStage genes at a time in shared
// memory).  First the normalisation sums, then norm = gemv_pair(...) and
// 1/norm exactly as trial_kernel does, setting the trial's `changed` flag
// (a mutated gene or a scale other than 1); then the first and third moment
// sums of the normalised trial -- each gene RN(x / norm) as trial_kernel
// forms it, so the moments are trial_kernel's to the bit.
__global__ void __launch_bounds__(kNormThreads) norm_kernel(RunDev* runs, const Work* work) {
    grid_dependency_wait();
    __shared__ ChainScratch s_chain[2];
    __shared__ double s_sum[2], s_recip;
    extern __shared__ __align__(16) double norm_s[];  // per side: [kNormStage] genes, [kNormStage] weights
    const Work wk = work[blockIdx.x];
    RunDev& R = runs[wk.run];
    if (R.done) return;
    const uint32_t i = wk.index;
    const uint32_t P = R.P, M = R.M, S = R.S;
    const uint64_t PM = (uint64_t)P * M;
    const uint32_t buf = 1u - R.cur[i];
    const uint32_t side = (threadIdx.x >> 5) / kChainWarps;
    const double* x = R.pop + ((uint64_t)buf * S + side) * PM + (uint64_t)i * M;
    double* s_x = norm_s + (uint64_t)side * 2 * kNormStage;
    double* s_w = s_x + kNormStage;
    const uint32_t tg = threadIdx.x - side * kChainWarps * 32;
    // the later stages' genes into L2 while the first stage's chain runs
    if (tg == 0 && side < S && M > kNormStage) prefetch_l2(x + kNormStage, M - kNormStage, x + M);
    // this side's row sum over weights wts, of the genes times rc when
    // `scaled`; each side's group runs on its own: its staging and chain
    // synchronise with the group's named barrier only
    auto side_sum = [&](const double* wts, bool scaled, double rc) -> double {
        double sum = 0.0;
        for (uint32_t k0 = 0; side < S && k0 < M; k0 += kNormStage) {
            const uint32_t len = M - k0 < kNormStage ? M - k0 : kNormStage;
            chain_detail::group_bar(1 + (int)side, kChainWarps * 32);  // the chain is done with the stage buffer
            {
                // this thread's steps tg*E .. tg*E+E-1 of the stage, all loads
                // in flight at once, stored step-major (chain_slot order) so
                // that the chain's threads read them without bank conflicts
                constexpr uint32_t E = kChainSteps, NT = kChainWarps * 32;
                double vx[E], vw[E];
                const uint32_t k = tg * E;
                if (k + E <= len) {
                    const double2* px = reinterpret_cast<const double2*>(x + k0 + k);
                    const double2* pw = reinterpret_cast<const double2*>(wts + k0 + k);
#pragma unroll
                    for (uint32_t u = 0; u < E / 2; ++u) {
                        const double2 a = px[u], b = pw[u];
                        vx[2 * u] = a.x;
                        vx[2 * u + 1] = a.y;
                        vw[2 * u] = b.x;
                        vw[2 * u + 1] = b.y;
                    }
                } else {
#pragma unroll
                    for (uint32_t u = 0; u < E; ++u) {
                        vx[u] = k + u < len ? x[k0 + k + u] : 0.0;
                        vw[u] = k + u < len ? wts[k0 + k + u] : 0.0;
                    }
                }
#pragma unroll
                for (uint32_t u = 0; u < E; ++u) {
                    s_x[u * NT + tg] = scaled ? vx[u] * rc : vx[u];
                    s_w[u * NT + tg] = vw[u];
                }
            }
            chain_detail::group_bar(1 + (int)side, kChainWarps * 32);
            sum = group_fma_chain<kChainWarps, kChainSteps, true, true>(s_x, s_w, len, sum, side * kChainWarps,
                                                                        1 + (int)side, s_chain[side],
                                                                        k0 == 0 ? 32u : 0u);
        }
        return sum;
    };
    const bool defer = (R.flags & kDeferNorm) != 0;
    if (defer) {
        const double sum = side_sum(side == 0 ? R.norm_pos : R.norm_neg, false, 1.0);
        if (tg == 0 && side < S) s_sum[side] = sum;
        __syncthreads();
        if (threadIdx.x == 0) {
            const double norm = gemv_pair(s_sum[0], S == 2 ? s_sum[1] : 0.0, R.alpha, S == 2);
            const double recip = 1.0 / norm;
            R.recip[i] = recip;
            s_recip = recip;
            if (recip != 1.0) R.changed[i] = 1;
        }
        __syncthreads();
    }
    // moment row sums with alpha = 1 (deac.cpp:1418-1477), of the trial as
    // it is kept: normalised when the run normalises
    const double rc = defer ? s_recip : 1.0;
    for (int which = 0; which < 2; ++which) {
        const uint32_t flag = which == 0 ? kFirstMoment : kThirdMoment;
        if (!(R.flags & flag)) continue;
        const double* wp = which == 0 ? R.first_pos : R.third_pos;
        const double* wn = which == 0 ? R.first_neg : R.third_neg;
        const double sum = side_sum(side == 0 ? wp : wn, defer, rc);
        if (tg == 0 && side < S) s_sum[side] = sum;
        __syncthreads();
        if (threadIdx.x == 0) R.moments[2 * i + which] = gemv_pair(s_sum[0], S == 2 ? s_sum[1] : 0.0, 1.0, S == 2);
        __syncthreads();
    }
}

// ------------------------------------------------------------- contract
// Dynamic shared memory: two stages of `chunk` genes of every pop row and K
// row the CTA needs ([S][member_tile] pop rows, then [S][tau_tile] K rows,
// row stride chunk+2), reused by the finishing CTA as 4 x 1024 reduction
// slots.
// One contraction item: tile w of run w.run in mode `mode`; in
// kModeRecheck the item's pass `pmode` is kModeParents or kModeTrials.
// `fin`: a packed tile, over the run's listed members (final_members,
// final_n) in the listed tiling instead of every member in the run's own --
// the final exact evaluations (the list is what they evaluate) and the exact
// pass (the list holds the members left open; each pass still evaluates
// only those it wants).
__device__ __forceinline__ void contract_body(RunDev* runs, const Work w, int mode, int pmode, double* dyn,
                                              bool fin = false) {
    __shared__ int s_last, s_any;
    const bool both = mode == kModeRecheck;
    RunDev& R = runs[w.run];
    const bool final_mode = mode == kModeFinal || mode == kModeFinalBest;
    if (R.done && !final_mode) return;
    if ((mode == kModeParents || mode == kModeTrials || both) && R.exact_idle) return;
    const bool init_mode = mode == kModeInit;
    // members evaluated by a pass, and which of their two buffers
    auto parents_of = [](int pm) {
        return pm == kModeInit || pm == kModeParents || pm == kModeFinal || pm == kModeFinalBest;
    };
    // kModeFinalBest: the lowest upper end of the parents' intervals (a
    // parent whose interval starts above it cannot hold the minimum)
    __shared__ double s_min_hi;
    if (mode == kModeFinalBest && !fin) {
        double mh = __longlong_as_double(0x7ff0000000000000ll);  // +inf
        for (uint32_t m = threadIdx.x; m < R.P; m += blockDim.x) mh = fmin(mh, R.f_hi[m]);
        for (int o = 16; o > 0; o >>= 1) mh = fmin(mh, __shfl_xor_sync(0xffffffffu, mh, o));
        if (threadIdx.x == 0) s_min_hi = mh;
        __syncthreads();
        if ((threadIdx.x & 31u) == 0) atomic_min_double_smem(&s_min_hi, mh);
        __syncthreads();
    }
    auto wanted_in = [&](int pm, uint32_t m) -> bool {
        if (pm == kModeGeneration) return true;
        // split engine: the members generation 0's interval left open (all
        // of them in runs whose statistics or terms need exact values)
        if (pm == kModeInit) return R.f_lo == nullptr || R.recheck[m] != 0;
        if (pm == kModeTrials) return R.recheck[m] != 0;
        const bool inexact = R.f_lo[m] != R.f_hi[m];
        if (pm == kModeFinalBest) return inexact && R.f_lo[m] <= s_min_hi;
        return pm == kModeFinal ? inexact : (R.recheck[m] != 0 && inexact);
    };
    const bool use_parent = parents_of(pmode);
    // the tile's member slots: every member in order, or the listed ones
    const uint32_t P = R.P, M = R.M, Nt = R.Nt, S = R.S;
    const uint32_t NM = fin ? R.final_n : P;
    auto member = [&](uint32_t slot) -> uint32_t { return fin ? R.final_members[slot] : slot; };
    auto wanted = [&](uint32_t m) -> bool { return (fin && final_mode) || wanted_in(pmode, m); };
    const uint32_t MT = fin ? R.final_mt : R.member_tile, TT = fin ? R.final_tt : R.tau_tile,
                   CH = fin ? R.final_chunk : R.chunk;
    const uint64_t PM = (uint64_t)P * M;
    const uint32_t member_tiles = NM ? (NM + MT - 1) / MT : 1u;
    const uint32_t mt = w.index % member_tiles, tt = w.index / member_tiles;
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    const uint32_t pair = S == 2 ? warp * 16 + (lane & 15u) : threadIdx.x;
    const uint32_t side = S == 2 ? (lane >> 4) : 0u;
    const uint32_t mi = pair % MT, ti = pair / MT;
    const uint32_t slot = mt * MT + mi, t = tt * TT + ti;
    const uint32_t i = slot < NM ? member(slot) : 0u;
    const bool valid = ti < TT && slot < NM && t < Nt && wanted(i);
    if (threadIdx.x == 0) s_any = 0;
    __syncthreads();
    if (valid) s_any = 1;
    __syncthreads();
    const uint32_t stride = stage_stride(CH);
    const uint32_t rows = S * (MT + TT);
    double* stage0 = dyn;
    double* stage1 = dyn + (uint64_t)rows * stride;
    const bool vec = (M & 1u) == 0;  // 16-byte copies need 16-byte aligned rows

    // Each thread owns fixed rows of every stage (at most two, since a stage
    // has at most 2*(64+1) rows) and a fixed stride of 16-byte units within
    // them, so issuing a copy costs one address add; resolved once here.
    const uint32_t tpr = rows >= blockDim.x ? 1u : blockDim.x / rows;  // threads per row
    const uint32_t sub = threadIdx.x % tpr;
    const uint32_t rstep = blockDim.x / tpr;
    const double* src_row[2] = {nullptr, nullptr};
    uint32_t dst_row[2] = {0u, 0u};
    {
        double* const pop = R.pop;
        const double* const kp = R.k_pos;
        const double* const kn = R.k_neg;
        for (uint32_t j = 0; j < 2; ++j) {
            const uint32_t r = threadIdx.x / tpr + j * rstep;
            if (r >= rows) break;
            dst_row[j] = r;
            if (r < S * MT) {
                const uint32_t s = r / MT, sl = mt * MT + (r - s * MT);
                const uint32_t m = sl < NM ? member(sl) : 0u;
                if (sl < NM && wanted(m)) {
                    const uint32_t bsel = use_parent ? R.cur[m] : 1u - R.cur[m];
                    src_row[j] = pop + ((uint64_t)bsel * S + s) * PM + (uint64_t)m * M;
                }
            } else {
                const uint32_t rr = r - S * MT;
                const uint32_t s = rr / TT, tau = tt * TT + (rr - s * TT);
                if (tau < Nt) src_row[j] = (s ? kn : kp) + (uint64_t)tau * M;
            }
        }
    }

    // stage `CH` genes starting at k0 of every row into buffer `b`
    auto issue = [&](double* b, uint32_t k0) {
        const uint32_t n = min(CH, M - k0);
        const uint32_t units = vec ? n / 2 : n;  // M even => k0 and n even
#pragma unroll
        for (uint32_t j = 0; j < 2; ++j) {
            if (src_row[j] == nullptr) continue;
            double* d = b + (uint64_t)dst_row[j] * stride;
            const double* src = src_row[j] + k0;
            if (vec) {
                for (uint32_t u = sub; u < units; u += tpr) cp_async16(d + 2 * u, src + 2 * u);
            } else {
                for (uint32_t u = sub; u < units; u += tpr) cp_async8(d + u, src + u);
            }
        }
        cp_async_commit();
    };

    // E[i,t]: one k-ascending FMA chain per side from 0 (gpu_matmul,
    // deac_gpu.cu:277-315), staged through shared memory, double-buffered
    double acc = 0.0;
    const uint32_t nst = s_any ? (M + CH - 1) / CH : 0u;  // nothing wanted in this tile
    if (nst) issue(stage0, 0);
    for (uint32_t st = 0; st < nst; ++st) {
        double* cur = (st & 1u) ? stage1 : stage0;
        if (st + 1 < nst) {
            issue((st & 1u) ? stage0 : stage1, (st + 1) * CH);
            cp_async_wait<1>();
        } else {
            cp_async_wait<0>();
        }
        __syncthreads();
        if (valid) {
            const double* xr = cur + (uint64_t)(side * MT + mi) * stride;
            const double* kr = cur + (uint64_t)(S * MT + side * TT + ti) * stride;
            acc = chain(xr, kr, min(CH, M - st * CH), acc);
        }
        __syncthreads();
    }
    // the two gpu_matmul calls: C = 1*c_pos + 0*C, then C = 1*c_neg + 1*C
    double e = acc;
    if (S == 2) e = __shfl_xor_sync(0xffffffffu, acc, 16) + acc;
    double* const model_out = both && pmode == kModeTrials ? R.model_isf2 : R.model_isf;
    if (valid && side == 0) model_out[(uint64_t)i * Nt + t] = e;

    // the last CTA of this run finishes the generation
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        const uint32_t done_ctas = atomicAdd(&R.ticket, 1u) + 1u;
        s_last = done_ctas == (both ? 2u : 1u) * (fin ? R.final_ctas : R.contract_ctas);
    }
    __syncthreads();
    if (!s_last) return;
    __threadfence();

    const uint32_t nwarps = blockDim.x >> 5;
    const uint32_t lanes = Nt < kTreeSlots ? Nt : kTreeSlots;
    const uint32_t width = pow2_ceil(lanes);
    double* sl = dyn + (uint64_t)warp * kTreeSlots;

    // reduced chi^2 (deac_gpu.cu:417-448) plus the moment terms
    // (deac_gpu.cu:450-456; order of deac.cpp:1479-1499), a warp per member;
    // kModeRecheck: the parents' pass, then the trials'
    for (int pass = 0; pass < (both ? 2 : 1); ++pass) {
    const int fmode = both ? (pass == 0 ? kModeParents : kModeTrials) : mode;
    const bool fit_parent = parents_of(fmode);
    double* fit_dst = fit_parent ? R.fit_old : R.fit_new;
    const volatile double* E_all = both && pass == 1 ? R.model_isf2 : R.model_isf;
    for (uint32_t k = warp; k < NM; k += nwarps) {
        const uint32_t m = member(k);
        if (!(fin && final_mode) && !wanted_in(fmode, m)) continue;  // warp-uniform
        for (uint32_t s = lane; s < width; s += 32) {
            double v = 0.0;
            for (uint32_t idx = s; idx < Nt; idx += kTreeSlots) {
                const double term = (R.isf[idx] - E_all[(uint64_t)m * Nt + idx]) / R.err[idx];
                v = fma(term, term, v);
            }
            sl[s] = v;
        }
        __syncwarp();
        const double total = warp_tree(sl, width);
        if (lane == 0) {
            double fit = total / (double)Nt;
            if (R.flags & kNegativeFirstMoment) {
                double mom = 0.0;
                for (uint32_t idx = 0; idx < Nt; ++idx) mom = fma(E_all[(uint64_t)m * Nt + idx], R.tau_w[idx], mom);
                const double term = (R.negfirst_target - mom) / R.negfirst_error;
                fit = fma(term, term, fit);
            }
            // the split engine keeps its parents' moments apart from the
            // trials' (an interval-accepted parent is evaluated again later)
            const double* mom = fit_parent && R.pmoments && fmode != kModeInit ? R.pmoments : R.moments;
            if (R.flags & kFirstMomentCpu) {
                // the CPU build's term (deac.cpp:969): a rounded square, a
                // rounded quotient and a rounded sum
                const double d = mom[2 * m] - R.first_target;
                fit = fit + (d * d) / R.first_target;
            } else if (R.flags & kFirstMoment) {
                const double term = (R.first_target - mom[2 * m]) / 1.0;
                fit = fma(term, term, fit);
            }
            if (R.flags & kThirdMoment) {
                const double term = (R.third_target - mom[2 * m + 1]) / R.third_error;
                fit = fma(term, term, fit);
            }
            if (fmode == kModeInit && R.pmoments) {
                R.pmoments[2 * m] = R.moments[2 * m];
                R.pmoments[2 * m + 1] = R.moments[2 * m + 1];
            }
            fit_dst[m] = fit;
            if (fit_parent && R.f_lo) R.f_lo[m] = R.f_hi[m] = fit;  // now exact
        }
        __syncwarp();
    }
    __syncthreads();
    }
    if (mode == kModeParents || final_mode) {
        if (threadIdx.x == 0) R.ticket = 0;
        return;  // no selection and no bookkeeping in these passes
    }

    uint64_t ii = R.ii;
    if (!init_mode) {
        // greedy selection, ties accept (deac_gpu.cu:551-582); the split
        // engine's trial pass settles only the members the intervals left open
        const int smode = both ? kModeTrials : mode;  // the members selected here
        for (uint32_t m = threadIdx.x; m < P; m += blockDim.x) {
            if (!wanted_in(smode, m)) continue;
            const double fn = R.fit_new[m];
            if ((R.flags & kTrace) && ii < R.trace_cap) R.trace[ii * P + m] = fn;
            if (fn <= R.fit_old[m]) {
                R.fit_old[m] = fn;
                if (R.f_lo) R.f_lo[m] = R.f_hi[m] = fn;
                if (R.pmoments) {
                    R.pmoments[2 * m] = R.moments[2 * m];
                    R.pmoments[2 * m + 1] = R.moments[2 * m + 1];
                }
                for (uint32_t s = 0; s < S; ++s) {
                    R.cr[s * P + m] = R.cr[(uint64_t)S * P + s * P + m];
                    R.fw[s * P + m] = R.fw[(uint64_t)S * P + s * P + m];
                }
                R.cur[m] = (uint8_t)(1u - R.cur[m]);
            }
        }
        ii += 1;
        __syncthreads();
        if (smode == kModeTrials && threadIdx.x >= 32) {
            // the next generation's jDE of the members settled here (the
            // selection kernel drew the others), beside the statistics
            for (uint32_t m = threadIdx.x - 32; m < P; m += blockDim.x - 32) {
                if (!wanted_in(smode, m)) continue;
                double cr[2], fw[2];
                uint32_t mut[3];
                jde_member(R, m, cr, fw, mut);
                for (int q = 0; q < 3; ++q) R.mutants[3 * m + q] = mut[q];
            }
        }
    }

    // top of the next generation (deac.cpp:1138-1166): statistics of the
    // parents and the stop test, done here so the host never has to look
    if (threadIdx.x < 32) {
        const volatile double* f = R.fit_old;
        if (ii + 2 <= R.N) {  // ii <= N-2: the loop continues to generation ii
            double mn = f[0];
            for (uint32_t m = 1; m < P; ++m) mn = f[m] < mn ? f[m] : mn;
            if (R.flags & kTrackStats) {
                // fitness mean and mean of squares (deac_gpu.cu:458-512)
                const uint32_t pl = P < kTreeSlots ? P : kTreeSlots;
                const uint32_t pw = pow2_ceil(pl);
                for (int sq = 0; sq < 2; ++sq) {
                    for (uint32_t s = lane; s < pw; s += 32) {
                        double v = 0.0;
                        if (s < P) v = sq ? f[s] * f[s] : f[s];
                        for (uint32_t idx = s + kTreeSlots; idx < P; idx += kTreeSlots)
                            v = sq ? fma(f[idx], f[idx], v) : v + f[idx];
                        sl[s] = v;
                    }
                    __syncwarp();
                    const double total = warp_tree(sl, pw);
                    if (lane == 0) R.stats[(uint64_t)(sq ? 2 : 0) * R.N + ii] = total / (double)P;
                    __syncwarp();
                }
                if (lane == 0) R.stats[R.N + ii] = mn;
            }
            if (lane == 0) {
                R.ii = ii;
                if (mn <= R.stop) {
                    R.generation = ii;
                    R.done = 1;
                }
            }
        } else if (lane == 0) {
            // the loop ran out: deac.cpp reports N-1 (host side)
            R.ii = ii;
            R.generation = R.N - 2;
            R.done = 1;
        }
    }
    if (threadIdx.x == 0) R.ticket = 0;
}

__global__ void __launch_bounds__(kContractThreads) contract_kernel(RunDev* runs, const Work* work, int mode) {
    grid_dependency_wait();
    extern __shared__ __align__(16) double dyn[];
    contract_body(runs, work[blockIdx.x], mode, mode, dyn);
}

// The split engine's exact pass: the items the selections left open, listed
// by split_select_kernel (run << 32 | pass << 31 | packed << 30 | tile, both
// passes of each listed run; packed: a tile of the run's listed members),
// shared out over a grid of at most one CTA per SM; with nothing listed
// every CTA returns at once.
__global__ void __launch_bounds__(kContractThreads) exact_pass_kernel(RunDev* runs, const uint64_t* list,
                                                                      const uint32_t* count) {
    // the next generation's trial parts read nothing before their own wait:
    // let them be scheduled while the selection still runs
    asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory");
    asm volatile("griddepcontrol.wait;\n" ::: "memory");
    extern __shared__ __align__(16) double dyn[];
    const uint32_t n = *reinterpret_cast<const volatile uint32_t*>(count);
    for (uint32_t k = blockIdx.x; k < n; k += gridDim.x) {
        const uint64_t e = list[k];
        const Work w{(uint32_t)(e >> 32), (uint32_t)e & 0x3FFFFFFFu};
        contract_body(runs, w, kModeRecheck, (e >> 31) & 1u ? kModeTrials : kModeParents, dyn, (e >> 30) & 1u);
        __syncthreads();  // shared memory is reused by the next item
    }
}

__global__ void final_list_kernel(RunDev* runs, int mode, uint64_t* items, uint32_t* count, uint32_t capacity,
                                  int* status) {
    RunDev& R = runs[blockIdx.x];
    const uint32_t lane = threadIdx.x, P = R.P;
    // kModeFinalBest: the lowest upper end of the parents' intervals (a
    // parent whose interval starts above it cannot hold the minimum)
    double mh = __longlong_as_double(0x7ff0000000000000ll);  // +inf
    if (mode == kModeFinalBest) {
        for (uint32_t m = lane; m < P; m += 32) mh = fmin(mh, R.f_hi[m]);
        for (int o = 16; o > 0; o >>= 1) mh = fmin(mh, __shfl_xor_sync(0xffffffffu, mh, o));
    }
    uint32_t n = 0;
    for (uint32_t m0 = 0; m0 < P; m0 += 32) {
        const uint32_t m = m0 + lane;
        const bool want = m < P && R.f_lo[m] != R.f_hi[m] && (mode != kModeFinalBest || R.f_lo[m] <= mh);
        const uint32_t mask = __ballot_sync(0xffffffffu, want);
        if (want) R.final_members[n + __popc(mask & ((1u << lane) - 1u))] = m;
        n += __popc(mask);
    }
    if (lane != 0) return;
    uint32_t mt = 1, tt = 1, chunk = 8, ctas = 0;
    if (n) final_tiling(n, R.S, R.Nt, mt, tt, chunk, ctas);
    uint32_t base = 0;
    if (ctas) {
        base = atomicAdd(count, ctas);
        if (base + ctas > capacity) {
            // (capacity covers the largest tiling of every run: not reached)
            atomicCAS(status, 0, kStatusFinalList);
            ctas = 0;
        }
    }
    R.final_n = ctas ? n : 0u;
    R.final_mt = mt;
    R.final_tt = tt;
    R.final_chunk = chunk;
    R.final_ctas = ctas;
    for (uint32_t k = 0; k < ctas; ++k) items[base + k] = ((uint64_t)blockIdx.x << 32) | k;
}

__global__ void __launch_bounds__(kContractThreads) final_exact_kernel(RunDev* runs, const uint64_t* items,
                                                                       const uint32_t* count, int mode) {
    extern __shared__ __align__(16) double dyn[];
    const uint32_t n = *reinterpret_cast<const volatile uint32_t*>(count);
    for (uint32_t k = blockIdx.x; k < n; k += gridDim.x) {
        const uint64_t e = items[k];
        contract_body(runs, Work{(uint32_t)(e >> 32), (uint32_t)e}, mode, mode, dyn, true);
        __syncthreads();  // shared memory is reused by the next item
    }
}

}  // namespace deac
