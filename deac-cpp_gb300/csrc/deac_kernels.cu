// deac_kernels.cu -- kernels of the plain FP64 engine (see deac_kernels.cuh).
// Compiled with --fmad=false: the only fused multiply-adds are the explicit
// fma() calls, placed where the reference's nvcc build fuses.
#include <cuda_runtime.h>

#include "deac_kernels.cuh"
#include "deac_rng.cuh"

namespace deac {

namespace {

constexpr int kTrialThreads = 256;
constexpr int kTailWarps = 2;      // warps of the last contract CTA that reduce chi^2
constexpr int kTreeSlots = 1024;   // GPU_BLOCK_SIZE of the reference reductions

__device__ __forceinline__ void load_state(const RunDev& R, uint64_t slot, uint64_t s[4]) {
    const uint64_t n = R.n_states;
    s[0] = R.rng[slot];
    s[1] = R.rng[n + slot];
    s[2] = R.rng[2 * n + slot];
    s[3] = R.rng[3 * n + slot];
}

__device__ __forceinline__ void store_state(const RunDev& R, uint64_t slot, const uint64_t s[4]) {
    const uint64_t n = R.n_states;
    R.rng[slot] = s[0];
    R.rng[n + slot] = s[1];
    R.rng[2 * n + slot] = s[2];
    R.rng[3 * n + slot] = s[3];
}

__device__ __forceinline__ double draw(uint64_t s[4]) {
    return to_unit(xoshiro_next(s[0], s[1], s[2], s[3]));
}

// k-ascending FMA chain from 0.0 (the inner loop of gpu_deac_gemv,
// deac_gpu.cu:359-363).
__device__ double row_chain(const double* __restrict__ x, const double* __restrict__ w, uint32_t n) {
    double acc = 0.0;
    uint32_t k = 0;
    for (; k + 4 <= n; k += 4) {
        const double x0 = x[k], x1 = x[k + 1], x2 = x[k + 2], x3 = x[k + 3];
        const double w0 = __ldg(w + k), w1 = __ldg(w + k + 1), w2 = __ldg(w + k + 2), w3 = __ldg(w + k + 3);
        acc = fma(x0, w0, acc);
        acc = fma(x1, w1, acc);
        acc = fma(x2, w2, acc);
        acc = fma(x3, w3, acc);
    }
    for (; k < n; ++k) acc = fma(x[k], __ldg(w + k), acc);
    return acc;
}

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

}  // namespace

// ---------------------------------------------------------------- trial
__global__ void __launch_bounds__(kTrialThreads)
trial_kernel(RunDev* runs, const Work* work, int init_mode, int smem_genes) {
    extern __shared__ double trial_s[];  // S*M trial genes when they fit
    __shared__ double s_cr[2], s_fw[2], s_sum[4];
    __shared__ uint32_t s_mut[3];

    const Work w = work[blockIdx.x];
    RunDev& R = runs[w.run];
    if (R.done) return;
    const uint32_t i = w.index;
    const uint32_t P = R.P, M = R.M, S = R.S;
    const uint64_t PM = (uint64_t)P * M;
    const uint32_t parent_buf = R.cur[i];
    const uint32_t dst_buf = init_mode ? parent_buf : 1u - parent_buf;
    double* dst = R.pop + ((uint64_t)dst_buf * S) * PM + (uint64_t)i * M;  // side s at + s*PM
    const bool in_smem = (uint64_t)S * M <= (uint64_t)smem_genes;
    const uint64_t base = (uint64_t)i * (1ull + (uint64_t)S * M);

    if (!init_mode) {
        if (threadIdx.x == 0) {
            // jDE (deac_gpu.cu:584-606): CR(+) on slot 0, F(+) slot 1,
            // CR(-) slot 2, F(-) slot 3; then mutant indices on slot 0
            // (deac_gpu.cu:608-633), the launch order of deac.cpp:1168-1219.
            uint64_t st[4];
            load_state(R, base, st);
            for (uint32_t s = 0; s < S; ++s) {
                uint64_t* cur = st;
                uint64_t tmp[4];
                if (s == 1) {
                    load_state(R, base + 2, tmp);
                    cur = tmp;
                }
                const double cr_old = R.cr[s * P + i];
                const double cr = draw(cur) < R.tau_cr ? draw(cur) : cr_old;
                if (s == 1) store_state(R, base + 2, tmp);
                s_cr[s] = cr;
                R.cr[(uint64_t)S * P + s * P + i] = cr;

                uint64_t fs[4];
                const uint64_t fslot = base + (s == 0 ? 1 : 3);
                load_state(R, fslot, fs);
                const double fw_old = R.fw[s * P + i];
                const double fw = draw(fs) < R.tau_f ? 2.0 * draw(fs) : fw_old;
                store_state(R, fslot, fs);
                s_fw[s] = fw;
                R.fw[(uint64_t)S * P + s * P + i] = fw;
            }
            uint64_t r0 = i, r1 = i, r2 = i;
            while (r0 == i) r0 = xoshiro_next(st[0], st[1], st[2], st[3]) % P;
            while (r1 == i || r1 == r0) r1 = xoshiro_next(st[0], st[1], st[2], st[3]) % P;
            while (r2 == i || r2 == r0 || r2 == r1) r2 = xoshiro_next(st[0], st[1], st[2], st[3]) % P;
            store_state(R, base, st);
            s_mut[0] = (uint32_t)r0;
            s_mut[1] = (uint32_t)r1;
            s_mut[2] = (uint32_t)r2;
        }
        __syncthreads();

        // crossover draw + DE/rand/1 mutation per gene
        // (deac_gpu.cu:514-539, 635-643)
        const uint32_t r0 = s_mut[0], r1 = s_mut[1], r2 = s_mut[2];
        const uint8_t b0 = R.cur[r0], b1 = R.cur[r1], b2 = R.cur[r2];
        const bool keep_sign = (R.flags & kSignedWeights) != 0;
        const uint64_t SM = (uint64_t)S * M;
        for (uint64_t q = threadIdx.x; q < SM; q += blockDim.x) {
            const uint32_t s = (uint32_t)(q / M);
            const uint32_t j = (uint32_t)(q - (uint64_t)s * M);
            uint64_t st[4];
            load_state(R, base + 1 + q, st);
            const bool mutate = draw(st) < s_cr[s];
            store_state(R, base + 1 + q, st);
            const double* side = R.pop + (uint64_t)s * PM;
            const uint64_t buf = (uint64_t)S * PM;  // stride between the two buffers
            double v;
            if (mutate) {
                const double a = side[b0 * buf + (uint64_t)r0 * M + j];
                const double b = side[b1 * buf + (uint64_t)r1 * M + j];
                const double c = side[b2 * buf + (uint64_t)r2 * M + j];
                v = fma(s_fw[s], b - c, a);
                if (!keep_sign) v = fabs(v);
            } else {
                v = side[parent_buf * buf + (uint64_t)i * M + j];
            }
            dst[(uint64_t)s * PM + j] = v;
            if (in_smem) trial_s[q] = v;
        }
        __syncthreads();
        if (S == 2 && threadIdx.x == 0) {
            // gpu_match_population_zero (deac_gpu.cu:541-549)
            const double z = in_smem ? trial_s[0] : dst[0];
            dst[PM] = z;
            if (in_smem) trial_s[M] = z;
        }
        __syncthreads();
    } else if (in_smem) {
        for (uint64_t q = threadIdx.x; q < (uint64_t)S * M; q += blockDim.x) {
            const uint32_t s = (uint32_t)(q / M);
            trial_s[q] = dst[(uint64_t)s * PM + (q - (uint64_t)s * M)];
        }
        __syncthreads();
    }

    const double* gene_pos = in_smem ? trial_s : dst;
    const double* gene_neg = in_smem ? trial_s + M : dst + PM;
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;

    if (R.flags & kNormalize) {
        // normalisation row sum and reciprocal scale
        // (deac_gpu.cu:345-374 with alpha = 1/F(0), then 406-415)
        if (lane == 0 && warp < S) s_sum[warp] = row_chain(warp == 0 ? gene_pos : gene_neg,
                                                           warp == 0 ? R.norm_pos : R.norm_neg, M);
        __syncthreads();
        const double norm = gemv_pair(s_sum[0], S == 2 ? s_sum[1] : 0.0, R.alpha, S == 2);
        const double recip = 1.0 / norm;
        for (uint64_t q = threadIdx.x; q < (uint64_t)S * M; q += blockDim.x) {
            const uint32_t s = (uint32_t)(q / M);
            const uint64_t g = (uint64_t)s * PM + (q - (uint64_t)s * M);
            const double v = (in_smem ? trial_s[q] : dst[g]) * recip;
            dst[g] = v;
            if (in_smem) trial_s[q] = v;
        }
        __syncthreads();
    }

    if (R.flags & (kFirstMoment | kThirdMoment)) {
        // moment row sums with alpha = 1 (deac.cpp:1418-1477)
        if (lane == 0) {
            const bool first = warp < 2 && (R.flags & kFirstMoment);
            const bool third = warp >= 2 && warp < 4 && (R.flags & kThirdMoment);
            const uint32_t side = warp & 1u;
            if ((first || third) && side < S) {
                const double* t = first ? (side ? R.first_neg : R.first_pos) : (side ? R.third_neg : R.third_pos);
                s_sum[warp] = row_chain(side ? gene_neg : gene_pos, t, M);
            }
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            if (R.flags & kFirstMoment)
                R.moments[2 * i] = gemv_pair(s_sum[0], S == 2 ? s_sum[1] : 0.0, 1.0, S == 2);
            if (R.flags & kThirdMoment)
                R.moments[2 * i + 1] = gemv_pair(s_sum[2], S == 2 ? s_sum[3] : 0.0, 1.0, S == 2);
        }
    }
}

// ------------------------------------------------------------- contract
__global__ void __launch_bounds__(256) contract_kernel(RunDev* runs, const Work* work, int init_mode) {
    __shared__ double slots[kTailWarps][kTreeSlots];
    __shared__ int s_last;

    const Work w = work[blockIdx.x];
    RunDev& R = runs[w.run];
    if (R.done) return;
    const uint32_t P = R.P, M = R.M, Nt = R.Nt, S = R.S;
    const uint64_t PM = (uint64_t)P * M;
    const uint32_t member_tiles = (P + R.member_tile - 1) / R.member_tile;
    const uint32_t mt = w.index % member_tiles, tt = w.index / member_tiles;
    const uint32_t i = mt * R.member_tile + threadIdx.x % R.member_tile;
    const uint32_t t = tt * R.tau_tile + threadIdx.x / R.member_tile;

    if (threadIdx.x < R.member_tile * R.tau_tile && i < P && t < Nt) {
        // E[i,t]: two k-ascending FMA chains (gpu_matmul, deac_gpu.cu:277-315,
        // called once per side: C = 1*c_pos + 0*C, then C = 1*c_neg + 1*C)
        const uint32_t buf = init_mode ? R.cur[i] : 1u - R.cur[i];
        const double* xp = R.pop + (uint64_t)buf * S * PM + (uint64_t)i * M;
        const double* kp = R.k_pos + (uint64_t)t * M;
        double cp = 0.0, cn = 0.0;
        if (S == 2) {
            const double* xn = xp + PM;
            const double* kn = R.k_neg + (uint64_t)t * M;
            uint32_t k = 0;
            // 16-byte loads need every row start 16-byte aligned: M even
            // (buffers come from cudaMalloc, 256-byte aligned)
            const uint32_t vec_end = (M & 1u) ? 0u : M;
            for (; k + 2 <= vec_end; k += 2) {
                const double2 a = *reinterpret_cast<const double2*>(xp + k);
                const double2 b = __ldg(reinterpret_cast<const double2*>(kp + k));
                const double2 c = *reinterpret_cast<const double2*>(xn + k);
                const double2 d = __ldg(reinterpret_cast<const double2*>(kn + k));
                cp = fma(a.x, b.x, cp);
                cn = fma(c.x, d.x, cn);
                cp = fma(a.y, b.y, cp);
                cn = fma(c.y, d.y, cn);
            }
            for (; k < M; ++k) {
                cp = fma(xp[k], __ldg(kp + k), cp);
                cn = fma(xn[k], __ldg(kn + k), cn);
            }
            R.model_isf[(uint64_t)i * Nt + t] = cn + cp;
        } else {
            for (uint32_t k = 0; k < M; ++k) cp = fma(xp[k], __ldg(kp + k), cp);
            R.model_isf[(uint64_t)i * Nt + t] = cp;
        }
    }

    // the last CTA of this run finishes the generation
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        const uint32_t done_ctas = atomicAdd(&R.ticket, 1u) + 1u;
        s_last = done_ctas == R.contract_ctas;
    }
    __syncthreads();
    if (!s_last) return;
    __threadfence();

    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    const uint32_t nwarps = blockDim.x >> 5;
    const uint32_t lanes = Nt < kTreeSlots ? Nt : kTreeSlots;
    const uint32_t width = pow2_ceil(lanes);
    double* fit_dst = init_mode ? R.fit_old : R.fit_new;

    // reduced chi^2 (deac_gpu.cu:417-448) plus the moment terms
    // (deac_gpu.cu:450-456; order of deac.cpp:1479-1499)
    if (warp < kTailWarps) {
        double* sl = slots[warp];
        const volatile double* E_all = R.model_isf;
        for (uint32_t m = warp; m < P; m += (nwarps < kTailWarps ? nwarps : kTailWarps)) {
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
                    for (uint32_t idx = 0; idx < Nt; ++idx)
                        mom = fma(E_all[(uint64_t)m * Nt + idx], R.tau_w[idx], mom);
                    const double term = (R.negfirst_target - mom) / R.negfirst_error;
                    fit = fma(term, term, fit);
                }
                if (R.flags & kFirstMoment) {
                    const double term = (R.first_target - R.moments[2 * m]) / 1.0;
                    fit = fma(term, term, fit);
                }
                if (R.flags & kThirdMoment) {
                    const double term = (R.third_target - R.moments[2 * m + 1]) / R.third_error;
                    fit = fma(term, term, fit);
                }
                fit_dst[m] = fit;
            }
            __syncwarp();
        }
    }
    __syncthreads();

    uint64_t ii = R.ii;
    if (!init_mode) {
        // greedy selection, ties accept (deac_gpu.cu:551-582)
        for (uint32_t m = threadIdx.x; m < P; m += blockDim.x) {
            const double fn = R.fit_new[m];
            if ((R.flags & kTrace) && ii < R.trace_cap) R.trace[ii * P + m] = fn;
            if (fn <= R.fit_old[m]) {
                R.fit_old[m] = fn;
                for (uint32_t s = 0; s < S; ++s) {
                    R.cr[s * P + m] = R.cr[(uint64_t)S * P + s * P + m];
                    R.fw[s * P + m] = R.fw[(uint64_t)S * P + s * P + m];
                }
                R.cur[m] = (uint8_t)(1u - R.cur[m]);
            }
        }
        ii += 1;
        __syncthreads();
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
                double* sl = slots[0];
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

}  // namespace deac
