// deac_split.cu -- split-precision (BF16 digit) evaluation on tcgen05 and the
// interval selection that keeps every decision equal to the FP64 engine's.
// See deac_split.cuh for the arithmetic.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>

#include "deac_split.cuh"

namespace deac {

namespace {

constexpr int kGroups = 2 * kDigits - 1;  // a+b = 0..10; groups above kDigits-1 are dropped
constexpr int kKept = kDigits;            // groups 0..5 kept
constexpr uint32_t kTmemCols = 512;       // 6 groups x 64 + bound x 64 = 448 used
constexpr uint32_t kBoundCol = kKept * kSplitTau;
constexpr uint64_t kWaitNs = 2000000000ull;  // bounded mbarrier waits: 2 s
constexpr uint32_t kFlush = 16;            // chunks per double-float run before the FP64 fold
constexpr int kStatusWait = 1;             // status: a tensor-core completion wait gave up

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// canonical K-major, no-swizzle layout of a [rows x kdim] BF16 tile: core
// matrix (8 rows x 16 bytes) of row group rg and k group kg at
// (rg * kdim/8 + kg) * 128 bytes, row r of it at + 16 r.
__device__ __forceinline__ uint32_t canon(uint32_t row, uint32_t k, uint32_t kdim) {
    return ((row >> 3) * (kdim >> 3) + (k >> 3)) * 128u + (row & 7u) * 16u + (k & 7u) * 2u;
}

// tcgen05 shared-memory matrix descriptor (no swizzle): start, leading byte
// offset (between k-adjacent core matrices), stride byte offset (between
// row-group-adjacent core matrices), descriptor version 1.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | ((uint64_t)1 << 46);
}

// instruction descriptor: kind::f16 with BF16 A and B, FP32 D, K-major A/B
__host__ __device__ constexpr uint32_t idesc_bf16(uint32_t m, uint32_t n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((n >> 3) << 17) | ((m >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem, uint64_t da, uint64_t db, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
        "l"(da), "l"(db), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Wait for the completion of the mbarrier phase with parity `phase`, giving
// up after kWaitNs of wall time (the caller then reports an error).
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t phase) {
    const uint64_t t0 = global_ns();
    for (;;) {
        uint32_t done;
        asm volatile(
            "{\n.reg .pred p;\nmbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(smem_u32(bar)), "r"(phase)
            : "memory");
        if (done) return true;
        if (global_ns() - t0 > kWaitNs) return false;
        __nanosleep(64);
    }
}

__device__ __forceinline__ void tmem_ld8(uint32_t taddr, uint32_t v[8]) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];\n"
                 : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7])
                 : "r"(taddr));
}

__device__ __forceinline__ void cp16(void* dst, const void* src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}

// exponent field of |v| (unbiased), or -2000 for zero / subnormal
__device__ __forceinline__ int exp_of(double v) {
    const uint64_t b = (uint64_t)__double_as_longlong(v) & 0x7FFFFFFFFFFFFFFFull;
    const int ef = (int)(b >> 52);
    return ef == 0 ? -2000 : ef - 1023;
}

// fixed-point fraction floor(|v| * 2^(42-e)) for a scale 2^e > |v|
__device__ __forceinline__ uint64_t frac42(double v, int e) {
    const uint64_t b = (uint64_t)__double_as_longlong(v) & 0x7FFFFFFFFFFFFFFFull;
    const int ef = (int)(b >> 52);
    if (ef == 0) return 0;  // zero or subnormal: below every scale used here
    const uint64_t mant = (b & 0xFFFFFFFFFFFFFull) | (1ull << 52);
    const int shift = 10 + e - (ef - 1023);
    return shift >= 64 ? 0 : (mant >> shift);
}

__device__ __forceinline__ uint16_t bf16_digit(uint32_t d, bool neg) {
    const uint32_t f = __float_as_uint((float)d);  // exact: d < 128
    return (uint16_t)((f >> 16) | (neg && d ? 0x8000u : 0u));
}

__device__ __forceinline__ void two_sum_add(float& hi, float& lo, float a, float b) {
    // (hi, lo) += (a, b) in double-float arithmetic
    const float s = hi + a;
    const float bp = s - hi;
    float e = (hi - (s - bp)) + (a - bp);
    e += lo + b;
    hi = s + e;
    lo = e - (hi - s);
}

}  // namespace

// -------------------------------------------------------------- digitize
// One CTA per (run, member): a warp per 32-gene chunk computes the chunk's
// scale exponent (max over both sides) and writes the six 7-bit digit planes.
__global__ void __launch_bounds__(256) digitize_kernel(RunDev* runs, SplitRun* split, const Work* work,
                                                       int all_members) {
    __shared__ int s_max[8];
    const Work w = work[blockIdx.x];
    RunDev& R = runs[w.run];
    if (R.done) return;
    SplitRun& X = split[w.run];
    const uint32_t i = w.index;
    if (!all_members && !X.changed[i]) return;
    const uint32_t P = R.P, M = R.M, S = R.S;
    const uint64_t PM = (uint64_t)P * M;
    // digitize the member's trial (buffer 1-cur) or, with all_members, its
    // parent (initial population)
    const uint32_t buf = all_members ? R.cur[i] : 1u - R.cur[i];
    const double* row = R.pop + (uint64_t)buf * S * PM + (uint64_t)i * M;
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u, nw = blockDim.x >> 5;
    const uint32_t C = M / kChunk;
    int wmax = -2000;
    for (uint32_t c = warp; c < C; c += nw) {
        const uint32_t j = c * kChunk + lane;
        double v[2];
        int e = -2000;
        for (uint32_t s = 0; s < S; ++s) {
            v[s] = row[(uint64_t)s * PM + j];
            e = max(e, exp_of(v[s]));
        }
        for (int o = 16; o > 0; o >>= 1) e = max(e, __shfl_xor_sync(0xffffffffu, e, o));
        e = e <= -1500 ? -1000 : e + 1;  // scale 2^e > every |v| of the chunk
        for (uint32_t s = 0; s < S; ++s) {
            const uint64_t f = frac42(v[s], e);
            const bool neg = v[s] < 0.0;
            for (int b = 0; b < kDigits; ++b) {
                const uint32_t d = (uint32_t)(f >> (7 * (kDigits - 1 - b))) & 127u;
                X.xdig[((uint64_t)b * S + s) * PM + (uint64_t)i * M + j] = bf16_digit(d, neg);
            }
        }
        if (lane == 0) X.xexp[(uint64_t)i * C + c] = (int16_t)e;
        wmax = max(wmax, e);
    }
    if (lane == 0) s_max[warp] = wmax;
    __syncthreads();
    if (threadIdx.x == 0) {
        int m = -2000;
        for (uint32_t k = 0; k < nw; ++k) m = max(m, s_max[k]);
        X.xexp_max[i] = (int16_t)m;
    }
}

// ----------------------------------------------------- split contraction
// One CTA per tile of up to 128 (run, member) rows that share a kernel
// matrix, times 64 timeslices.  Thread t owns row t (TMEM lane t).  For each
// 32-gene chunk: stage the digit tiles of both operands, issue the kept digit
// pairs into six TMEM group accumulators plus one rank-1 MMA of the chunk
// scales into the bound accumulator, wait, and fold the exact group sums into
// double-float accumulators.
__global__ void __launch_bounds__(kSplitThreads, 1)
split_contract_kernel(RunDev* runs, SplitRun* split, const SplitTile* tiles, const SplitRow* rows, int* status) {
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ uint32_t s_tmem;
    __shared__ __align__(8) uint64_t s_bar;
    __shared__ int s_kexp[kSplitTau];
    __shared__ int s_kmax[kSplitTau];
    __shared__ int s_live;

    // a failed wait in an earlier launch leaves the status set: do nothing
    // more until the host has seen it
    if (*reinterpret_cast<volatile int*>(status) != 0) return;
    const SplitTile tile = tiles[blockIdx.x];
    const uint32_t tid = threadIdx.x, warp = tid >> 5;
    const RunDev& R0 = runs[tile.run0];
    const SplitRun& X0 = split[tile.run0];
    const uint32_t S = R0.S, M = R0.M, Nt = R0.Nt;
    const uint32_t C = M / kChunk;

    // which rows of the tile need an estimate this generation
    const bool has_row = tid < tile.rows;
    SplitRow my = has_row ? rows[tile.first_row + tid] : SplitRow{tile.run0, 0};
    const RunDev& R = runs[my.run];
    const SplitRun& X = split[my.run];
    const bool live = has_row && !R.done && X.changed[my.member];
    if (tid == 0) s_live = 0;
    __syncthreads();
    if (live) atomicOr(&s_live, 1);
    __syncthreads();
    if (!s_live) return;

    // shared memory: A digits [6][S] x (128 x 32), B digits [6][S] x (64 x 32),
    // bound operands A (128 x 16) and B (64 x 16), FP64 rows 128 x 64
    const uint32_t a_tile = kSplitRows * kChunk * 2;  // 8 KB
    const uint32_t b_tile = kSplitTau * kChunk * 2;   // 4 KB
    uint8_t* sA = smem;
    uint8_t* sB = sA + kDigits * S * a_tile;
    uint8_t* sAb = sB + kDigits * S * b_tile;
    uint8_t* sBb = sAb + kSplitRows * 16 * 2;

    // zero the rank-1 bound operands once (only k = 0 is written per chunk)
    for (uint32_t e = tid; e < (kSplitRows + kSplitTau) * 16; e += blockDim.x)
        reinterpret_cast<uint16_t*>(sAb)[e] = 0;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(&s_tmem)),
                     "r"(kTmemCols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&s_bar)));
        asm volatile("fence.mbarrier_init.release.cluster;\n");
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n");
    const uint32_t tmem = s_tmem;

    const uint64_t PM = (uint64_t)R.P * M;
    const uint16_t* xrow = X.xdig + (uint64_t)my.member * M;  // + (b*S + s)*PM
    const int16_t* xexp = X.xexp + (uint64_t)my.member * C;
    const int xmax = live ? X.xexp_max[my.member] : 0;
    const uint32_t tau0 = tile.tau0;
    if (tid < kSplitTau) s_kmax[tid] = (tau0 + tid < Nt) ? X0.kexp_max[tau0 + tid] : 0;

    // per-row accumulators: a double-float pair per timeslice in registers,
    // folded into an FP64 row in shared memory every kFlush chunks
    double* e64 = reinterpret_cast<double*>(sBb + kSplitTau * 16 * 2) + (uint64_t)tid * kSplitTau;
    for (int t = 0; t < kSplitTau; ++t) e64[t] = 0.0;
    float acc_hi[kSplitTau], acc_lo[kSplitTau];
#pragma unroll
    for (int t = 0; t < kSplitTau; ++t) acc_hi[t] = acc_lo[t] = 0.0f;
    auto flush = [&]() {
#pragma unroll
        for (int t = 0; t < kSplitTau; ++t) {
            e64[t] += (double)acc_hi[t] + (double)acc_lo[t];
            acc_hi[t] = acc_lo[t] = 0.0f;
        }
    };

    const uint32_t idesc = idesc_bf16(kSplitRows, kSplitTau);
    bool ok = true;
    for (uint32_t c = 0; c < C && ok; ++c) {
        const uint32_t g0 = c * kChunk;
        // --- stage this chunk's digits (16-byte units = 8 genes of a row)
        if (live) {
            for (uint32_t b = 0; b < kDigits; ++b)
                for (uint32_t s = 0; s < S; ++s) {
                    const uint16_t* src = xrow + ((uint64_t)b * S + s) * PM + g0;
                    uint8_t* dst = sA + (b * S + s) * a_tile;
#pragma unroll
                    for (uint32_t u = 0; u < kChunk / 8; ++u) cp16(dst + canon(tid, u * 8, kChunk), src + u * 8);
                }
        }
        {
            // B: thread -> (timeslice row, half of the digit/side planes)
            const uint32_t trow = tid & (kSplitTau - 1), half = tid / kSplitTau;
            if (tau0 + trow < Nt) {
                for (uint32_t q = half; q < kDigits * S; q += 2) {
                    const uint32_t b = q / S, s = q % S;
                    const uint16_t* src = X0.kdig + (((uint64_t)b * S + s) * Nt + tau0 + trow) * M + g0;
                    uint8_t* dst = sB + q * b_tile;
#pragma unroll
                    for (uint32_t u = 0; u < kChunk / 8; ++u) cp16(dst + canon(trow, u * 8, kChunk), src + u * 8);
                }
            }
        }
        asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;\n" ::: "memory");
        // bound operands: 2^(e_x - max_x) and 2^(e_K - max_K) at k = 0
        const int ex = live ? xexp[c] : -1000;
        {
            const int d = ex - xmax;
            const float v = (live && d >= -126) ? __uint_as_float((uint32_t)(d + 127) << 23) : 0.0f;
            *reinterpret_cast<uint16_t*>(sAb + canon(tid, 0, 16)) = (uint16_t)(__float_as_uint(v) >> 16);
        }
        if (tid < kSplitTau) {
            const int ek = (tau0 + tid < Nt) ? X0.kexp[(uint64_t)(tau0 + tid) * C + c] : -1000;
            s_kexp[tid] = ek;
            const int d = ek - s_kmax[tid];
            const float v = (tau0 + tid < Nt && d >= -126) ? __uint_as_float((uint32_t)(d + 127) << 23) : 0.0f;
            *reinterpret_cast<uint16_t*>(sBb + canon(tid, 0, 16)) = (uint16_t)(__float_as_uint(v) >> 16);
        }
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;\n");
        __syncthreads();
        asm volatile("tcgen05.fence::after_thread_sync;\n");

        // --- MMAs (one thread)
        if (tid == 0) {
            const uint32_t lbo = 128, sbo = (kChunk / 8) * 128;
            for (uint32_t g = 0; g < (uint32_t)kKept; ++g) {
                uint32_t first = 1;
                for (uint32_t a = 0; a <= g; ++a) {
                    const uint32_t b = g - a;
                    if (a >= (uint32_t)kDigits || b >= (uint32_t)kDigits) continue;
                    for (uint32_t s = 0; s < S; ++s)
                        for (uint32_t ks = 0; ks < kChunk / 16; ++ks) {
                            const uint64_t da =
                                smem_desc(smem_u32(sA + (a * S + s) * a_tile) + ks * 256, lbo, sbo);
                            const uint64_t db =
                                smem_desc(smem_u32(sB + (b * S + s) * b_tile) + ks * 256, lbo, sbo);
                            mma_bf16(tmem + g * kSplitTau, da, db, idesc, first ? 0u : 1u);
                            first = 0;
                        }
                }
            }
            const uint64_t dab = smem_desc(smem_u32(sAb), 128, 256);
            const uint64_t dbb = smem_desc(smem_u32(sBb), 128, 256);
            mma_bf16(tmem + kBoundCol, dab, dbb, idesc, c > 0 ? 1u : 0u);
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                smem_u32(&s_bar)));
        }
        ok = __syncthreads_and(mbar_wait(&s_bar, c & 1u)) != 0;  // uniform across the CTA
        asm volatile("tcgen05.fence::after_thread_sync;\n");
        if (!ok) break;

        // --- fold the six exact group sums of this chunk into the accumulators
        const uint32_t lane_base = tmem + ((warp * 32u) << 16);
#pragma unroll
        for (uint32_t ts = 0; ts < kSplitTau / 8; ++ts) {
            uint32_t d[kKept][8];
#pragma unroll
            for (int g = 0; g < kKept; ++g) tmem_ld8(lane_base + g * kSplitTau + ts * 8, d[g]);
            asm volatile("tcgen05.wait::ld.sync.aligned;\n");
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                // sum_g D_g 2^(7(5-g)): exact in 64 bits (every D_g < 2^24)
                long long s = 0;
#pragma unroll
                for (int g = 0; g < kKept; ++g) s += (long long)(int)__uint_as_float(d[g][j]) << (7 * (kKept - 1 - g));
                const float hi = (float)s;
                const float lo = (float)(s - (long long)hi);
                const int sc = ex + s_kexp[ts * 8 + j] - 7 * (kKept + 1);  // weight of g = 5 is 2^-49
                two_sum_add(acc_hi[ts * 8 + j], acc_lo[ts * 8 + j], ldexpf(hi, sc), ldexpf(lo, sc));
            }
        }
        if ((c + 1) % kFlush == 0) flush();
        asm volatile("tcgen05.fence::before_thread_sync;\n");
        __syncthreads();
        asm volatile("tcgen05.fence::after_thread_sync;\n");
    }
    flush();

    if (ok) {  // CTA-uniform: the .sync.aligned TMEM loads need whole warps
        // bound sums sum_c 2^(e_x + e_K), then the interval half-width
        const uint32_t lane_base = tmem + ((warp * 32u) << 16);
        for (uint32_t ts = 0; ts < kSplitTau / 8; ++ts) {
            uint32_t d[8];
            tmem_ld8(lane_base + kBoundCol + ts * 8, d);
            asm volatile("tcgen05.wait::ld.sync.aligned;\n");
            if (!live) continue;
            for (int j = 0; j < 8; ++j) {
                const uint32_t t = tau0 + ts * 8 + j;
                if (t >= Nt) continue;
                const double scale = ldexp(1.0, xmax + s_kmax[ts * 8 + j]);
                // FP32 accumulation of C terms: relative error < C * 2^-24;
                // terms that underflowed are each < 2^-126
                const double bsum = ((double)__uint_as_float(d[j]) * (1.0 + 1e-4) + (double)C * 0x1.0p-126) * scale;
                const uint64_t o = (uint64_t)my.member * Nt + t;
                X.e_mp[o] = e64[ts * 8 + j];
                // |estimate - FP64 chain| <= (2^-33.2 digits + 2^-33 chain
                // rounding + 2^-35.4 double-float + 2^-42 FP64 folds) * B_sum
                X.e_bound[o] = 0x1.0p-31 * bsum + (double)C * 0x1.0p-140;
            }
        }
    }
    if (!ok && tid == 0) atomicCAS(status, 0, kStatusWait);
    asm volatile("tcgen05.fence::before_thread_sync;\n");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(kTmemCols));
}

// ---------------------------------------------------------------- decide
// One CTA per run: the estimate's chi^2 and its interval, then the
// selection decisions that the interval settles.  Undecided members are
// flagged for the exact FP64 evaluation (contract_kernel, recheck mode).
__global__ void __launch_bounds__(256) split_decide_kernel(RunDev* runs, SplitRun* split, int init_mode) {
    RunDev& R = runs[blockIdx.x];
    if (R.done) return;
    SplitRun& X = split[blockIdx.x];
    const uint32_t P = R.P, Nt = R.Nt, S = R.S;
    const bool force_exact = (R.flags & kTrackStats) != 0;
    unsigned long long n_tie = 0, n_interval = 0, n_exact = 0;
    for (uint32_t i = threadIdx.x; i < P; i += blockDim.x) {
        X.recheck[i] = 0;
        if (!X.changed[i]) {
            // the trial is the parent: the same fitness, and ties accept
            X.t_lo[i] = X.f_lo[i];
            X.t_hi[i] = X.f_hi[i];
            R.fit_new[i] = X.f_lo[i];
            for (uint32_t s = 0; s < S; ++s) {
                R.cr[s * P + i] = R.cr[(uint64_t)S * P + s * P + i];
                R.fw[s * P + i] = R.fw[(uint64_t)S * P + s * P + i];
            }
            R.cur[i] = (uint8_t)(1u - R.cur[i]);
            ++n_tie;
            continue;
        }
        // chi^2 of the estimate and a bound on its distance from the value
        // the FP64 engine computes
        double chi = 0.0, dchi = 0.0;
        for (uint32_t t = 0; t < Nt; ++t) {
            const uint64_t o = (uint64_t)i * Nt + t;
            const double r = (R.isf[t] - X.e_mp[o]) / R.err[t];
            const double dr = X.e_bound[o] / R.err[t] * (1.0 + 0x1.0p-50) + fabs(r) * 0x1.0p-51;
            chi = fma(r, r, chi);
            dchi += (2.0 * fabs(r) + dr) * dr;
        }
        chi /= (double)Nt;
        dchi = dchi / (double)Nt * (1.0 + 0x1.0p-40) + chi * (double)(Nt + 8) * 0x1.0p-52;
        double lo = chi - dchi, hi = chi + dchi;
        X.t_lo[i] = lo;
        X.t_hi[i] = hi;
        if (lo > X.f_hi[i]) {  // certainly worse: reject
            ++n_interval;
            continue;
        }
        const bool certain_accept = hi <= X.f_lo[i];
        if (certain_accept && !force_exact && lo > R.stop) {
            // certainly no worse: accept with the interval as its fitness
            X.f_lo[i] = lo;
            X.f_hi[i] = hi;
            R.fit_old[i] = 0.5 * (lo + hi);
            for (uint32_t s = 0; s < S; ++s) {
                R.cr[s * P + i] = R.cr[(uint64_t)S * P + s * P + i];
                R.fw[s * P + i] = R.fw[(uint64_t)S * P + s * P + i];
            }
            R.cur[i] = (uint8_t)(1u - R.cur[i]);
            ++n_interval;
            continue;
        }
        X.recheck[i] = 1;  // settle with the exact FP64 value
        ++n_exact;
    }
    if (n_tie) atomicAdd(&X.counts[0], n_tie);
    if (n_interval) atomicAdd(&X.counts[1], n_interval);
    if (n_exact) atomicAdd(&X.counts[2], n_exact);
    (void)init_mode;
}

// ------------------------------------------------------------------ host
void digits_of(double v, int e, uint16_t out[kDigits]) {
    const double m = std::fabs(v);
    uint64_t f = 0;
    if (m > 0.0) {
        int ev;
        std::frexp(m, &ev);  // m = f * 2^ev, f in [0.5, 1)
        const int ef = ev - 1;
        if (ef >= -1022) {
            uint64_t bits;
            std::memcpy(&bits, &m, 8);
            const uint64_t mant = (bits & 0xFFFFFFFFFFFFFull) | (1ull << 52);
            const int shift = 10 + e - ef;
            f = shift >= 64 ? 0 : (mant >> shift);
        }
    }
    for (int b = 0; b < kDigits; ++b) {
        const uint32_t d = (uint32_t)(f >> (7 * (kDigits - 1 - b))) & 127u;
        float fd = (float)d;
        uint32_t fb;
        std::memcpy(&fb, &fd, 4);
        out[b] = (uint16_t)((fb >> 16) | ((v < 0.0 && d) ? 0x8000u : 0u));
    }
}

}  // namespace deac
