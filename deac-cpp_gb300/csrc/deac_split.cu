// deac_split.cu -- split-precision (BF16 digit) evaluation on tcgen05 and the
// interval selection that keeps every decision equal to the FP64 engine's.
// See deac_split.cuh for the arithmetic.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>

#include "deac_async.cuh"
#include "deac_jde.cuh"
#include "deac_split.cuh"

namespace deac {

namespace {

constexpr int kKept = kDigits;            // digit-pair groups a+b = 0..6 kept
constexpr uint32_t kTmemCols = 512;       // 7 groups x 64 rows + bound x 64 rows = 512
constexpr int kStatusWait = 1;             // status: a tensor-core completion wait gave up

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

__device__ __forceinline__ void tmem_ld8(uint32_t taddr, uint32_t v[8]) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];\n"
                 : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7])
                 : "r"(taddr));
}

// one 3-D tiled TMA load into shared memory, completing on `bar` (tensor map
// in global memory, coordinates innermost first; the innermost one, in
// 8-byte elements, is even: a 16-byte multiple)
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int c0, int c1, int c2,
                                            uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];\n" ::"r"(smem_u32(dst)),
        "l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(smem_u32(bar))
        : "memory");
}

// Error-free transformations in FP32 (IEEE round-to-nearest; the file is
// compiled without FMA contraction): s + e == a + b exactly.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = a + b;
    const float bp = s - a;
    e = (a - (s - bp)) + (b - bp);
}
__device__ __forceinline__ void fast_two_sum(float a, float b, float& s, float& e) {  // |a| >= |b|
    s = a + b;
    e = b - (s - a);
}

// (ah, al) += (bh, bl): the accurate double-float sum of Joldes, Muller and
// Popescu (ACM TOMS 44(2), 2017, Alg. 6), relative error below 3 * 2^-48.
__device__ __forceinline__ void dw_add(float& ah, float& al, float bh, float bl) {
    float sh, sl, th, tl, vh, vl;
    two_sum(ah, bh, sh, sl);
    two_sum(al, bl, th, tl);
    sl += th;
    fast_two_sum(sh, sl, vh, vl);
    vl += tl;
    fast_two_sum(vh, vl, ah, al);
}

__device__ __forceinline__ float exp2_int(int n) {  // 2^n for -126 <= n <= 127
    return __uint_as_float((uint32_t)(n + 127) << 23);
}

// (hi, lo) *= 2^k for k <= 60: exact unless the result is subnormal (then
// each factor rounds once, by at most 2^-150)
__device__ __forceinline__ void scale_pow2(float& hi, float& lo, int k) {
    const int k1 = k < -126 ? -126 : k;
    int k2 = k - k1;
    k2 = k2 < -126 ? -126 : k2;
    const float f1 = __uint_as_float((uint32_t)(k1 + 127) << 23);
    const float f2 = __uint_as_float((uint32_t)(k2 + 127) << 23);
    hi = hi * f1 * f2;
    lo = lo * f1 * f2;
}

}  // namespace

// x 2^k as two multiplications by powers of two (exact but where the
// result leaves the double's normal range; no library call)
__device__ __forceinline__ double times_pow2(double x, int k) {
    k = k > 2046 ? 2046 : (k < -2044 ? -2044 : k);
    const int k1 = k / 2, k2 = k - k1;  // each in [-1022, 1023]
    return x * __longlong_as_double((long long)(k1 + 1023) << 52) * __longlong_as_double((long long)(k2 + 1023) << 52);
}

// The estimate of output (row rw, timeslice t) and its bound from the
// tile's summed double-float (hi, lo) and bound accumulator b (see below).
__device__ __forceinline__ void store_estimate(const RunDev& R, SplitRun& X, const SplitRow rw, uint32_t t,
                                               const SplitTile& tile, float hi, float lo, float b) {
    const double M = (double)R.M, C = (double)split_chunks(R.M), ks = (double)tile.nsplit;
    const int emax = X.xexp_max[rw.member] + X.kexp_max[t];
    // B >= sum_c 2^(e_x + e_K): FP32 sums of powers of two (relative error
    // below 2^-23 per addition), terms under 2^-126 dropped
    const double bsum = times_pow2(((double)b * (1.0 + (C + ks + 9.0) * 0x1p-23) + C * 0x1p-126), emax);
    // Error of the estimate against the FP64 chain value, in parts:
    //  digits: dropped digit pairs and remainders, 2^-45.9 2^(e_x+e_K) per
    //    product, 128 products a chunk:                    2^-38 B
    //  digit-group sums in FP32 (TwoSum cascade of seven exact terms):
    //    30 u^2 times the chunk's |terms| <= 128 2^(e_x+e_K): 2^-36 B
    //  double-float additions, 3 u^2 |partial| each, along the longest
    //    path (a split's chunks, then the combine):  depth 3 u^2 |sum|
    //  the FP64 chains themselves, 2^-53 per step of |partial sum|, and
    //    the final FP64 sum.
    // |sum| is at most 128 B in general; when every product is >= 0 the
    // partial sums are at most the value itself, bounded by E' below.
    const double depth = (double)tile.per + (double)((tile.nsplit + 7) / 8) + 10.0;
    // (hi, lo) count in units of 2^emax (the fold's scaling)
    const double e = times_pow2((double)hi + (double)lo, emax);
    const double gen = 0x1p-38 + 0x1p-36 + depth * 3.0 * 0x1p-41;  // units of B
    double eb;
    if (R.flags & kNonNegProducts) {
        const double Ep = (fabs(e) + bsum * gen * 1.01) * (1.0 + 0x1p-40);
        eb = bsum * 0x1p-38 + Ep * ((M + 1.0) * 0x1p-53 + 0x1p-43 + depth * 3.0 * 0x1p-48 + 0x1p-51);
    } else {
        eb = bsum * (gen + M * 0x1p-46 + 0x1p-45);
    }
    // Absolute terms: subnormal roundings of the scaled chunk sums (2^-149
    // each, a few per chunk, in units of 2^emax), and the values below the
    // double's normal range, which the digits drop: at most M genes or K
    // entries per output, each product below 2^-1022 times the other
    // operand's largest scale.
    const double absolute = times_pow2((C + ks + 10.0) * 0x1p-140, emax) + times_pow2(M, X.xexp_max[rw.member] - 1022) +
                            times_pow2(M, X.kexp_max[t] - 1022);
    const uint64_t o = (uint64_t)rw.member * R.Nt + t;
    X.e_mp[o] = e;
    X.e_bound[o] = eb * (1.0 + 0x1p-40) + absolute * (1.0 + 0x1p-40);
}

// ----------------------------------------------------- split contraction
// Wait for the mbarrier phase with parity `phase` to complete, giving up when
// another role of the CTA gave up (*abort) or after kWaitNs (then setting
// *abort, which makes every role of the CTA leave its loop).
__device__ __forceinline__ bool mbar_wait_or(uint64_t* bar, uint32_t phase, volatile int* abort) {
    if (mbar_try(bar, phase)) return true;
    const uint64_t t0 = global_ns();
    for (;;) {
        if (mbar_try(bar, phase)) return true;
        if (*abort) return false;
        if (global_ns() - t0 > kWaitNs) {
            *abort = 1;
            return false;
        }
    }
}

__device__ __forceinline__ void tma_load_5d(void* dst, const CUtensorMap* map, int c0, int c1, int c2, int c3, int c4,
                                            uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, "
        "%5, %6}], [%7];\n" ::"r"(smem_u32(dst)),
        "l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(c4), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(smem_u32(bar)));
}

// One CTA per (tile, chunk range).  The tile is 128 timeslices (MMA M, one
// TMEM lane each) x 64 trial rows in two halves of 32, each half with its own
// TMEM buffer of 256 columns: seven group accumulators of 32 columns and the
// bound accumulator.  A chunk's operands arrive in two 16-gene stages (one
// per MMA K step), each with its own full / empty barriers.  Warp roles:
//  producer warp: per chunk the exponents of its 128 timeslices and 64 rows
//    and the bound operands 2^(e - max) (two buffers; written once the fold
//    is done with the chunk two before), then per stage, once the MMAs of the
//    chunk before are done with it, the digit planes of both operands by TMA;
//  MMA warp (one thread): per stage and half -- the half's buffer free once
//    the fold has read the chunk before -- for each K digit d and side one
//    MMA over the trial digits 0..6-d (N = 32(7-d)) into groups d..6, the
//    half's bound MMA with the second stage; commits per half (accumulators
//    full) and per stage (operands free);
//  16 fold warps: per half, read all seven exact group sums of their rows
//    into registers, release the buffer at once, and fold the sums into
//    double-float accumulators while the tensor cores go on.
// Every wait is bounded; a CTA that gives up reports it in *status.
// One CTA per SM: 18 warps, so two SM sub-partitions hold 5 warps each,
// and a sub-partition's 16K registers cap a thread at 96 (5 x 32 x 96 <=
// 16384; more is refused at launch).
__global__ void __maxnreg__(96)
split_contract_kernel(RunDev* runs, SplitRun* split, const SplitTile* tiles, const SplitWork* work,
                      const SplitRow* rows, const CUtensorMap* maps, float4* partial, int* status) {
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ uint32_t s_tmem;
    __shared__ __align__(8) uint64_t s_full[2];    // a stage's digit planes have landed
    __shared__ __align__(8) uint64_t s_empty[2];   // the MMAs are done with a stage
    __shared__ __align__(8) uint64_t s_scales[2];  // a chunk's exponents and bound operands are written
    __shared__ __align__(8) uint64_t s_tfull[2];   // a half's accumulators hold the chunk's sums
    __shared__ __align__(8) uint64_t s_tempty[2];  // the fold warps have read a half's accumulators
    __shared__ __align__(8) uint64_t s_mma_done;   // every MMA issued has completed
    __shared__ int s_ek[2][kTauTile], s_ex[2][kRowTile];
    __shared__ int s_kmax[kTauTile], s_xmax[kRowTile];
    __shared__ int s_live;
    __shared__ int s_abort;
    __shared__ uint32_t s_armed[2];  // phases of each stage armed (arrivals made) so far

    const SplitWork wk = work[blockIdx.x];
    const SplitTile tile = tiles[wk.tile];
    const uint32_t tid = threadIdx.x, warp = tid >> 5, lane = tid & 31u;
    const RunDev& R0 = runs[tile.run0];
    const SplitRun& X0 = split[tile.run0];
    const uint32_t S = R0.S, M = R0.M, Nt = R0.Nt;
    const uint32_t C = split_chunks(M);
    const uint32_t tau0 = tile.tau0;
    const uint32_t nchunks = wk.c1 - wk.c0;
    constexpr uint32_t kProducerWarp = kFoldWarps, kMmaWarp = kFoldWarps + 1;
    constexpr uint32_t kBufCols = 256;  // TMEM columns per half: 7 x 32 group sums, then the bound
    constexpr uint32_t kBoundCol = kKept * kHalfRows;

    // shared memory: two operand stages (16 genes each; a chunk streams
    // through them in four) of [K digits: 7S planes x 2 units x 128 x 16 B]
    // [trials: S x 2 units x 2 halves x 7 digits x 32 x 16 B], then two
    // buffers of the bound operands (128 x 16 and 64 x 16, canonical)
    const uint32_t a_stage = kDigits * S * (2 * kTauTile * 16);  // 56 KB for two sides
    const uint32_t b_stage = kDigits * S * (2 * kRowTile * 16);  // 28 KB
    auto sA = [&](uint32_t ks) { return smem + ks * (a_stage + b_stage); };
    auto sB = [&](uint32_t ks) { return smem + ks * (a_stage + b_stage) + a_stage; };
    constexpr uint32_t kBoundBytes = (kTauTile + kRowTile) * 16 * 2;
    uint8_t* const sBound = smem + 2 * (a_stage + b_stage);
    auto sAb = [&](uint32_t buf) { return sBound + buf * kBoundBytes; };
    auto sBb = [&](uint32_t buf) { return sBound + buf * kBoundBytes + kTauTile * 16 * 2; };
    const CUtensorMap* map_k = maps + 2 * tile.group;
    const CUtensorMap* map_x = maps + 2 * tile.group + 1;
    // stage q of chunk c into buffer sb: units 8c + 2q and 8c + 2q + 1 of
    // both operands
    auto load_k = [&](uint32_t c, uint32_t q, uint32_t sb) {
        tma_load_3d(sA(sb), map_k, (int)(2 * tau0), (int)(c * (kChunk / 8) + 2 * q), 0, &s_full[sb]);
    };
    auto load_x = [&](uint32_t c, uint32_t q, uint32_t sb) {
        tma_load_5d(sB(sb), map_x, 0, 0, (int)(2 * (tile.grow0 / kRowTile)), (int)(c * (kChunk / 8) + 2 * q), 0,
                    &s_full[sb]);
    };
    // operand stages of chunk c: four, or two for a final 32-gene chunk
    auto chunk_stages = [&](uint32_t c) {
        const uint32_t left = (M - c * kChunk) / kStage;
        return left < (uint32_t)(kChunk / kStage) ? left : (uint32_t)(kChunk / kStage);
    };

    // the bound operands are written at k = 0 only: zero both buffers once
    for (uint32_t e = tid; e < kBoundBytes; e += blockDim.x) reinterpret_cast<uint16_t*>(sBound)[e] = 0;
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(&s_tmem)),
                     "r"(kTmemCols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
    }
    if (tid == 0) {
        for (int q = 0; q < 2; ++q) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&s_full[q])));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&s_empty[q])));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&s_scales[q])));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&s_tfull[q])));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(&s_tempty[q])), "r"(kFoldWarps));
        }
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&s_mma_done)));
        asm volatile("fence.mbarrier_init.release.cluster;\n");
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        s_abort = 0;
        s_armed[0] = s_armed[1] = 0;
        // K is constant: the first chunk's first two K stages load while
        // the trial kernel ends
        for (uint32_t q = 0; q < 2; ++q) {
            mbar_add_tx(&s_full[q], a_stage);
            load_k(wk.c0, q, q);
        }
    }
    if (tid < kTauTile) s_kmax[tid] = (tau0 + tid < Nt) ? X0.kexp_max[tau0 + tid] : 0;

    // everything below reads what the trial kernel wrote
    grid_dependency_wait();
    // is any row of the tile a trial of a running run?  (Nothing is done
    // either after a failed wait in an earlier launch, until the host has
    // seen the status; one thread reads it so the CTA agrees.)
    if (tid == 0) s_live = *reinterpret_cast<volatile int*>(status) != 0 ? -1 : 0;
    __syncthreads();
    if (s_live == 0 && tid < tile.rows) {
        const SplitRow rw = rows[tile.first_row + tid];
        if (!runs[rw.run].done) atomicOr(&s_live, 1);
    }
    __syncthreads();
    if (s_live <= 0) {
        // nothing to do: let the K loads land, then release TMEM
        if (tid == 0)
            for (uint32_t ks = 0; ks < 2; ++ks) {
                mbar_arrive(&s_full[ks]);
                mbar_wait(&s_full[ks], 0);
            }
        asm volatile("tcgen05.fence::before_thread_sync;\n");
        __syncthreads();
        if (warp == 0)
            asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(s_tmem), "r"(kTmemCols));
        return;
    }
    if (tid >= kTauTile && tid < kTauTile + kRowTile) {
        const uint32_t r = tid - kTauTile;
        int m = 0;
        if (r < tile.rows) {
            const SplitRow rw = rows[tile.first_row + r];
            m = split[rw.run].xexp_max[rw.member];
        }
        s_xmax[r] = m;
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n");
    __syncthreads();  // s_kmax, s_xmax, the barriers, the TMEM address
    asm volatile("tcgen05.fence::after_thread_sync;\n");
    const uint32_t tmem = s_tmem;
    volatile int* abort = &s_abort;
    bool ok = true;

    if (warp == kProducerWarp) {
        // ---- producer: exponents, bound operands and operand stages
        // lane l: timeslices l + 32q (q < 4), rows l + 32q (q < 2)
        const int16_t* krow[4];
        const int16_t* xrow[2];
#pragma unroll
        for (uint32_t q = 0; q < 4; ++q) {
            const uint32_t t = lane + 32 * q;
            krow[q] = tau0 + t < Nt ? X0.kexp + (uint64_t)(tau0 + t) * C : nullptr;
        }
#pragma unroll
        for (uint32_t q = 0; q < 2; ++q) {
            const uint32_t r = lane + 32 * q;
            xrow[q] = nullptr;
            if (r < tile.rows) {
                const SplitRow rw = rows[tile.first_row + r];
                xrow[q] = split[rw.run].xexp + (uint64_t)rw.member * C;
            }
        }
        int pk[4], px[2];
        auto load_scales = [&](uint32_t c) {
#pragma unroll
            for (uint32_t q = 0; q < 4; ++q) pk[q] = krow[q] ? (int)krow[q][c] : -1000;
#pragma unroll
            for (uint32_t q = 0; q < 2; ++q) px[q] = xrow[q] ? (int)xrow[q][c] : -1000;
        };
        auto pow2_bf16 = [](int d, bool valid) -> uint16_t {
            const float v = (valid && d >= -126) ? __uint_as_float((uint32_t)(d + 127) << 23) : 0.0f;
            return (uint16_t)(__float_as_uint(v) >> 16);
        };
        load_scales(wk.c0);
        uint32_t n = 0;  // operand stages issued: stage n goes to buffer n & 1
        for (uint32_t it = 0; it < nchunks && ok; ++it) {
            const uint32_t c = wk.c0 + it, buf = it & 1u;
            // the chunk's operand stages, each once the MMAs are done with the
            // stage two before (which used the same buffer)
            if (lane == 0) {
                const uint32_t nst = chunk_stages(c);
                for (uint32_t q = 0; q < nst && ok; ++q, ++n) {
                    const uint32_t sb = n & 1u;
                    if (n < 2) {
                        mbar_expect_tx(&s_full[sb], b_stage);  // K in flight since the start
                        load_x(c, q, sb);
                    } else {
                        if (!mbar_wait_or(&s_empty[sb], ((n - 2) >> 1) & 1u, abort)) {
                            ok = false;
                            break;
                        }
                        mbar_expect_tx(&s_full[sb], a_stage + b_stage);
                        load_k(c, q, sb);
                        load_x(c, q, sb);
                    }
                    s_armed[sb] = (n >> 1) + 1;
                }
                // the exponents' buffer is free once the fold warps are done
                // with the chunk before's second half (so with the chunk two
                // before, the buffer's last user)
                if (ok && it > 0) ok = mbar_wait_or(&s_tempty[1], (it - 1) & 1u, abort);
            }
            ok = __shfl_sync(0xffffffffu, ok ? 1 : 0, 0) != 0;
            if (!ok) break;
#pragma unroll
            for (uint32_t q = 0; q < 4; ++q) {
                const uint32_t t = lane + 32 * q;
                s_ek[buf][t] = pk[q];
                *reinterpret_cast<uint16_t*>(sAb(buf) + canon(t, 0, 16)) = pow2_bf16(pk[q] - s_kmax[t], krow[q]);
            }
#pragma unroll
            for (uint32_t q = 0; q < 2; ++q) {
                const uint32_t r = lane + 32 * q;
                s_ex[buf][r] = px[q];
                *reinterpret_cast<uint16_t*>(sBb(buf) + canon(r, 0, 16)) = pow2_bf16(px[q] - s_xmax[r], xrow[q]);
            }
            asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
            __syncwarp();
            if (lane == 0) mbar_arrive(&s_scales[buf]);
            if (it + 1 < nchunks) load_scales(c + 1);
        }
    } else if (warp == kMmaWarp) {
        // ---- MMA issue (one thread)
        if (lane == 0) {
            const uint32_t idesc_b = idesc_bf16(kTauTile, kHalfRows);
            uint32_t n = 0;  // operand stages consumed (stage n in buffer n & 1)
            for (uint32_t it = 0; it < nchunks && ok; ++it) {
                const uint32_t buf = it & 1u;
                const uint32_t nst = chunk_stages(wk.c0 + it);
                for (uint32_t q = 0; q < nst && ok; ++q, ++n) {
                    const uint32_t sb = n & 1u;
                    const bool last = q + 1 == nst;
                    ok = mbar_wait_or(&s_full[sb], (n >> 1) & 1u, abort);
                    if (ok && last) ok = mbar_wait_or(&s_scales[buf], (it >> 1) & 1u, abort);
                    for (uint32_t h = 0; h < 2 && ok; ++h) {
                        // the buffer of half h: read by the fold for the chunk before
                        if (q == 0 && it > 0) ok = mbar_wait_or(&s_tempty[h], (it - 1) & 1u, abort);
                        if (!ok) break;
                        asm volatile("tcgen05.fence::after_thread_sync;\n");
                        const uint32_t d_half = tmem + h * kBufCols;
                        // K planes: units 128 timeslice rows apart; trial
                        // digits of half h: units 2 x 7 x 32 rows apart,
                        // digits 32 rows apart, rows 16 bytes
                        const uint64_t dA = smem_desc(smem_u32(sA(sb)), kTauTile * 16, 128);
                        const uint64_t dB = smem_desc(smem_u32(sB(sb)) + h * kDigits * kHalfRows * 16,
                                                      2 * kDigits * kHalfRows * 16, 128);
                        constexpr uint32_t a_plane = 2 * kTauTile * 16 / 16;          // a K plane, 16-byte units
                        constexpr uint32_t b_side = 2 * 2 * kDigits * kHalfRows;     // a side of the trials
#pragma unroll
                        for (uint32_t d = 0; d < (uint32_t)kDigits; ++d)
#pragma unroll
                            for (uint32_t s2 = 0; s2 < 2; ++s2) {
                                if (s2 >= S) continue;
                                const uint64_t da = dA + (uint64_t)((d * S + s2) * a_plane);
                                const uint64_t db = dB + (uint64_t)(s2 * b_side);
                                // groups d..6 (trial digits 0..6-d); the chunk's
                                // first MMA of a half clears its groups
                                mma_bf16(d_half + d * kHalfRows, da, db, idesc_bf16(kTauTile, kHalfRows * (kDigits - d)),
                                         (q | d | s2) ? 1u : 0u);
                            }
                        if (last) {
                            // the bound: sum_c 2^(e_x-max_x) 2^(e_K-max_K), rank 1
                            const uint64_t dab = smem_desc(smem_u32(sAb(buf)), 128, 256);
                            const uint64_t dbb = smem_desc(smem_u32(sBb(buf)) + h * (kHalfRows / 8) * 256, 128, 256);
                            mma_bf16(d_half + kBoundCol, dab, dbb, idesc_b, it > 0 ? 1u : 0u);
                            mma_commit(&s_tfull[h]);
                        }
                    }
                    if (ok) mma_commit(&s_empty[sb]);
                }
            }
            // every MMA issued completes before TMEM is released
            mma_commit(&s_mma_done);
            if (!mbar_wait_or(&s_mma_done, 0, abort)) ok = false;
        }
    } else {
        // ---- fold warps
        // warp w reads TMEM lane quarter w % 4 (a tcgen05.ld rule): timeslice
        // tl; of each half the 8 rows 8 (w / 4) .. 8 (w / 4) + 7
        const uint32_t quarter = warp & 3u, slice = warp >> 2;
        const uint32_t tl = quarter * 32 + lane;
        const uint32_t lane_base = tmem + ((quarter * 32u) << 16);
        float acc_hi[16], acc_lo[16];  // [h * 8 + j]: row 32 h + 8 slice + j
#pragma unroll
        for (uint32_t r = 0; r < 16; ++r) acc_hi[r] = acc_lo[r] = 0.0f;
        for (uint32_t it = 0; it < nchunks && ok; ++it) {
            const uint32_t buf = it & 1u;
            ok = mbar_wait_or(&s_scales[buf], (it >> 1) & 1u, abort);
            if (!ok) break;
            const int kd = s_ek[buf][tl] - s_kmax[tl];
#pragma unroll
            for (uint32_t h = 0; h < 2; ++h) {
                ok = mbar_wait_or(&s_tfull[h], it & 1u, abort);
                if (!ok) break;
                asm volatile("tcgen05.fence::after_thread_sync;\n");
                // the half's 8 rows: all their group sums into registers at
                // once, then the buffer is released -- the next chunk's MMAs
                // of this half may start -- and folded meanwhile
                uint32_t dg[kKept][8];
#pragma unroll
                for (int g = 0; g < kKept; ++g) tmem_ld8(lane_base + h * kBufCols + g * kHalfRows + 8 * slice, dg[g]);
                asm volatile("tcgen05.wait::ld.sync.aligned;\n");
                asm volatile("tcgen05.fence::before_thread_sync;\n");
                __syncwarp();
                if (lane == 0) mbar_arrive(&s_tempty[h]);  // the buffer is free for the next chunk
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    const uint32_t r = h * kHalfRows + 8 * slice + j;
                    // sum_g D_g 2^(7(6-g)) as a double-float: every term is exact
                    float sh = __uint_as_float(dg[0][j]) * exp2_int(7 * (kKept - 1)), sl = 0.0f;
#pragma unroll
                    for (int g = 1; g < kKept; ++g) {
                        float e;
                        two_sum(sh, __uint_as_float(dg[g][j]) * exp2_int(7 * (kKept - 1 - g)), sh, e);
                        sl += e;
                    }
                    float hi, lo;
                    fast_two_sum(sh, sl, hi, lo);
                    // weight of the lowest kept group, 2^(e_x + e_K - 56), in
                    // units of the output's largest scale 2^(max_x + max_K):
                    // the accumulators stay inside the FP32 range whatever
                    // the magnitude of K (e^{-tau omega} spans hundreds of
                    // binades)
                    scale_pow2(hi, lo, (s_ex[buf][r] - s_xmax[r]) + kd - 7 * (kKept + 1));
                    dw_add(acc_hi[h * 8 + j], acc_lo[h * 8 + j], hi, lo);
                }
            }
        }
        if (ok) {
            // the estimates (a tile with one CTA) or the partial sums, and the
            // bound accumulators sum_c 2^(e_x-max_x + e_K-max_K)
#pragma unroll
            for (uint32_t h = 0; h < 2; ++h) {
                uint32_t bd[8];
                tmem_ld8(lane_base + h * kBufCols + kBoundCol + 8 * slice, bd);
                asm volatile("tcgen05.wait::ld.sync.aligned;\n");
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    const uint32_t r = h * kHalfRows + 8 * slice + j;
                    if (tile.nsplit == 1) {
                        const uint32_t t = tau0 + tl;
                        if (r >= tile.rows || t >= Nt) continue;
                        const SplitRow rw = rows[tile.first_row + r];
                        const RunDev& R = runs[rw.run];
                        if (R.done) continue;
                        store_estimate(R, split[rw.run], rw, t, tile, acc_hi[h * 8 + j], acc_lo[h * 8 + j],
                                       __uint_as_float(bd[j]));
                    } else {
                        partial[(uint64_t)wk.block * kPartialBlock + (uint64_t)r * kTauTile + tl] =
                            make_float4(acc_hi[h * 8 + j], acc_lo[h * 8 + j], __uint_as_float(bd[j]), 0.0f);
                    }
                }
            }
        }
    }

    if (*abort && tid == 0) atomicCAS(status, 0, kStatusWait);
    asm volatile("tcgen05.fence::before_thread_sync;\n");
    __syncthreads();
    if (*abort && tid == kProducerWarp * 32) {
        // a CTA that gave up: the copies it issued land before it exits
        // (bounded; the MMA thread has waited for its MMAs above).  A stage's
        // latest armed phase is the only one that can be in flight.
        for (uint32_t ks = 0; ks < 2; ++ks) {
            const uint32_t n = s_armed[ks];
            if (n == 0) continue;
            mbar_wait(&s_full[ks], (n - 1) & 1u);
        }
    }
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(kTmemCols));
}

// ------------------------------------------------------------- combine
// A CTA per 32 (row, timeslice) outputs of a tile: warp w adds the partial
// sums of the splits w, w+8, ... for its lane's output (coalesced 512-byte
// loads, eight in flight), then lane-wise the eight warps' sums are added in
// a fixed order and turned into the estimate and its error bound.
__global__ void __launch_bounds__(256) split_combine_kernel(RunDev* runs, SplitRun* split, const SplitTile* tiles,
                                                            const uint32_t* combine_tiles, const SplitRow* rows,
                                                            const float4* partial) {
    grid_dependency_wait();
    __shared__ float4 s_part[8][32];
    const SplitTile tile = tiles[combine_tiles[blockIdx.x / kCombineCtasPerTile]];
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    const uint32_t idx = (blockIdx.x % kCombineCtasPerTile) * 32 + lane;
    const uint32_t r = idx / kTauTile, tl = idx % kTauTile;
    // rows and timeslices outside the tile or not evaluated this generation
    // are summed anyway (uniform control flow) and not written
    float hi = 0.0f, lo = 0.0f, b = 0.0f;
    const float4* p = partial + (uint64_t)tile.block0 * kPartialBlock + idx;
    constexpr uint32_t kAhead = 8;
    for (uint32_t s0 = warp; s0 < tile.nsplit; s0 += 8 * kAhead) {
        float4 v[kAhead];
#pragma unroll
        for (uint32_t u = 0; u < kAhead; ++u) {
            const uint32_t s = s0 + 8 * u;
            v[u] = s < tile.nsplit ? p[(uint64_t)s * kPartialBlock] : make_float4(0.f, 0.f, 0.f, 0.f);
        }
#pragma unroll
        for (uint32_t u = 0; u < kAhead; ++u) {
            dw_add(hi, lo, v[u].x, v[u].y);
            b += v[u].z;
        }
    }
    s_part[warp][lane] = make_float4(hi, lo, b, 0.0f);
    __syncthreads();
    if (warp != 0 || r >= tile.rows) return;
    hi = lo = b = 0.0f;
    for (uint32_t w = 0; w < 8; ++w) {
        const float4 v = s_part[w][lane];
        dw_add(hi, lo, v.x, v.y);
        b += v.z;
    }
    const SplitRow rw = rows[tile.first_row + r];
    const RunDev& R = runs[rw.run];
    SplitRun& X = split[rw.run];
    const uint32_t t = tile.tau0 + tl;
    if (R.done || t >= R.Nt) return;
    store_estimate(R, X, rw, t, tile, hi, lo, b);
}

// The same sums for batches whose tiles are split over at most
// kCombineWideSplits CTAs: a thread per output adds its tile's partial
// sums in order (no warp has to share the splits), 256 outputs a CTA.
__global__ void __launch_bounds__(256) split_combine_wide_kernel(RunDev* runs, SplitRun* split,
                                                                 const SplitTile* tiles,
                                                                 const uint32_t* combine_tiles,
                                                                 const SplitRow* rows, const float4* partial) {
    grid_dependency_wait();
    const SplitTile tile = tiles[combine_tiles[blockIdx.x / kCombineWideCtasPerTile]];
    const uint32_t idx = (blockIdx.x % kCombineWideCtasPerTile) * 256 + threadIdx.x;
    const uint32_t r = idx / kTauTile, tl = idx % kTauTile;
    if (r >= tile.rows) return;
    float hi = 0.0f, lo = 0.0f, b = 0.0f;
    const float4* p = partial + (uint64_t)tile.block0 * kPartialBlock + idx;
    float4 v[kCombineWideSplits];
#pragma unroll
    for (uint32_t u = 0; u < kCombineWideSplits; ++u)
        v[u] = u < tile.nsplit ? p[(uint64_t)u * kPartialBlock] : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (uint32_t u = 0; u < kCombineWideSplits; ++u) {
        dw_add(hi, lo, v[u].x, v[u].y);
        b += v[u].z;
    }
    const SplitRow rw = rows[tile.first_row + r];
    const RunDev& R = runs[rw.run];
    SplitRun& X = split[rw.run];
    const uint32_t t = tile.tau0 + tl;
    if (R.done || t >= R.Nt) return;
    store_estimate(R, X, rw, t, tile, hi, lo, b);
}

// ------------------------------------------------- chi^2 and its interval
// One timeslice's term of chi^2 from the estimate em (of the raw trial when
// `defer`, to be scaled by rc = 1/norm) with its bound eb0, and of the bound
// on chi^2's distance from the value the FP64 engine computes (any summation
// order: the rounding term covers n-term sums).  kDeferNorm: the kept trial
// is RN(gene / norm) per gene; scaled estimate and bound: the raw bound twice
// over (its FP64-chain term counts normalised genes, whose scale exponents
// can exceed the raw ones times 1/norm by a factor two), 0.001 of it more
// for the per-gene roundings (at most 2^-47 B while the raw bound is at
// least 2^-33 B), and 2^-51 |E| for the product's rounding.  The bound is
// formed in FP64 rounded upward (every term is non-negative, so each rounding
// up keeps an upper bound): early in a run with sigma far below F's scale
// the residuals reach 1e130 sigma and more, beyond the float range.
__device__ __forceinline__ void chi_term(double em, double eb0, double f, double ie, bool defer, double rc,
                                         double& chi, double& dchi) {
    const double e = defer ? em * rc : em;
    // r carries up to three roundings of 2^-53 each
    const double r = (f - e) * ie;
    chi = fma(r, r, chi);
    const double ar = fabs(r);
    const double eb =
        defer ? __dadd_ru(__dmul_ru(__dmul_ru(2.001, eb0), fabs(rc)), __dmul_ru(fabs(e), 0x1p-51)) : eb0;
    const double dr = __dadd_ru(__dmul_ru(__dmul_ru(eb, ie), 1.0 + 0x1p-20), __dmul_ru(ar, 0x1p-51));
    dchi = __fma_ru(__dadd_ru(2.0 * ar, dr), dr, dchi);
}

// The interval [lo, hi] holding the FP64 engine's fitness, from the summed
// chi (any order) and bound dchi: /Nt as a product with 1/Nt rounded once
// (two roundings where a quotient has one, covered by two more units of the
// slack), then the exact moment terms (mom1, mom3: the member's first and
// third moments) added as contract_kernel adds them -- each step is
// monotone in the fitness so far, so the interval's ends map to the ends.
__device__ __forceinline__ void chi_interval(const RunDev& R, double chi, double dchi, double inv_nt, double mom1,
                                             double mom3, double& lo, double& hi) {
    const uint32_t Nt = R.Nt;
    chi *= inv_nt;
    const double dchi_d = __dadd_ru(__dmul_ru(__dmul_ru(dchi, inv_nt), 1.0 + 0x1p-50),
                                    __dmul_ru(__dmul_ru(chi, (double)(Nt + 10)), 0x1p-52));
    lo = __dsub_rd(chi, dchi_d);
    hi = __dadd_ru(chi, dchi_d);
    if (R.flags & kFirstMomentCpu) {
        const double d = mom1 - R.first_target, q = (d * d) / R.first_target;
        lo = lo + q;
        hi = hi + q;
    } else if (R.flags & kFirstMoment) {
        const double t1 = (R.first_target - mom1) / 1.0;
        lo = fma(t1, t1, lo);
        hi = fma(t1, t1, hi);
    }
    if (R.flags & kThirdMoment) {
        const double t3 = (R.third_target - mom3) / R.third_error;
        lo = fma(t3, t3, lo);
        hi = fma(t3, t3, hi);
    }
}

// ---------------------------------------------------------------- select
// One CTA per member, in roles.  Warps 0-3 form the estimate's chi^2 and
// its interval and make the selection decision the interval settles
// (undecided members are flagged for the exact FP64 evaluation,
// contract_kernel's recheck mode); thread 0 then keeps the run's tallies,
// and the run's last CTA does the generation's bookkeeping when no member
// needs the exact pass.  Warps 4-14 meanwhile load the raw trial of
// kDeferNorm runs and, once the decision is known, normalise it when it is
// kept or rechecked; the last warp's first thread draws the next
// generation's jDE, which it stores once the decision is known.
// kThreads: kSelectThreads, or kSelectLeanThreads (no scaling warps) for
// batches without kDeferNorm runs.
template <uint32_t kThreads>
__device__ __forceinline__ void split_select_body(RunDev* runs, SplitRun* split, const Work* work) {
    grid_dependency_wait();
    constexpr uint32_t kChiWarps = 4, kChiThreads = kChiWarps * 32;
    __shared__ double s_chi[kChiWarps];
    __shared__ double s_dchi[kChiWarps];
    __shared__ int s_outcome;
    enum { kReject = 0, kAccept = 1, kRecheck = 2, kSame = 3 };
    const Work wk = work[blockIdx.x];
    RunDev& R = runs[wk.run];
    SplitRun& X = split[wk.run];
    if (R.done) return;
    const uint32_t i = wk.index;
    const uint32_t P = R.P, Nt = R.Nt, S = R.S, M = R.M;
    const bool defer = (R.flags & kDeferNorm) != 0;
    // statistics need every parent's exact fitness; the negative first
    // moment is formed from the model ISF itself: both decided exactly
    const bool force_exact = (R.flags & (kTrackStats | kNegativeFirstMoment)) != 0;
    const uint32_t tid = threadIdx.x, warp = tid >> 5, lane = tid & 31u;
    constexpr uint32_t kJdeThread = kThreads - 32;
    // read by every thread before thread 0 may change them, in one round
    // trip with the chi^2 warps' first timeslice and the generation index
    const uint32_t cur0 = R.cur[i];
    const bool changed = X.changed[i] != 0;
    const double rc = defer ? R.recip[i] : 1.0;
    const bool t0_ok = tid < kChiThreads && tid < Nt;
    const uint64_t o0 = (uint64_t)i * Nt + tid;
    const double em0 = t0_ok ? X.e_mp[o0] : 0.0, eb00 = t0_ok ? X.e_bound[o0] : 0.0;
    const double f0 = t0_ok ? R.isf[tid] : 0.0, ie0 = t0_ok ? X.inv_err[tid] : 0.0;
    const uint64_t ii0 = tid == 0 ? R.ii : 0;  // changed only by the run's bookkeeping below
    double fit_kept = tid == 0 ? R.fit_old[i] : 0.0;  // the member's fitness after the selection
    // the decision's other operands (thread 0)
    const double f_lo0 = tid == 0 ? X.f_lo[i] : 0.0, f_hi0 = tid == 0 ? X.f_hi[i] : 0.0;
    const double inv_nt = tid == 0 ? X.inv_nt : 0.0, stop = tid == 0 ? R.stop : 0.0;
    // the trial's exact moments (norm_kernel) for the moment terms
    const double mom1 = tid == 0 && (R.flags & kFirstMoment) ? R.moments[2 * i] : 0.0;
    const double mom3 = tid == 0 && (R.flags & kThirdMoment) ? R.moments[2 * i + 1] : 0.0;
    double cr_t[2] = {0.0, 0.0}, fw_t[2] = {0.0, 0.0};  // the trial's CR / F, kept on acceptance
    if (tid == 0) {
#pragma unroll
        for (uint32_t s = 0; s < 2; ++s)
            if (s < S) {
                cr_t[s] = R.cr[(uint64_t)S * P + s * P + i];
                fw_t[s] = R.fw[(uint64_t)S * P + s * P + i];
            }
    }
    __syncthreads();

    if (warp == kJdeThread / 32) {
        // the member's jDE slots and both halves of its CR / F (the
        // parent's, the trial's); every draw is made now, the selection only
        // picks the CR / F they apply to
        uint64_t jst[4][4];
        double cr2[2][2], fw2[2][2];  // [parent, trial][side]
        JdeDraws jd;
        if (tid == kJdeThread) {
            jde_load(R, i, jst);
#pragma unroll
            for (uint32_t h = 0; h < 2; ++h)
#pragma unroll
                for (uint32_t s = 0; s < 2; ++s) {
                    cr2[h][s] = s < S ? R.cr[(uint64_t)h * S * P + s * P + i] : 0.0;
                    fw2[h][s] = s < S ? R.fw[(uint64_t)h * S * P + s * P + i] : 0.0;
                }
            jde_draws(R, i, jst, jd);
        }
        // the decision (warp 0 arrives once s_outcome is written)
        asm volatile("barrier.sync 2, 64;" ::: "memory");
        if (tid == kJdeThread) {
            const int outcome = s_outcome;
            // the next generation's jDE once the selection is final (the
            // exact passes leave the member alone); the exact trial pass
            // draws the others
            if (outcome != kRecheck) {
                double cr_old[2], fw_old[2], cr_new[2], fw_new[2];
                // the CR / F the selection kept: the trial's unless rejected
                const uint32_t h = outcome == kReject ? 0u : 1u;
#pragma unroll
                for (uint32_t s = 0; s < 2; ++s) {
                    cr_old[s] = h ? cr2[1][s] : cr2[0][s];
                    fw_old[s] = h ? fw2[1][s] : fw2[0][s];
                }
                jde_apply(jd, cr_old, fw_old, cr_new, fw_new);
                jde_store(R, i, jst, cr_new, fw_new, jd.mut, true);
            }
            // the next generation's trial parts set the flag and raise the maximum
            X.changed[i] = 0;
            X.xexp_max[i] = (int32_t)0x80808080;
        }
        return;
    }
    constexpr uint32_t NS = kThreads - kChiThreads - 32;  // threads of the scaling warps
    if constexpr (NS > 0) if (warp >= kChiWarps) {
        // The trial (buffer 1 - cur) of kDeferNorm runs, kept or rechecked,
        // normalised: every gene times 1/norm, as trial_kernel does.  Its
        // genes are loaded while warps 0-3 decide (all loads of the first
        // pass in flight at once: one pass for M = 4096); the FP64
        // multiplies wait for the decision, which has the narrow FP64 pipe
        // to itself meanwhile, and are skipped for a rejected trial.
        const bool need = defer && changed;
        const uint64_t PM = (uint64_t)P * M;
        const uint32_t half = M / 2, pairs = S * half;  // M is a multiple of the 32-gene chunk: gene pairs
        constexpr uint32_t U = 12;
        double2* const row0 = reinterpret_cast<double2*>(R.pop + (uint64_t)(1u - cur0) * S * PM + (uint64_t)i * M);
        // pair q of side 1 lies PM doubles (PM/2 pairs) beyond the same pair of side 0
        auto at = [&](uint32_t q) { return q < half ? row0 + q : row0 + PM / 2 + (q - half); };
        const uint32_t q0 = tid - kChiThreads;
        double2 v[U];
        if (need) {
#pragma unroll
            for (uint32_t u = 0; u < U; ++u) {
                const uint32_t q = q0 + u * NS;
                if (q < pairs) v[u] = *at(q);
            }
        }
        // the decision (warp 0 arrives once s_outcome is written)
        asm volatile("barrier.sync 3, %0;" ::"r"(NS + 32) : "memory");
        const int outcome = s_outcome;
        if (need && (outcome == kAccept || outcome == kRecheck)) {
#pragma unroll
            for (uint32_t u = 0; u < U; ++u) {
                const uint32_t q = q0 + u * NS;
                if (q < pairs) *at(q) = make_double2(v[u].x * rc, v[u].y * rc);
            }
            for (uint32_t qb = q0 + U * NS; qb < pairs; qb += U * NS) {
#pragma unroll
                for (uint32_t u = 0; u < U; ++u) {
                    const uint32_t q = qb + u * NS;
                    if (q < pairs) v[u] = *at(q);
                }
#pragma unroll
                for (uint32_t u = 0; u < U; ++u) {
                    const uint32_t q = qb + u * NS;
                    if (q < pairs) *at(q) = make_double2(v[u].x * rc, v[u].y * rc);
                }
            }
        }
        return;
    }

    // ---- warps 0-3: the decision
    if (!changed) {
        if (tid == 0) {
            // the trial is the parent: the same fitness, and ties accept
            X.recheck[i] = 0;
            X.t_lo[i] = f_lo0;
            X.t_hi[i] = f_hi0;
            R.fit_new[i] = f_lo0;
#pragma unroll
            for (uint32_t s = 0; s < 2; ++s)
                if (s < S) {
                    R.cr[s * P + i] = cr_t[s];
                    R.fw[s * P + i] = fw_t[s];
                }
            R.cur[i] = (uint8_t)(1u - cur0);
            s_outcome = kSame;
        }
    } else {
        // chi^2 of the estimate and a bound on its distance from the value
        // the FP64 engine computes (chi_term)
        double chi = 0.0, dchi = 0.0;
        if (t0_ok) chi_term(em0, eb00, f0, ie0, defer, rc, chi, dchi);
        for (uint32_t t = tid + kChiThreads; t < Nt; t += kChiThreads) {
            const uint64_t o = (uint64_t)i * Nt + t;
            chi_term(X.e_mp[o], X.e_bound[o], R.isf[t], X.inv_err[t], defer, rc, chi, dchi);
        }
        for (int o = 16; o > 0; o >>= 1) {
            chi += __shfl_xor_sync(0xffffffffu, chi, o);
            dchi = __dadd_ru(dchi, __shfl_xor_sync(0xffffffffu, dchi, o));
        }
        if (lane == 0) {
            s_chi[warp] = chi;
            s_dchi[warp] = dchi;
        }
        asm volatile("barrier.sync 1, %0;" ::"r"(kChiThreads) : "memory");
        if (tid == 0) {
            // the warps' sums (any order: the bound covers it)
            chi = (s_chi[0] + s_chi[1]) + (s_chi[2] + s_chi[3]);
            dchi = __dadd_ru(__dadd_ru(s_dchi[0], s_dchi[1]), __dadd_ru(s_dchi[2], s_dchi[3]));
            X.recheck[i] = 0;
            double lo, hi;
            chi_interval(R, chi, dchi, inv_nt, mom1, mom3, lo, hi);
            X.t_lo[i] = lo;
            X.t_hi[i] = hi;
            int outcome;
            if (lo > f_hi0) {  // certainly worse: reject
                outcome = kReject;
            } else if (hi <= f_lo0 && !force_exact && lo > stop) {
                // certainly no worse: accept with the interval as its fitness
                X.f_lo[i] = lo;
                X.f_hi[i] = hi;
                fit_kept = 0.5 * (lo + hi);
                R.fit_old[i] = fit_kept;
                if (R.flags & (kFirstMoment | kThirdMoment)) {
                    R.pmoments[2 * i] = mom1;
                    R.pmoments[2 * i + 1] = mom3;
                }
#pragma unroll
                for (uint32_t s = 0; s < 2; ++s)
                    if (s < S) {
                        R.cr[s * P + i] = cr_t[s];
                        R.fw[s * P + i] = fw_t[s];
                    }
                R.cur[i] = (uint8_t)(1u - cur0);
                outcome = kAccept;
            } else {
                X.recheck[i] = 1;  // settle with the exact FP64 value
                outcome = kRecheck;
            }
            s_outcome = outcome;
        }
    }
    if (warp != 0) return;
    __syncwarp();
    // the decision to the jDE warp and the scaling warps, without waiting
    asm volatile("barrier.arrive 2, 64;" ::: "memory");
    if constexpr (NS > 0) asm volatile("barrier.arrive 3, %0;" ::"r"(NS + 32) : "memory");
    if (tid != 0) return;
    const int outcome = s_outcome;
    // the run's tallies: the members' fitness minimum (non-negative doubles
    // order as their bit patterns) and the outcome counts; then the ticket,
    // which counts the members through (low word) and those left for the
    // exact pass (high word)
    atomicMin(&X.sel_min_bits, (unsigned long long)__double_as_longlong(fit_kept));
    atomicAdd(&X.counts[outcome == kSame ? 0 : outcome == kRecheck ? 2 : 1], 1ull);
    const unsigned long long mine = 1ull + (outcome == kRecheck ? (1ull << 32) : 0ull);
    __threadfence();
    const unsigned long long before = atomicAdd(&X.sel_ticket, mine);
    if ((uint32_t)before == P - 1) {
        // The run's last member: with nothing left for the exact passes,
        // finish the generation here -- the bookkeeping of contract_kernel's
        // trial pass (generation index, minimum and stop test); the fitness
        // of an interval-accepted member lies above the stop fitness, so its
        // midpoint decides the stop test exactly.  Runs that track
        // statistics keep the exact pass, which forms them.
        const uint32_t nre = (uint32_t)((before + mine) >> 32);
        __threadfence();
        const double mn =
            __longlong_as_double((long long)*reinterpret_cast<volatile unsigned long long*>(&X.sel_min_bits));
        X.sel_ticket = 0;
        X.sel_min_bits = ~0ull;
        const bool idle = nre == 0 && !force_exact;
        R.exact_idle = idle ? 1 : 0;
        if (!idle) {
            // list both passes of the run for the exact pass: tiles packed
            // with the members left open (ascending), so that the FP64
            // chains run on them alone -- or, with none left open (a run that
            // keeps the exact pass for its statistics), the run's own tiles,
            // whose last CTA does the bookkeeping
            uint32_t n = 0;
            for (uint32_t m = 0; m < P; ++m)
                if (*reinterpret_cast<const volatile uint8_t*>(X.recheck + m)) R.final_members[n++] = m;
            uint32_t ctas = R.contract_ctas, packed = 0;
            if (n) {
                uint32_t mt, tt, chunk;
                final_tiling(n, S, R.Nt, mt, tt, chunk, ctas, kExactMinMembers);
                R.final_n = n;
                R.final_mt = mt;
                R.final_tt = tt;
                R.final_chunk = chunk;
                R.final_ctas = ctas;
                packed = 1;
            }
            const uint32_t base = atomicAdd(R.exact_count, 2 * ctas);
            for (uint32_t k = 0; k < 2 * ctas; ++k) {
                const uint64_t pass = k >= ctas ? 1u : 0u;
                R.exact_list[base + k] =
                    ((uint64_t)wk.run << 32) | (pass << 31) | ((uint64_t)packed << 30) | (pass ? k - ctas : k);
            }
        }
        if (idle) {
            const uint64_t ii = ii0 + 1;
            R.ii = ii;
            if (ii + 2 > R.N) {
                R.generation = R.N - 2;
                R.done = 1;
            } else if (mn <= R.stop) {
                R.generation = ii;
                R.done = 1;
            }
        }
    }
}

__global__ void __launch_bounds__(kSelectThreads) split_select_kernel(RunDev* runs, SplitRun* split,
                                                                     const Work* work) {
    split_select_body<kSelectThreads>(runs, split, work);
}
__global__ void __launch_bounds__(kSelectLeanThreads) split_select_lean_kernel(RunDev* runs, SplitRun* split,
                                                                              const Work* work) {
    split_select_body<kSelectLeanThreads>(runs, split, work);
}

// ------------------------------------------------------ generation 0
// Split engine, generation 0: one CTA (kInitThreads) per member.  The
// initial parent's fitness as the interval of the tensor-core estimate (its
// digits by parent_digits_kernel; normalised in place already, so no 1/norm
// is deferred) plus the exact moment terms of trial_kernel's initial pass.
// An interval above the stop fitness stands as the parent's fitness (its
// midpoint in fit_old); the others, and every member of a run whose
// statistics or negative-first-moment term need exact values, are flagged
// for contract_kernel's initial pass, which evaluates just those exactly
// and does generation 0's bookkeeping.  Resets the member's `changed` flag
// and maximum chunk exponent for the first generation's trials.
__global__ void __launch_bounds__(kInitThreads) split_init_kernel(RunDev* runs, SplitRun* split, const Work* work) {
    __shared__ double s_chi[kInitThreads / 32], s_dchi[kInitThreads / 32];
    const Work wk = work[blockIdx.x];
    RunDev& R = runs[wk.run];
    SplitRun& X = split[wk.run];
    const uint32_t i = wk.index, Nt = R.Nt;
    const uint32_t tid = threadIdx.x, warp = tid >> 5, lane = tid & 31u;
    const bool force_exact = (R.flags & (kTrackStats | kNegativeFirstMoment)) != 0;
    double chi = 0.0, dchi = 0.0;
    if (!force_exact)
        for (uint32_t t = tid; t < Nt; t += kInitThreads) {
            const uint64_t o = (uint64_t)i * Nt + t;
            chi_term(X.e_mp[o], X.e_bound[o], R.isf[t], X.inv_err[t], false, 1.0, chi, dchi);
        }
    for (int o = 16; o > 0; o >>= 1) {
        chi += __shfl_xor_sync(0xffffffffu, chi, o);
        dchi = __dadd_ru(dchi, __shfl_xor_sync(0xffffffffu, dchi, o));
    }
    if (lane == 0) {
        s_chi[warp] = chi;
        s_dchi[warp] = dchi;
    }
    __syncthreads();
    if (tid != 0) return;
    X.changed[i] = 0;
    X.xexp_max[i] = (int32_t)0x80808080;
    if (force_exact) {
        X.recheck[i] = 1;
        return;
    }
    chi = (s_chi[0] + s_chi[1]) + (s_chi[2] + s_chi[3]);
    dchi = __dadd_ru(__dadd_ru(s_dchi[0], s_dchi[1]), __dadd_ru(s_dchi[2], s_dchi[3]));
    const double mom1 = (R.flags & kFirstMoment) ? R.moments[2 * i] : 0.0;
    const double mom3 = (R.flags & kThirdMoment) ? R.moments[2 * i + 1] : 0.0;
    double lo, hi;
    chi_interval(R, chi, dchi, X.inv_nt, mom1, mom3, lo, hi);
    if (lo > R.stop) {
        X.f_lo[i] = lo;
        X.f_hi[i] = hi;
        R.fit_old[i] = 0.5 * (lo + hi);
        if (R.pmoments) {
            R.pmoments[2 * i] = mom1;
            R.pmoments[2 * i + 1] = mom3;
        }
        X.recheck[i] = 0;
    } else {
        X.recheck[i] = 1;  // settle with the exact FP64 value
    }
}

// ------------------------------------------------------------ K digits
__global__ void k_digits_kernel(const double* kp, const double* kn, uint32_t Nt, uint32_t M, uint16_t* kdig,
                                int16_t* kexp, int16_t* kexp_max) {
    __shared__ int s_max[8];
    const uint32_t t = blockIdx.x, warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    const uint32_t S = kn ? 2u : 1u, C = split_chunks(M), nw = blockDim.x >> 5;
    int wmax = -1000;
    // the exponents of the normal values (zeros, subnormals and non-finite
    // values set no scale, as std::isnormal on the host)
    auto ex = [](double v) { const int e = exp_of(v); return e > 1023 ? -2000 : e; };
    for (uint32_t c = warp; c < C; c += nw) {
        // lane: genes 64c + lane and 64c + 32 + lane (the second absent in
        // a final 32-gene chunk)
        double v[2][2];
        int e = -2000;
#pragma unroll
        for (uint32_t h = 0; h < 2; ++h) {
            const uint32_t j = c * kChunk + h * 32 + lane;
            const bool in = j < M;
            v[h][0] = in ? kp[(uint64_t)t * M + j] : 0.0;
            v[h][1] = in && kn ? kn[(uint64_t)t * M + j] : 0.0;
            e = max(e, max(ex(v[h][0]), ex(v[h][1])));
        }
        for (int o = 16; o > 0; o >>= 1) e = max(e, __shfl_xor_sync(0xffffffffu, e, o));
        e = e <= -1500 ? -1000 : e + 1;  // scale 2^e above every |v| of the chunk
#pragma unroll
        for (uint32_t h = 0; h < 2; ++h) {
            const uint32_t j = c * kChunk + h * 32 + lane;
            if (j >= M) continue;
            for (uint32_t sd = 0; sd < S; ++sd) {
                const double x = v[h][sd];
                const uint64_t f = frac_digits(x, e);
                const bool neg = x < 0.0;
                for (int d = 0; d < kDigits; ++d) {
                    const uint32_t dg = (uint32_t)(f >> (7 * (kDigits - 1 - d))) & 127u;
                    kdig[((((uint64_t)d * S + sd) * (M / 8) + j / 8) * Nt + t) * 8 + (j & 7u)] = bf16_digit(dg, neg);
                }
            }
        }
        if (lane == 0) kexp[(uint64_t)t * C + c] = (int16_t)e;
        wmax = max(wmax, e);
    }
    if (lane == 0) s_max[warp] = wmax;
    __syncthreads();
    if (threadIdx.x == 0) {
        int m = -1000;
        for (uint32_t k = 0; k < nw; ++k) m = max(m, s_max[k]);
        kexp_max[t] = (int16_t)m;
    }
}

}  // namespace deac
