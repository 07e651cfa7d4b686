// deac_split.cuh -- the split-precision evaluation of the contraction on the
// tcgen05 tensor cores, used by DEAC_ENGINE_SPLIT_BF16.
//
// E[i,t] = sum_k x[i,k] K[t,k] (both sides) is evaluated from exact BF16
// digit slices:  every value v of a 64-gene chunk is written as
//     v = sign * 2^e * sum_{b=0..6} d_b 2^(-7(b+1)) + r,   0 <= d_b <= 127,
// with one power-of-two scale 2^e per (row, chunk) shared by both sides
// (|r| < 2^(e-49)).  Digit products d_a d'_b <= 127^2 and a group of equal
// weight (a+b = g, g <= 6: at most 7 pairs) summed over 64 genes x 2 sides
// is at most 7 * 128 * 127^2 = 14,451,584 < 2^24 in magnitude, so the
// tensor core's FP32 accumulation of each group is exact (the last chunk of
// a genome whose size is an odd multiple of 32 has 32 genes).  Per chunk the
// seven group sums are combined into a double-float (FP32 pair) value,
// scaled by 2^(e_x + e_K - 56) relative to the output's largest scale and
// added to double-float accumulators; CTAs split the chunks of a tile and a
// combine kernel adds their partial sums when a tile has several.  What is
// dropped -- remainders and digit pairs with a+b > 6 -- is below 2^-45.9 *
// 2^(e_x+e_K) per product, and the bound's chunk sums B = sum_c 2^(e_x+e_K)
// are accumulated by one extra rank-1 MMA per chunk.  With the rounding
// bounds of the double-float steps and of the FP64 chain itself this gives
// an interval that contains the value the plain FP64 engine computes, so
// selection decisions made from it are the FP64 decisions (deac_kernels.cuh,
// contract_kernel).
//
// Digit planes are stored pre-tiled for the tensor memory accelerator, rows
// 16 bytes (8 genes) wide.
//  K (the A operand, rows = timeslices): plane q = digit*S + side, then
//    units of 8 genes, then timeslices: element (q, t, gene j) at
//        ((q * M/8 + j/8) * Nt + t) * 8 + j%8.
//    A unit's timeslices are consecutive, so one 3-D box {128 timeslices x
//    16 bytes (as 8-byte elements), 4 units, 7S planes} -- 2 KB lines --
//    lands in shared memory as [plane][unit][timeslice][8].
//  Trials (the B operand, rows = members of the runs sharing K, in 64-row
//    tiles of two 32-row halves): side, then unit, then (tile, half), then
//    digit, then the half's 32 rows: element (s, row, digit d, gene j) at
//        ((((s * M/8 + j/8) * H + row/32) * 7 + d) * 32 + row%32) * 8 + j%8
//    with H = 2 * (64-row tiles).  One 5-D box {32 rows x 16 bytes, 7
//    digits, 2 halves, 4 units, S sides} -- 512-byte lines -- lands as
//    [side][unit][half][digit][row][8]: for a half, the rows of consecutive
//    digits follow each other, so one MMA of N = 32 n rows takes n digits.
// Both are the canonical K-major no-swizzle operand layout: core matrices 8
// rows apart (128 bytes), the two 8-gene halves of a 16-gene MMA step one
// unit apart.
#pragma once

#include <cuda.h>

#include <cstdint>

#include "deac_kernels.cuh"

namespace deac {

constexpr int kDigits = 7;         // 7-bit digits per value (49 bits)
constexpr int kDigitBits = 7 * kDigits;
constexpr int kChunk = 64;         // genes per scale chunk
constexpr int kStage = 16;         // genes per operand stage (one MMA K step)
constexpr int kGeneStep = 32;      // the split engine's genome sizes are multiples of this
// scale chunks of a genome of M genes (the last one 32 genes when M is an
// odd multiple of 32)
__host__ __device__ inline uint32_t split_chunks(uint64_t M) { return (uint32_t)((M + kChunk - 1) / kChunk); }
constexpr int kTauTile = 128;      // MMA M: timeslices, one TMEM lane each
constexpr int kRowTile = 64;       // trial rows per output tile
constexpr int kHalfRows = 32;      // rows per TMEM buffer (a tile's half)
constexpr int kFoldWarps = 16;     // fold warps: four per TMEM lane quarter, 8 rows of each half each
// split_contract_kernel: the fold warps, a producer warp (TMA loads and the
// chunk scales) and an MMA warp
constexpr int kSplitThreads = (kFoldWarps + 2) * 32;
// elements between a half's digit blocks in the trial planes (32 rows x 8)
constexpr uint64_t kXdigDigit = (uint64_t)kHalfRows * 8;
// the trial planes' element offset of `row` (within its group) at unit 0,
// side 0, digit 0
__host__ __device__ inline uint64_t xdig_row_offset(uint32_t row) {
    return ((uint64_t)(row >> 5) * kDigits * kHalfRows + (row & 31u)) * 8;
}
constexpr int kSelectThreads = 512;
// dynamic shared memory of split_contract_kernel for S sides: two operand
// stages of K digits [7][S] x (128 x 16) and trial digits [7][S] x (64 x 16),
// and two buffers of the bound operands (128 x 16, 64 x 16)
constexpr uint32_t split_smem_bytes(uint32_t S) {
    return 2 * ((uint32_t)kDigits * S * (kTauTile * kStage * 2) + (uint32_t)kDigits * S * (kRowTile * kStage * 2)) +
           2 * (kTauTile + kRowTile) * 16 * 2;
}

// Split-engine buffers of one run (device pointers).
struct SplitRun {
    int16_t* xexp;       // [P][split_chunks(M)] chunk scale exponents of the trial
    const uint16_t* kdig;  // tiled digit planes of K, rows = timeslices (shared)
    const int16_t* kexp;   // [Nt][split_chunks(M)]
    const int16_t* kexp_max;  // [Nt] max over chunks
    int32_t* xexp_max;   // [P] max over chunks
    double* e_mp;        // [P][Nt] split estimate of the model ISF
    double* e_bound;     // [P][Nt] bound on |estimate - FP64 chain value|
    uint8_t* changed;    // [P] trial differs from its parent
    uint8_t* recheck;    // [P] needs the exact FP64 evaluation
    double* f_lo;        // [P] interval of the parent's exact fitness
    double* f_hi;
    double* t_lo;        // [P] interval of the trial's exact fitness
    double* t_hi;
    unsigned long long* counts;  // [3]: trials equal to the parent, settled by
                                 // the interval, settled by the exact FP64 value
    unsigned long long sel_ticket;  // this generation: members through split_select_kernel (low
                                    // word) and of them left for the exact pass (high word)
    unsigned long long sel_min_bits;  // their fitness minimum (bits; all ones: none yet)
    const double* inv_err;  // [Nt] 1/sigma, rounded once
    double inv_nt;            // 1/Nt, rounded once
};

// One output tile: up to 64 (run, member) rows sharing one K, x 128
// timeslices, whose chunks are split over `nsplit` CTAs; their partial sums
// are the blocks block0 .. block0+nsplit-1 of the partial buffer.
struct SplitTile {
    uint32_t tau0;       // first timeslice
    uint32_t first_row;  // index into the row list
    uint32_t rows;       // valid rows (<= 64)
    uint32_t run0;       // a run of the tile (for the shared K pointers)
    uint32_t nsplit;
    uint32_t block0;
    uint32_t per;        // chunks of its longest split
    uint32_t group;      // runs sharing K: index of its tensor maps
    uint32_t grow0;      // first row within the group's trial digit planes
};
// One CTA of split_contract_kernel: chunks [c0, c1) of a tile.
struct SplitWork {
    uint32_t tile, c0, c1, block;
};
struct SplitRow {
    uint32_t run, member;
};
// partial sums of one CTA: [kRowTile][kTauTile] of (hi, lo, bound, 0)
constexpr uint64_t kPartialBlock = (uint64_t)kRowTile * kTauTile;

// tensor maps per group: [2g] the K digit planes (box 128 timeslice rows),
// [2g+1] the trial digit planes (box 64 rows)
__global__ void split_contract_kernel(RunDev* runs, SplitRun* split, const SplitTile* tiles, const SplitWork* work,
                                      const SplitRow* rows, const CUtensorMap* maps, float4* partial, int* status);
// combine_tiles: the tiles split over several CTAs (a tile with one CTA
// has its estimates formed by that CTA)
__global__ void split_combine_kernel(RunDev* runs, SplitRun* split, const SplitTile* tiles,
                                     const uint32_t* combine_tiles, const SplitRow* rows, const float4* partial);
__global__ void split_select_kernel(RunDev* runs, SplitRun* split, const Work* work);
// the same without the scaling warps (batches without kDeferNorm runs)
constexpr int kSelectLeanThreads = 160;
__global__ void split_select_lean_kernel(RunDev* runs, SplitRun* split, const Work* work);
// generation 0: the initial parents' fitness intervals, one CTA per member
constexpr int kInitThreads = 128;
__global__ void split_init_kernel(RunDev* runs, SplitRun* split, const Work* work);
// The digit planes of K (kn null for one-sided K), one CTA per timeslice t:
// per 32-gene chunk the scale exponent shared by both sides (kexp[t][c]),
// seven 7-bit digits per value as BF16 in the tiled planes
// [plane][unit of 8 genes][timeslice][8], and the timeslice's largest scale
// exponent (kexp_max[t]).
__global__ void k_digits_kernel(const double* kp, const double* kn, uint32_t Nt, uint32_t M, uint16_t* kdig,
                                int16_t* kexp, int16_t* kexp_max);
constexpr int kCombineCtasPerTile = (int)(kPartialBlock / 32);  // 32 outputs per CTA
// split_combine_wide_kernel: tiles split over at most this many CTAs, 256
// outputs per CTA
constexpr uint32_t kCombineWideSplits = 8;
constexpr int kCombineWideCtasPerTile = (int)(kPartialBlock / 256);
__global__ void split_combine_wide_kernel(RunDev* runs, SplitRun* split, const SplitTile* tiles,
                                          const uint32_t* combine_tiles, const SplitRow* rows,
                                          const float4* partial);

// ---- digit slicing of one value (shared by trial_kernel and the host)
// exponent field of |v| (unbiased), or -2000 for zero / subnormal.  The
// field is read from the high word, without masking the sign off the whole
// value: the compiler turns such a mask into an FP64 absolute value, a slot
// of GB300's narrow FP64 pipe.
__device__ __forceinline__ int exp_of(double v) {
    const int ef = (int)(((uint32_t)__double2hiint(v) >> 20) & 0x7FFu);
    return ef == 0 ? -2000 : ef - 1023;
}

// fixed-point fraction floor(|v| * 2^(49-e)) for a scale 2^e > |v|
__device__ __forceinline__ uint64_t frac_digits(double v, int e) {
    const uint64_t b = (uint64_t)__double_as_longlong(v);
    const int ef = (int)(((uint32_t)__double2hiint(v) >> 20) & 0x7FFu);
    if (ef == 0) return 0;  // zero or subnormal: below every scale used here
    const uint64_t mant = (b & 0xFFFFFFFFFFFFFull) | (1ull << 52);
    const int shift = (52 - kDigitBits) + e - (ef - 1023);
    return shift >= 64 ? 0 : (mant >> shift);
}

__device__ __forceinline__ uint16_t bf16_digit(uint32_t d, bool neg) {
    const uint32_t f = __float_as_uint((float)d);  // exact: d < 128
    return (uint16_t)((f >> 16) | (neg && d ? 0x8000u : 0u));
}

// Position in shared memory of gene j (of a trial part) within its side's
// row: the 16-byte pairs of each 8-gene unit permuted (by bits 4 and 5 of j)
// so that the eight threads of one side of a chunk in digitize_trial, which
// read the same pair of eight consecutive units, hit eight distinct bank
// groups.
__device__ __forceinline__ uint32_t part_slot(uint32_t j) {
    return j ^ ((((j >> 4) & 1u) << 2) | (((j >> 5) & 1u) << 1));
}

// The seven digit planes of one 16-byte unit (8 genes v) at scale 2^e:
// one 16-byte store per plane at q, q + kXdigDigit, ...  Two genes' digits
// d, d' (7 bits each) of a plane are made at once, as one exact packed BF16
// FMA: sign * (128 + d) - sign * 128 = sign * d (128 + d and 128 are BF16
// numbers; d = 0 gives +0 on either sign), the pair packed as the plane's
// 32-bit word (gene 2k in the low half).
__device__ __forceinline__ void store_unit_digits(const double v[8], int e, uint16_t* q) {
    uint64_t f[8];
    uint32_t sg[4], nb[4];  // per pair: the signs as BF16 +-1, and -sign * 128
#pragma unroll
    for (uint32_t k = 0; k < 8; ++k) f[k] = frac_digits(v[k], e);
#pragma unroll
    for (uint32_t k = 0; k < 4; ++k) {
        // the sign bits (integer tests: FP64 compares share the narrow FP64 pipe)
        const uint32_t n0 = (uint32_t)__double2hiint(v[2 * k]) >> 31;
        const uint32_t n1 = (uint32_t)__double2hiint(v[2 * k + 1]) >> 31;
        const uint32_t m = (n0 << 15) | (n1 << 31);  // sign bits of the two halves
        sg[k] = 0x3F803F80u | m;                      // +-1.0
        nb[k] = 0xC300C300u ^ m;                      // -+128.0
    }
#pragma unroll
    for (int b = 0; b < kDigits; ++b) {
        const int sh = 7 * (kDigits - 1 - b);
        uint32_t w[4];
#pragma unroll
        for (uint32_t k = 0; k < 4; ++k) {
            const uint32_t lo = (uint32_t)(f[2 * k] >> sh) & 127u, hi = (uint32_t)(f[2 * k + 1] >> sh) & 127u;
            const uint32_t x = 0x43004300u | lo | (hi << 16);  // BF16 pair (128 + d, 128 + d')
            asm("fma.rn.bf16x2 %0, %1, %2, %3;" : "=r"(w[k]) : "r"(sg[k]), "r"(x), "r"(nb[k]));
        }
        *reinterpret_cast<uint4*>(q + b * kXdigDigit) = make_uint4(w[0], w[1], w[2], w[3]);
    }
}

// The digit planes of the `len` genes (a multiple of 32) of one trial part,
// both sides, read from shared memory `x` (side s at s * side_stride, gene j
// at part_slot(j)) by the calling CTA (blockDim.x a multiple of 32): sixteen
// threads per 64-gene chunk, each one 16-byte unit of 8 genes of one side.
// A chunk's scale exponent is the maximum over both sides; each gene gets
// seven 7-bit digits, written as one 16-byte store per digit plane; the
// part's maximum exponent is raised into *xexp_max.  `xdig` points at the
// trial's row in the tiled planes at the part's first unit; units are
// unit_stride elements apart, sides xside_stride, digits kXdigDigit.
// `s_max` is shared scratch of one int per warp.
__device__ __forceinline__ void digitize_trial(const double* x, uint32_t side_stride, uint32_t S, uint32_t len,
                                               uint16_t* xdig, uint64_t unit_stride, uint64_t xside_stride,
                                               int16_t* xexp, int32_t* xexp_max, int* s_max) {
    const uint32_t warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const uint32_t s = (threadIdx.x >> 3) & 1u, uq = threadIdx.x & 7u;
    const uint32_t C = (len + kChunk - 1) / kChunk, per_pass = blockDim.x >> 4;
    int wmax = -2000;
    for (uint32_t c0 = 0; c0 < C; c0 += per_pass) {
        const uint32_t c = c0 + (threadIdx.x >> 4);
        const uint32_t u = c * 8 + uq;  // this thread's unit within the part
        const bool live = c < C && s < S && u * 8 < len;
        double v[8];
        int e = -2000;
        if (live) {
            const double* row = x + s * side_stride;
#pragma unroll
            for (uint32_t k = 0; k < 4; ++k) {
                const double2 q = *reinterpret_cast<const double2*>(row + part_slot(u * 8 + 2 * k));
                v[2 * k] = q.x;
                v[2 * k + 1] = q.y;
            }
#pragma unroll
            for (uint32_t k = 0; k < 8; ++k) e = max(e, exp_of(v[k]));
        }
#pragma unroll
        for (int o = 1; o < 16; o <<= 1) e = max(e, __shfl_xor_sync(0xffffffffu, e, o));
        e = e <= -1500 ? -1000 : e + 1;  // scale 2^e > every |v| of the chunk
        if (live) {
            store_unit_digits(v, e, xdig + s * xside_stride + (uint64_t)u * unit_stride);
            if ((threadIdx.x & 15u) == 0) xexp[c] = (int16_t)e;
        }
        if (c < C) wmax = max(wmax, e);
    }
    wmax = __reduce_max_sync(0xffffffffu, wmax);
    if ((threadIdx.x & 31u) == 0) s_max[warp] = wmax;
    __syncthreads();
    if (threadIdx.x == 0) {
        int m = -2000;
        for (uint32_t k = 0; k < nw; ++k) m = max(m, s_max[k]);
        atomicMax(xexp_max, m);
    }
}

// ---- trial slices: the split engine's trials for batches on counter
// streams, runs of at most kSliceRows members.  An item of a run is
// slice_chunks(P, S) consecutive 64-gene chunks of every member, both sides.
// trial_slice_kernel is persistent, one CTA per SM: each CTA walks its items
// (seg_start[b] .. seg_start[b+1] of the segment list) through three
// shared-memory stages, each holding every member's parent rows of one item
// (bulk copies, so each parent gene leaves HBM once however many trials use
// it as a donor).  Warp w forms the trials of one group of members for one
// chunk of the item: lane = (member, side, unit of 8 genes), so the chunk's
// scale exponent is a shuffle maximum over the member's lanes, the digits
// are made from registers, and each trial gene is written once.  The last
// warp done with an item stages the item three ahead in its place.
constexpr int kSliceThreads = 1024;
constexpr uint32_t kSliceWarps = kSliceThreads / 32;
constexpr uint32_t kSliceRows = 64;   // largest population of a sliced run
constexpr uint32_t kSliceStages = 3;
// one stage: the parents of an item, [member][side][slice_chunks x 64] --
// at most 64 x 2 x 64 doubles (slice_chunks keeps P S chunks <= 128)
constexpr uint32_t kSliceStageDoubles = kSliceRows * 2 * kChunk;
constexpr uint32_t kSliceSmemBytes = kSliceStages * kSliceStageDoubles * 8;
// members per warp: 32 lanes over 8 units x S sides each
__host__ __device__ inline uint32_t slice_rows_per_warp(uint32_t S) { return 4 / S; }
// member groups of a run: one warp each per chunk
__host__ __device__ inline uint32_t slice_groups(uint32_t P, uint32_t S) {
    return (P + slice_rows_per_warp(S) - 1) / slice_rows_per_warp(S);
}
// chunks per item: the groups times the chunks fill at most the CTA's warps
__host__ __device__ inline uint32_t slice_chunks(uint32_t P, uint32_t S) {
    const uint32_t g = slice_groups(P, S);
    return g >= kSliceWarps ? 1u : kSliceWarps / g;
}
struct SliceSeg {
    uint32_t run, item0, item1;  // items [item0, item1) of one run
};
__global__ void trial_slice_kernel(RunDev* runs, const SliceSeg* segs, const uint32_t* seg_start, int* status);
// status value of a CTA whose bulk-copy wait gave up
constexpr int kStatusSliceWait = 2;


}  // namespace deac
