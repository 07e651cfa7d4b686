// deac_split.cuh -- the split-precision evaluation of the contraction on the
// tcgen05 tensor cores, used by DEAC_ENGINE_SPLIT_BF16.
//
// E[i,t] = sum_k x[i,k] K[t,k] (both sides) is evaluated from exact BF16
// digit slices:  every value v of a 32-gene chunk is written as
//     v = sign * 2^e * sum_{b=0..5} d_b 2^(-7(b+1)) + r,   0 <= d_b <= 127,
// with one power-of-two scale 2^e per (row, chunk) shared by both sides
// (|r| < 2^(e-42)).  Digit products d_a d'_b < 2^14 and a group of equal
// weight (a+b = g, g <= 5) summed over 32 genes x 2 sides is < 2^23, so the
// tensor core's FP32 accumulation of each group is exact.  Per chunk the six
// group sums are combined into a double-float (FP32 pair) value, scaled by
// 2^(e_x + e_K - 49) and added to double-float accumulators; CTAs split the
// chunks of a tile and a combine kernel adds their partial sums.  What is
// dropped -- remainders and digit pairs with a+b > 5 -- is below
// 2^-39.2 * 2^(e_x+e_K) per product, and the bound's chunk sums
// B = sum_c 2^(e_x+e_K) are accumulated by one extra rank-1 MMA per chunk.
// With the rounding bounds of the double-float steps and of the FP64 chain
// itself this gives an interval that contains the value the plain FP64
// engine computes, so selection decisions made from it are the FP64
// decisions (deac_kernels.cuh, contract_kernel).
#pragma once

#include <cstdint>

#include "deac_kernels.cuh"

namespace deac {

constexpr int kDigits = 6;         // 7-bit digits per value (42 bits)
constexpr int kChunk = 32;         // genes per scale chunk and per MMA stage
constexpr int kTauTile = 128;      // MMA M: timeslices, one TMEM lane each
constexpr int kRowTile = 64;       // MMA N: trial rows
constexpr int kSplitThreads = 256; // two warps per TMEM lane quarter
constexpr int kDigitizeThreads = 512;
constexpr int kDecideThreads = 512;
constexpr uint32_t kDecideMaxTau = 2048;  // timeslices whose 1/sigma is kept in shared memory
// dynamic shared memory of split_contract_kernel for S sides: K digits
// [6][S] x (128 x 32), trial digits [6][S] x (64 x 32), the two bound
// operands (128 x 16, 64 x 16) and the double-float accumulators 64 x 128
constexpr uint32_t split_smem_bytes(uint32_t S) {
    return (uint32_t)kDigits * S * (kTauTile * kChunk * 2) + (uint32_t)kDigits * S * (kRowTile * kChunk * 2) +
           (kTauTile + kRowTile) * 16 * 2 + kRowTile * kTauTile * 8;
}

// Split-engine buffers of one run (device pointers).
struct SplitRun {
    uint16_t* xdig;      // [kDigits][S][P][M] BF16 digits of the trial genes
    int16_t* xexp;       // [P][M/kChunk] chunk scale exponents of the trial
    const uint16_t* kdig;  // [kDigits][S][Nt][M] digits of K (shared)
    const int16_t* kexp;   // [Nt][M/kChunk]
    const int16_t* kexp_max;  // [Nt] max over chunks
    int16_t* xexp_max;   // [P] max over chunks
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

__global__ void digitize_kernel(RunDev* runs, SplitRun* split, const Work* work, int all_members);
__global__ void split_contract_kernel(RunDev* runs, SplitRun* split, const SplitTile* tiles, const SplitWork* work,
                                      const SplitRow* rows, float4* partial, int* status);
__global__ void split_combine_kernel(RunDev* runs, SplitRun* split, const SplitTile* tiles, const SplitRow* rows,
                                     const float4* partial);
__global__ void split_decide_kernel(RunDev* runs, SplitRun* split);
constexpr int kCombineCtasPerTile = (int)(kPartialBlock / 256);

// host-side digit decomposition of one value for a given scale exponent
void digits_of(double v, int e, uint16_t out[kDigits]);

}  // namespace deac
