// deac_jde.cuh -- the jDE step of one member (self-adaptation of CR and F per
// side, then three distinct mutant indices by rejection sampling), shared by
// the trial kernels and by the split engine's decisions, which draw the next
// generation's jDE as soon as a run's selections are final.
//
// RNG slots of member i (base = i * (1 + S*M), word-major table of n states):
// base (CR of side 0, then the mutant indices), base+1 (F of side 0),
// base+2 / base+3 (CR / F of side 1) -- deac_gpu.cu's per-member states.
// With counter streams (kCounterStreams) the table holds one slot per member
// whose first word counts the member's jDE steps; step n draws from the jDE
// stream at the positions deac_rng.cuh lists, and the slot's other words are
// unused.
#pragma once

#include <cstdint>

#include "deac_kernels.cuh"
#include "deac_rng.cuh"

namespace deac {

// x % P for the 64-bit draws of the mutant indices: q = floor(x * m / 2^64)
// with m = floor((2^64 - 1) / P) is at most two below floor(x / P), so two
// corrections give the exact remainder (no 64-bit division routine).
__device__ __forceinline__ uint64_t mod_p(uint64_t x, uint64_t P, uint64_t m) {
    uint64_t r = x - __umul64hi(x, m) * P;
    if (r >= P) r -= P;
    if (r >= P) r -= P;
    return r;
}

// the jDE slots of member i (every load at once); with counter streams the
// member's step count in st[0][0]
__device__ __forceinline__ void jde_load(const RunDev& R, uint32_t i, uint64_t (&st)[4][4]) {
    if (R.flags & kCounterStreams) {
#pragma unroll
        for (uint32_t q = 0; q < 4; ++q)
#pragma unroll
            for (uint32_t w = 0; w < 4; ++w) st[q][w] = 0ull;
        st[0][0] = R.rng[i];
        return;
    }
    const uint64_t base = (uint64_t)i * (1ull + (uint64_t)R.S * R.M);
    const uint64_t n = R.n_states;
    const uint64_t* rng = R.rng;
#pragma unroll
    for (uint32_t q = 0; q < 4; ++q)
#pragma unroll
        for (uint32_t w = 0; w < 4; ++w) st[q][w] = (q < 2 * R.S) ? rng[w * n + base + q] : 0ull;
}

// Every draw of member i's jDE step from its slots st (advanced in place):
// per side whether CR / F take a new value and that value, then the mutant
// indices.  None of it depends on the current CR / F, so the draws can be
// made before the selection that decides which CR / F the member keeps.
struct JdeDraws {
    double cr[2], fw[2];
    bool cr_new[2], fw_new[2];
    uint32_t mut[3];
};

__device__ __forceinline__ void jde_draws(const RunDev& R, uint32_t i, uint64_t (&st)[4][4], JdeDraws& d) {
    const uint32_t P = R.P;
    // draw < tau  <=>  (x >> 11) < ceil(tau 2^53) (draw = (x >> 11) 2^-53
    // exactly): integer tests, a conversion only for a new value
    const uint64_t thr_cr = R.tau_cr_thr, thr_f = R.tau_f_thr;
    auto bits = [](uint64_t (&st)[4]) { return xoshiro_next(st[0], st[1], st[2], st[3]) >> 11; };
    auto side = [&](uint32_t s, uint64_t (&cs)[4], uint64_t (&fs)[4]) {
        d.cr_new[s] = bits(cs) < thr_cr;
        d.cr[s] = d.cr_new[s] ? (double)bits(cs) * 0x1.0p-53 : 0.0;
        d.fw_new[s] = bits(fs) < thr_f;
        d.fw[s] = d.fw_new[s] ? (double)bits(fs) * 0x1.0p-52 : 0.0;  // 2 * draw
    };
    d.cr_new[1] = d.fw_new[1] = false;
    d.cr[1] = d.fw[1] = 0.0;
    if (R.flags & kCounterStreams) {
        // jDE step n of member i: fixed positions of the run's jDE stream
        const uint64_t n = st[0][0];
        const uint64_t pos0 = kJdeSpan * (n * P + i);
        auto at = [&](uint64_t k) { return stream_draw(R.key_jde, pos0 + k) >> 11; };
#pragma unroll
        for (uint32_t s = 0; s < 2; ++s)
            if (s < R.S) {
                d.cr_new[s] = at(4 * s) < thr_cr;
                d.cr[s] = d.cr_new[s] ? (double)at(4 * s + 1) * 0x1.0p-53 : 0.0;
                d.fw_new[s] = at(4 * s + 2) < thr_f;
                d.fw[s] = d.fw_new[s] ? (double)at(4 * s + 3) * 0x1.0p-52 : 0.0;  // 2 * draw
            }
        // rejection sampling from draw 8 on (an admissible index has
        // probability >= 1/4 per draw for P >= 4: the span of 2^16 - 8 draws
        // is never exhausted in practice; if it were, the first admissible
        // index is taken so that the result stays defined)
        const uint64_t pm = R.p_magic;
        uint64_t k = kJdeMutantDraw0, r[3] = {i, i, i};
#pragma unroll
        for (uint32_t q = 0; q < 3; ++q) {
            auto bad = [&](uint64_t v) { return v == i || (q > 0 && v == r[0]) || (q > 1 && v == r[1]); };
            while (bad(r[q]) && k < kJdeSpan) r[q] = mod_p(stream_draw(R.key_jde, pos0 + k++), P, pm);
            for (uint64_t v = 0; bad(r[q]); ++v) r[q] = v;
        }
        d.mut[0] = (uint32_t)r[0];
        d.mut[1] = (uint32_t)r[1];
        d.mut[2] = (uint32_t)r[2];
        st[0][0] = n + 1;
        return;
    }
    side(0, st[0], st[1]);
    if (R.S == 2) side(1, st[2], st[3]);
    // rejection sampling as in the reference; P >= 4 is enforced on the
    // host, so every loop has an admissible outcome
    uint64_t r0 = i, r1 = i, r2 = i;
    const uint64_t pm = R.p_magic;
    while (r0 == i) r0 = mod_p(xoshiro_next(st[0][0], st[0][1], st[0][2], st[0][3]), P, pm);
    while (r1 == i || r1 == r0) r1 = mod_p(xoshiro_next(st[0][0], st[0][1], st[0][2], st[0][3]), P, pm);
    while (r2 == i || r2 == r0 || r2 == r1) r2 = mod_p(xoshiro_next(st[0][0], st[0][1], st[0][2], st[0][3]), P, pm);
    d.mut[0] = (uint32_t)r0;
    d.mut[1] = (uint32_t)r1;
    d.mut[2] = (uint32_t)r2;
}

// the new CR / F from the draws and the CR / F the member keeps
__device__ __forceinline__ void jde_apply(const JdeDraws& d, const double cr_old[2], const double fw_old[2],
                                          double cr_new[2], double fw_new[2]) {
#pragma unroll
    for (uint32_t s = 0; s < 2; ++s) {
        cr_new[s] = d.cr_new[s] ? d.cr[s] : cr_old[s];
        fw_new[s] = d.fw_new[s] ? d.fw[s] : fw_old[s];
    }
}

// the draws of member i from its slots st (advanced in place) and its
// current CR / F
__device__ __forceinline__ void jde_draw(const RunDev& R, uint32_t i, uint64_t (&st)[4][4], const double cr_old[2],
                                         const double fw_old[2], double cr_new[2], double fw_new[2], uint32_t mut[3]) {
    JdeDraws d;
    jde_draws(R, i, st, d);
    jde_apply(d, cr_old, fw_old, cr_new, fw_new);
    mut[0] = d.mut[0];
    mut[1] = d.mut[1];
    mut[2] = d.mut[2];
}

// store the outcome: the new CR / F (upper halves of cr / fw), the advanced
// slots and, when `mutants` is set, the indices
__device__ __forceinline__ void jde_store(RunDev& R, uint32_t i, const uint64_t (&st)[4][4], const double cr_new[2],
                                          const double fw_new[2], const uint32_t mut[3], bool mutants) {
    const uint32_t P = R.P, S = R.S;
    const uint64_t base = (uint64_t)i * (1ull + (uint64_t)S * R.M);
    const uint64_t n = R.n_states;
#pragma unroll
    for (uint32_t s = 0; s < 2; ++s)
        if (s < S) {
            R.cr[(uint64_t)S * P + s * P + i] = cr_new[s];
            R.fw[(uint64_t)S * P + s * P + i] = fw_new[s];
        }
    if (R.flags & kCounterStreams) {
        R.rng[i] = st[0][0];
    } else {
#pragma unroll
        for (uint32_t q = 0; q < 4; ++q)
            if (q < 2 * S)
#pragma unroll
                for (uint32_t w = 0; w < 4; ++w) R.rng[w * n + base + q] = st[q][w];
    }
    if (mutants)
        for (uint32_t q = 0; q < 3; ++q) R.mutants[3 * i + q] = mut[q];
}

}  // namespace deac
