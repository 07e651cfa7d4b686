// deac_rng.cuh -- the reference PRNG, usable on host and device.
//
// xoshiro256+ seeded through splitmix64 exactly as the reference does it
// (src/deac/include/rng.hpp:10-59): each 64-bit splitmix output fills two
// state words with its low and high 32-bit halves.  The 2^128 jump
// (rng.hpp:64-87) separates the per-gene states of the GPU path
// (deac.cpp:1114-1135).  Uniform doubles are (x >> 11) * 2^-53
// (rng.hpp:129-131).
#pragma once

#include <cstdint>

#if defined(__CUDACC__)
#define DEAC_HD __host__ __device__ __forceinline__
#else
#define DEAC_HD inline
#endif

namespace deac {

DEAC_HD uint64_t rotl64(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

// One xoshiro256+ step on four words held by the caller.
DEAC_HD uint64_t xoshiro_next(uint64_t& s0, uint64_t& s1, uint64_t& s2, uint64_t& s3) {
    const uint64_t result = s0 + s3;
    const uint64_t t = s1 << 17;
    s2 ^= s0;
    s3 ^= s1;
    s1 ^= s2;
    s0 ^= s3;
    s2 ^= t;
    s3 = rotl64(s3, 45);
    return result;
}

DEAC_HD double to_unit(uint64_t x) { return static_cast<double>(x >> 11) * 0x1.0p-53; }

struct Xoshiro {
    uint64_t s[4];

    DEAC_HD uint64_t next() { return xoshiro_next(s[0], s[1], s[2], s[3]); }

    static uint64_t splitmix(uint64_t& x) {
        uint64_t r = (x += 0x9E3779B97f4A7C15ULL);
        r = (r ^ (r >> 30)) * 0xBF58476D1CE4E5B9ULL;
        r = (r ^ (r >> 27)) * 0x94D049BB133111EBULL;
        return r ^ (r >> 31);
    }

    static Xoshiro seeded(uint64_t seed) {
        Xoshiro g;
        uint64_t x = seed;
        const uint64_t a = splitmix(x);
        g.s[0] = static_cast<uint32_t>(a);
        g.s[1] = a >> 32;
        const uint64_t b = splitmix(x);
        g.s[2] = static_cast<uint32_t>(b);
        g.s[3] = b >> 32;
        return g;
    }

    // Advance by 2^128 steps (the published xoshiro256 jump polynomial).
    void jump() {
        static const uint64_t kJump[4] = {0x180ec6d33cfd0abaULL, 0xd5a61266f0c9392cULL,
                                          0xa9582618e03fc9aaULL, 0x39abdc4529b1661cULL};
        uint64_t a = 0, b = 0, c = 0, d = 0;
        for (int w = 0; w < 4; ++w)
            for (int bit = 0; bit < 64; ++bit) {
                if (kJump[w] & (1ULL << bit)) {
                    a ^= s[0];
                    b ^= s[1];
                    c ^= s[2];
                    d ^= s[3];
                }
                next();
            }
        s[0] = a;
        s[1] = b;
        s[2] = c;
        s[3] = d;
    }
};

// ---- counter streams (the batched forms' compact draw layout)
//
// SplitMix64 (Steele, Lea and Flood, "Fast splittable pseudorandom number
// generators", OOPSLA 2014) is a Weyl sequence key + n * gamma passed through
// a bijective 64-bit mixer; its n-th output depends on n alone.  A run's
// per-generation draws are outputs of two such streams at positions computed
// from (generation, member, side, gene), so no per-gene state is stored or
// streamed: the draws are reproducible for any launch shape, and the plain
// and split engines draw the same values.  The mixer is the one of the
// splitmix step above.
DEAC_HD uint64_t splitmix_mix(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

// Output `pos` (0, 1, ...) of the SplitMix64 stream whose state starts at key.
DEAC_HD uint64_t stream_draw(uint64_t key, uint64_t pos) {
    return splitmix_mix(key + (pos + 1) * 0x9E3779B97F4A7C15ULL);
}

// The two keys of a run (crossover draws, jDE draws): the third and fourth
// outputs of the splitmix sequence seeded with the run's seed, whose first
// two seed the initial population's generator (Xoshiro::seeded).
inline void stream_keys(uint64_t seed, uint64_t& key_crossover, uint64_t& key_jde) {
    uint64_t x = seed;
    Xoshiro::splitmix(x);
    Xoshiro::splitmix(x);
    key_crossover = Xoshiro::splitmix(x);
    key_jde = Xoshiro::splitmix(x);
}

// Positions within the streams.  jDE step n of member i (the draws for the
// trial of its n-th generation) reads the jDE stream at kJdeSpan * (n P + i)
// + k: k = 4s (CR test of side s), 4s+1 (new CR), 4s+2 (F test), 4s+3 (new
// F), and k = 8, 9, ... the mutant-index draws of the rejection sampling.
// Crossover draw of gene j, side s in that trial: ((n P + i) S + s) M + j of
// the crossover stream.
constexpr uint64_t kJdeSpan = 1ull << 16;
constexpr uint64_t kJdeMutantDraw0 = 8;

// The jump as a linear map of the 256-bit state over GF(2): a 256 x 256
// matrix stored as 256 columns of 4 words (column i = jump(e_i)).  J^k s,
// the state k jumps on, is then a product of the matrices J^(2^b) of k's
// set bits -- independent per k, where the jumps themselves form a chain.
DEAC_HD void gf2_matvec(const uint64_t* cols, const uint64_t v[4], uint64_t out[4]) {
    uint64_t a = 0, b = 0, c = 0, d = 0;
    for (uint32_t i = 0; i < 256; ++i) {
        const uint64_t m = 0ull - ((v[i >> 6] >> (i & 63u)) & 1ull);
        a ^= cols[4 * i] & m;
        b ^= cols[4 * i + 1] & m;
        c ^= cols[4 * i + 2] & m;
        d ^= cols[4 * i + 3] & m;
    }
    out[0] = a;
    out[1] = b;
    out[2] = c;
    out[3] = d;
}

inline void jump_matrix(uint64_t cols[1024]) {
    for (uint32_t i = 0; i < 256; ++i) {
        Xoshiro x{{0, 0, 0, 0}};
        x.s[i >> 6] = 1ull << (i & 63u);
        x.jump();
        for (int w = 0; w < 4; ++w) cols[4 * i + w] = x.s[w];
    }
}

// One generator step (xoshiro256+'s state update) as the same kind of
// matrix: column i = step(e_i).
inline void step_matrix(uint64_t cols[1024]) {
    for (uint32_t i = 0; i < 256; ++i) {
        Xoshiro x{{0, 0, 0, 0}};
        x.s[i >> 6] = 1ull << (i & 63u);
        x.next();
        for (int w = 0; w < 4; ++w) cols[4 * i + w] = x.s[w];
    }
}

// C = A B (column j of C is A times column j of B)
inline void gf2_matmul(const uint64_t* A, const uint64_t* B, uint64_t* C) {
    for (uint32_t j = 0; j < 256; ++j) gf2_matvec(A, B + 4 * j, C + 4 * j);
}

}  // namespace deac
