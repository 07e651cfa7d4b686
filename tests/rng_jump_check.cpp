// The PRNG table's states k jumps on, formed from the GF(2) matrices
// J^(2^b) of the jump (deac_rng.cuh: jump_matrix, gf2_matmul, gf2_matvec,
// as rng_table_kernel does), must equal the reference's chain of jumps
// (deac.cpp:1114-1126) word for word; likewise the states the initial
// population's draws start from, formed from the powers of one generator
// step.  Prints "ok" or the first mismatch.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "deac_rng.cuh"

int main(int argc, char** argv) {
    using namespace deac;
    const uint64_t n = argc > 1 ? std::strtoull(argv[1], nullptr, 10) : 70000;
    uint32_t bits = 1;
    while ((1ull << bits) < n) ++bits;
    std::vector<uint64_t> tab((size_t)bits * 1024);
    jump_matrix(tab.data());
    for (uint32_t b = 1; b < bits; ++b)
        gf2_matmul(tab.data() + (b - 1) * 1024, tab.data() + (b - 1) * 1024, tab.data() + b * 1024);
    for (uint64_t seed = 1; seed <= 3; ++seed) {
        Xoshiro g = Xoshiro::seeded(1407513600ULL + seed);
        for (uint64_t i = 0; i < 1000 * seed; ++i) g.next();  // the initial population's draws
        const uint64_t s0[4] = {g.s[0], g.s[1], g.s[2], g.s[3]};
        for (uint64_t k = 0; k < n; ++k) {
            if (k < 512 || k % 61 == 0 || k + 64 > n) {
                uint64_t v[4] = {s0[0], s0[1], s0[2], s0[3]};
                for (uint32_t b = 0; b < bits; ++b)
                    if ((k >> b) & 1u) {
                        uint64_t o[4];
                        gf2_matvec(tab.data() + (size_t)b * 1024, v, o);
                        for (int w = 0; w < 4; ++w) v[w] = o[w];
                    }
                for (int w = 0; w < 4; ++w)
                    if (v[w] != g.s[w]) {
                        std::printf("mismatch: seed %llu state %llu word %d\n", (unsigned long long)seed,
                                    (unsigned long long)k, w);
                        return 1;
                    }
            }
            g.jump();
        }
    }
    // the initial populations' threads: the state after k draws, from the
    // GF(2) powers J^(2^b) of one step (step_matrix, as population_kernel
    // and the set-up's start state use them), equals k sequential draws
    {
        std::vector<uint64_t> st((size_t)24 * 1024);
        step_matrix(st.data());
        for (uint32_t b = 1; b < 24; ++b)
            gf2_matmul(st.data() + (b - 1) * 1024, st.data() + (b - 1) * 1024, st.data() + b * 1024);
        Xoshiro g = Xoshiro::seeded(1407513600ULL + 7);
        const uint64_t s0[4] = {g.s[0], g.s[1], g.s[2], g.s[3]};
        for (uint64_t k = 0; k <= (1ull << 21) + 5; ++k) {
            if (k < 2100 || k % 1024 == 0 || k % 99991 == 0 || k + 8 > (1ull << 21)) {
                uint64_t v[4] = {s0[0], s0[1], s0[2], s0[3]};
                for (uint32_t b = 0; b < 24; ++b)
                    if ((k >> b) & 1u) {
                        uint64_t o[4];
                        gf2_matvec(st.data() + (size_t)b * 1024, v, o);
                        for (int w = 0; w < 4; ++w) v[w] = o[w];
                    }
                for (int w = 0; w < 4; ++w)
                    if (v[w] != g.s[w]) {
                        std::printf("step mismatch: draw %llu word %d\n", (unsigned long long)k, w);
                        return 1;
                    }
            }
            g.next();
        }
    }
    std::printf("ok\n");
    return 0;
}
