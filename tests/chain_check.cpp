// CPU check of the blocked exact FMA-chain arithmetic (deac_chain.cuh):
// host_fma_chain and host_group_fma_chain (the sequential walk of the
// device's group form, term shifts included) must equal the plain
// sequential fma chain bit for bit on
// random and adversarial inputs (ties, sign changes, cancellation,
// subnormal, huge and zero terms).  Prints "ok <cases> <plain-steps>" or the
// first mismatch and exits 1.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <random>
#include <vector>

#include "deac_chain.cuh"

static uint64_t bits(double d) {
    uint64_t b;
    std::memcpy(&b, &d, 8);
    return b;
}

// term() against its definition evaluated with 128-bit integers: |v| =
// mx*mw / 2^(ea - ex - ew), F = floor(|v|), the fraction above / at / below
// one half, a term of 2^54 or more (or non-finite) flagged kBad.
static bool term_matches(double x, double w, int ea, uint32_t neg_acc) {
    using namespace deac::chain_detail;
    const Term t = term(x, w, ea, neg_acc);
    const uint64_t bx = bits(x), bw = bits(w);
    const int Ex = (int)((bx >> 52) & 0x7FF), Ew = (int)((bw >> 52) & 0x7FF);
    if (Ex == 0x7FF || Ew == 0x7FF) return (t.flags & kBad) != 0;
    const uint64_t mx = (bx & ((1ull << 52) - 1)) | (Ex ? (1ull << 52) : 0), mw = (bw & ((1ull << 52) - 1)) | (Ew ? (1ull << 52) : 0);
    if (mx == 0 || mw == 0) return t.F == 0 && t.flags == 0;
    const int ex = Ex ? Ex - 1075 : -1074, ew = Ew ? Ew - 1075 : -1074;
    const unsigned __int128 P = (unsigned __int128)mx * mw;
    const int r = ea - ex - ew;
    unsigned __int128 F;
    bool half = false, sticky = false;
    if (r <= 0) {
        if (-r >= 54 || (P >> (54 + r)) != 0) return (t.flags & kBad) != 0;
        F = P << -r;
    } else if (r >= 128) {
        F = 0;
        sticky = true;
    } else {
        F = P >> r;
        half = ((P >> (r - 1)) & 1) != 0;
        sticky = r > 1 && (P & ((((unsigned __int128)1) << (r - 1)) - 1)) != 0;
    }
    if ((F >> 54) != 0) return (t.flags & kBad) != 0;
    const uint32_t neg = (uint32_t)((bx ^ bw) >> 63) ^ neg_acc;
    const uint32_t flags = (half && sticky ? kGtHalf : 0u) | (half && !sticky ? kTie : 0u) |
                           (half || sticky ? kGtZero : 0u) | (neg ? kNeg : 0u);
    return t.F == (uint64_t)F && t.flags == flags;
}

int main(int argc, char** argv) {
    const int cases = argc > 1 ? std::atoi(argv[1]) : 4000;
    {
        // decoded terms: random significands, every exponent gap around the
        // decoding paths, subnormal and power-of-two operands
        std::mt19937_64 trng(777);
        for (int k = 0; k < 400000; ++k) {
            const uint64_t u = trng(), v = trng();
            double x, w;
            const int mode = k % 4;
            uint64_t bx = (u & ((1ull << 52) - 1)) | ((uint64_t)(1 + trng() % 2046) << 52) | (u & (1ull << 63));
            uint64_t bw = (v & ((1ull << 52) - 1)) | ((uint64_t)(1 + trng() % 2046) << 52);
            if (mode == 1) bx &= ~((1ull << (trng() % 53)) - 1);  // few significant bits: exact halves
            if (mode == 2) bw = (bw & ~((1ull << 52) - 1));         // power-of-two weight
            if (mode == 3) bx &= (1ull << 52) - 1;                  // subnormal gene
            std::memcpy(&x, &bx, 8);
            std::memcpy(&w, &bw, 8);
            const int Ex = (int)((bx >> 52) & 0x7FF), Ew = (int)((bw >> 52) & 0x7FF);
            const int base = (Ex ? Ex - 1075 : -1074) + (Ew ? Ew - 1075 : -1074);
            const int ea = base + (int)(trng() % 200) - 20;  // gaps r from -20 to 179
            if (!term_matches(x, w, ea, (uint32_t)(trng() & 1))) {
                std::printf("term mismatch x=%a w=%a ea=%d\n", x, w, ea);
                return 1;
            }
        }
    }
    std::mt19937_64 rng(12345);
    std::uniform_real_distribution<double> U(0.0, 1.0);
    uint64_t plain_total = 0, steps_total = 0;
    for (int c = 0; c < cases; ++c) {
        const int kind = c % 9;
        const uint64_t n = 1 + rng() % (kind == 0 ? 8192 : 1200);
        std::vector<double> x(n), w(n);
        for (uint64_t k = 0; k < n; ++k) {
            double a = U(rng), b = U(rng);
            switch (kind) {
                case 0:  // normalisation-like: positive genes, smooth weights
                    b = 0.125 * (k == 0 || k + 1 == n ? 0.5 : 1.0);
                    break;
                case 1:  // few significant bits: many exact ties
                    a = std::ldexp((double)(rng() % 64), (int)(rng() % 8) - 4);
                    b = std::ldexp((double)(rng() % 16 + 1), (int)(rng() % 6) - 3);
                    if (rng() % 4 == 0) a = -a;
                    break;
                case 2:  // signed terms around zero: cancellation, sign flips
                    a = U(rng) - 0.5;
                    b = std::ldexp(1.0, (int)(rng() % 40) - 20);
                    break;
                case 3:  // wide dynamic range (like e^{-tau omega} kernels)
                    b = std::exp(-0.37 * (double)k);
                    a = U(rng) * 3.0;
                    break;
                case 4:  // huge, tiny, subnormal and zero terms mixed in
                    if (rng() % 7 == 0) a = 0.0;
                    if (rng() % 11 == 0) b = std::ldexp(1.0, -1060);
                    if (rng() % 13 == 0) a = std::ldexp(a, 300);
                    if (rng() % 17 == 0) b = std::ldexp(b, -300);
                    if (rng() % 5 == 0) a = -a;
                    break;
                case 5:  // values that make the sum land on binade edges
                    a = std::ldexp(1.0, (int)(rng() % 12) - 6) * (rng() % 3 ? 1.0 : -1.0);
                    b = 1.0 + std::ldexp((double)(rng() % 4), -52);
                    break;
                case 6:  // integers near 2^53: ulp 1 and 2 around the start
                    a = (double)(rng() % 5);
                    b = rng() % 2 ? 0.5 : 1.5;
                    break;
                case 8:  // positive, few significant bits: ties inside predicted binades
                    a = std::ldexp((double)(rng() % 64 + 1), (int)(rng() % 8) - 4);
                    b = std::ldexp((double)(rng() % 16 + 1), (int)(rng() % 6) - 3);
                    break;
                default:  // generic random doubles of random sign and scale
                    a = (U(rng) - 0.5) * std::ldexp(1.0, (int)(rng() % 60) - 30);
                    b = (U(rng) - 0.25) * std::ldexp(1.0, (int)(rng() % 60) - 30);
            }
            x[k] = a;
            w[k] = b;
        }
        double start = 0.0;
        if (kind == 6) start = std::ldexp(1.0, 53) - (double)(rng() % 64);
        if (kind == 5 && rng() % 2) start = -std::ldexp(1.0, (int)(rng() % 10));
        double ref = start;
        for (uint64_t k = 0; k < n; ++k) ref = std::fma(x[k], w[k], ref);
        for (uint64_t sb : {2048ull, 61ull, 4096ull}) {
            const double got = deac::host_group_fma_chain(x.data(), w.data(), n, start, sb);
            if (bits(got) != bits(ref) && !(std::isnan(got) && std::isnan(ref))) {
                std::printf("group mismatch case %d kind %d n %llu sb %llu: %.17g vs %.17g\n", c, kind,
                            (unsigned long long)n, (unsigned long long)sb, got, ref);
                return 1;
            }
        }
        for (uint64_t block : {256ull, 37ull}) {
            uint64_t plain = 0;
            const double got = deac::host_fma_chain(x.data(), w.data(), n, start, block, &plain);
            if (bits(got) != bits(ref) && !(std::isnan(got) && std::isnan(ref))) {
                std::printf("mismatch case %d kind %d n %llu block %llu: %.17g vs %.17g\n", c, kind,
                            (unsigned long long)n, (unsigned long long)block, got, ref);
                return 1;
            }
            plain_total += plain;
            steps_total += n;
        }
    }
    std::printf("ok %d %llu %llu\n", cases, (unsigned long long)plain_total, (unsigned long long)steps_total);
    return 0;
}
