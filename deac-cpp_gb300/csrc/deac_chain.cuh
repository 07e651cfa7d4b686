// deac_chain.cuh -- exact parallel evaluation of a k-ascending FMA chain
//
//     acc <- fma(x[k], w[k], acc),   k = 0 .. n-1,
//
// bit-identical to running the chain one step at a time (the row sums of the
// normalisation and moment terms, gpu_deac_gemv in deac_gpu.cu:345-374).
//
// Why it can be parallel: while |acc| stays in one binade [2^e, 2^(e+1)),
// every representable value there is a multiple of u = 2^(e-52), so the
// rounded step fma(x, w, acc) = RN(acc + x*w) equals acc + q*u with q the
// integer nearest to x*w/u (ties to the even result).  A run of such steps is
// an integer prefix sum of the q's -- with one sequential dependency left,
// the tie rule, which needs the parity of the running integer; parities
// compose as affine maps over GF(2) and are scanned first.  A step is valid
// when the exact sum acc + x*w lies in the binade; the first invalid step of
// a block ends the block, runs as a plain fma, and the next block starts in
// the new binade.  Zero, subnormal and non-finite states also step plainly.
//
// Everything is integer arithmetic on the IEEE fields, so the host and the
// device share the per-step code below; the device form scans a group of
// warps at a time (group_fma_chain), the host form walks blocks sequentially
// and is the CPU check of the arithmetic.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#ifndef __CUDACC__
#define __host__
#define __device__
#define __forceinline__ inline
#endif

namespace deac {
namespace chain_detail {

constexpr uint64_t kTwo52 = 1ull << 52;
constexpr uint64_t kTwo53 = 1ull << 53;

// One step's product relative to the grid of acc:  v = sigma * x*w / u,
// |v| = F + frac with the fraction classified.
struct Term {
    uint64_t F;        // floor(|v|), < 2^54 when usable
    uint32_t flags;    // kGtHalf | kTie | kGtZero | kNeg | kBad
};
constexpr uint32_t kGtHalf = 1u, kTie = 2u, kGtZero = 4u, kNeg = 8u, kBad = 16u;

// A term packed in one word (F < 2^54 in the low bits, the flags above) to
// keep the per-thread caches of the group form in registers.
__host__ __device__ __forceinline__ uint64_t pack(const Term& t) { return t.F | ((uint64_t)t.flags << 56); }
__host__ __device__ __forceinline__ Term unpack(uint64_t v) {
    return Term{v & ((1ull << 54) - 1), (uint32_t)(v >> 56)};
}

__host__ __device__ __forceinline__ uint64_t bits_of(double d) {
#ifdef __CUDA_ARCH__
    return (uint64_t)__double_as_longlong(d);
#else
    uint64_t b;
    std::memcpy(&b, &d, 8);
    return b;
#endif
}
__host__ __device__ __forceinline__ double double_of(uint64_t b) {
#ifdef __CUDA_ARCH__
    return __longlong_as_double((long long)b);
#else
    double d;
    std::memcpy(&d, &b, 8);
    return d;
#endif
}

__host__ __device__ __forceinline__ void mul_wide(uint64_t a, uint64_t b, uint64_t& hi, uint64_t& lo) {
#ifdef __CUDA_ARCH__
    lo = a * b;
    hi = __umul64hi(a, b);
#else
    const unsigned __int128 p = (unsigned __int128)a * b;
    lo = (uint64_t)p;
    hi = (uint64_t)(p >> 64);
#endif
}

// A state the block scan can start from: finite, nonzero, and away from the
// subnormal and overflow ends (biased exponent 2 .. 2045).
__host__ __device__ __forceinline__ bool state_ok(double acc) {
    const uint32_t E = (uint32_t)(bits_of(acc) >> 52) & 0x7FFu;
    return E >= 2u && E <= 2045u;
}

// acc = sigma * A * 2^ea with A in [2^52, 2^53)
__host__ __device__ __forceinline__ void state_split(double acc, uint32_t& neg, uint64_t& A, int& ea) {
    const uint64_t b = bits_of(acc);
    neg = (uint32_t)(b >> 63);
    A = (b & (kTwo52 - 1)) | kTwo52;
    ea = (int)((b >> 52) & 0x7FF) - 1075;
}
// inverse of state_split for A in [2^52, 2^53]
__host__ __device__ __forceinline__ double state_join(uint32_t neg, uint64_t A, int ea) {
    const uint64_t sign = (uint64_t)neg << 63;
    if (A == kTwo53) return double_of(sign | ((uint64_t)(ea + 1075 + 1) << 52));
    return double_of(sign | ((uint64_t)(ea + 1075) << 52) | (A - kTwo52));
}

// x*w relative to the grid 2^ea of a state with sign `neg_acc`
__host__ __device__ __forceinline__ Term term(double x, double w, int ea, uint32_t neg_acc) {
    Term t{0ull, 0u};
    const uint64_t bx = bits_of(x), bw = bits_of(w);
    const uint32_t Ex = (uint32_t)(bx >> 52) & 0x7FFu, Ew = (uint32_t)(bw >> 52) & 0x7FFu;
    if (Ex == 0x7FFu || Ew == 0x7FFu) {
        t.flags = kBad;
        return t;
    }
    const uint64_t mx = (bx & (kTwo52 - 1)) | (Ex ? kTwo52 : 0ull);
    const uint64_t mw = (bw & (kTwo52 - 1)) | (Ew ? kTwo52 : 0ull);
    if (mx == 0 || mw == 0) return t;  // the product is zero: acc unchanged
    const int ex = Ex ? (int)Ex - 1075 : -1074;
    const int ew = Ew ? (int)Ew - 1075 : -1074;
    const uint32_t neg = (uint32_t)((bx ^ bw) >> 63) ^ neg_acc;
    uint64_t hi, lo;
    mul_wide(mx, mw, hi, lo);  // < 2^106
    const int sh = ex + ew - ea;
    uint32_t half = 0, sticky = 0;
    if (sh >= 0) {
        if (sh >= 54 || hi != 0 || (lo >> (54 - sh)) != 0) {
            t.flags = kBad;  // |v| >= 2^54: leaves the binade for sure
            return t;
        }
        t.F = lo << sh;
    } else {
        const int r = -sh;
        if (r >= 128) {
            t.F = 0;
            sticky = 1;  // 0 < |v| < 2^-21
        } else {
            uint64_t fh, fl;
            if (r < 64) {
                fl = (lo >> r) | (hi << (64 - r));
                fh = hi >> r;
            } else {
                fl = hi >> (r - 64);
                fh = 0;
            }
            if (fh != 0 || (fl >> 54) != 0) {
                t.flags = kBad;
                return t;
            }
            t.F = fl;
            const int hb = r - 1;  // the half bit
            half = hb < 64 ? (uint32_t)(lo >> hb) & 1u : (uint32_t)(hi >> (hb - 64)) & 1u;
            if (hb == 0) sticky = 0;
            else if (hb < 64) sticky = (lo & ((1ull << hb) - 1)) != 0;
            else if (hb == 64) sticky = lo != 0;
            else sticky = (lo != 0) || (hi & ((1ull << (hb - 64)) - 1)) != 0;
        }
    }
    t.flags = (half && sticky ? kGtHalf : 0u) | (half && !sticky ? kTie : 0u) | (half || sticky ? kGtZero : 0u) |
              (neg ? kNeg : 0u);
    return t;
}

// parity change of the step when it is not a tie (a tie makes the result even)
__host__ __device__ __forceinline__ uint32_t parity_flip(const Term& t) {
    return (uint32_t)(t.F & 1u) ^ ((t.flags & kGtHalf) ? 1u : 0u);
}

// The step from state A (parity par): q with A' = A + q, or false when the
// step is not one of the binade (it then runs as a plain fma).
__host__ __device__ __forceinline__ bool step(const Term& t, uint64_t A, uint32_t par, int64_t& q) {
    if ((t.flags & kBad) || A < kTwo52 || A >= kTwo53) return false;
    const uint64_t mag = t.F + ((t.flags & kGtHalf) ? 1u : 0u) + ((t.flags & kTie) ? (par ^ (uint32_t)(t.F & 1u)) : 0u);
    if (!(t.flags & kNeg)) {
        if (A + t.F > kTwo53 - 1) return false;  // exact sum reaches the next binade
        q = (int64_t)mag;
    } else {
        const uint64_t down = t.F + ((t.flags & kGtZero) ? 1u : 0u);
        if (down > A - kTwo52) return false;  // exact sum falls below 2^e
        q = -(int64_t)mag;
    }
    return true;
}

// the grid of a state moved up by d binades: v' = v / 2^d
__host__ __device__ __forceinline__ void shift_term(Term& t, int d) {
    if (d == 0 || (t.flags & kBad)) return;
    const uint32_t neg = t.flags & kNeg;
    const uint32_t below_old = (t.flags & kGtZero) != 0;  // anything under the old integer part
    uint64_t F = t.F;
    uint32_t half, sticky;
    if (d >= 64) {
        half = 0;
        sticky = (F != 0) || below_old;
        F = 0;
    } else {
        half = (uint32_t)(F >> (d - 1)) & 1u;
        sticky = (d > 1 && (F & ((1ull << (d - 1)) - 1)) != 0) || below_old;
        F >>= d;
    }
    t.F = F;
    t.flags = (half && sticky ? kGtHalf : 0u) | (half && !sticky ? kTie : 0u) | (half || sticky ? kGtZero : 0u) | neg;
}

}  // namespace chain_detail

// Host form: the same blocks of `block` steps as the device form, walked one
// step at a time.  Returns the chain value; `plain_steps` counts the steps
// that ran as plain fma.
inline double host_fma_chain(const double* x, const double* w, uint64_t n, double acc, uint64_t block = 256,
                             uint64_t* plain_steps = nullptr) {
    using namespace chain_detail;
    uint64_t k = 0, plain = 0;
    while (k < n) {
        if (!state_ok(acc)) {
            acc = std::fma(x[k], w[k], acc);
            ++k;
            ++plain;
            continue;
        }
        uint32_t neg;
        uint64_t A;
        int ea;
        state_split(acc, neg, A, ea);
        const uint64_t L = n - k < block ? n - k : block;
        uint64_t i = 0;
        for (; i < L; ++i) {
            const Term t = term(x[k + i], w[k + i], ea, neg);
            int64_t q;
            if (!step(t, A, (uint32_t)(A & 1u), q)) break;
            A = (uint64_t)((int64_t)A + q);
        }
        acc = state_join(neg, A, ea);
        if (i < L) {
            acc = std::fma(x[k + i], w[k + i], acc);
            ++plain;
            ++i;
        }
        k += i;
    }
    if (plain_steps) *plain_steps = plain;
    return acc;
}

// Host form of group_fma_chain: the same super-blocks, plain first steps,
// rounds and term shifts, with the scans walked sequentially.
inline double host_group_fma_chain(const double* x, const double* w, uint64_t n, double acc, uint64_t SB,
                                   uint64_t* rounds_out = nullptr) {
    using namespace chain_detail;
    uint64_t rounds = 0;
    std::vector<uint64_t> tp(SB);
    for (uint64_t base = 0; base < n; base += SB) {
        const uint64_t len = n - base < SB ? n - base : SB;
        uint64_t k0 = 0;
        const uint64_t early = base == 0 ? (len < 32 ? len : 32) : 0;
        while (k0 < early || (k0 < len && !state_ok(acc))) {
            acc = std::fma(x[base + k0], w[base + k0], acc);
            ++k0;
        }
        if (k0 >= len) continue;
        uint32_t neg;
        uint64_t A0;
        int ea;
        state_split(acc, neg, A0, ea);
        for (uint64_t s = 0; s < len; ++s) tp[s] = s >= k0 ? pack(term(x[base + s], w[base + s], ea, neg)) : 0ull;
        for (;;) {
            ++rounds;
            uint64_t A = A0, bad = len;
            for (uint64_t s = k0; s < len; ++s) {
                int64_t q;
                if (!step(unpack(tp[s]), A, (uint32_t)(A & 1u), q)) {
                    bad = s;
                    break;
                }
                A = (uint64_t)((int64_t)A + q);
            }
            acc = state_join(neg, A, ea);
            if (bad == len) break;
            acc = std::fma(x[base + bad], w[base + bad], acc);
            k0 = bad + 1;
            while (k0 < len && !state_ok(acc)) {
                acc = std::fma(x[base + k0], w[base + k0], acc);
                ++k0;
            }
            if (k0 >= len) break;
            uint32_t neg2;
            uint64_t A2;
            int ea2;
            state_split(acc, neg2, A2, ea2);
            const bool shift = neg2 == neg && ea2 >= ea;
            for (uint64_t s = k0; s < len; ++s) {
                Term t = unpack(tp[s]);
                if (shift && !(t.flags & kBad)) {
                    shift_term(t, ea2 - ea);
                    tp[s] = pack(t);
                } else {
                    tp[s] = pack(term(x[base + s], w[base + s], ea2, neg2));
                }
            }
            neg = neg2;
            A0 = A2;
            ea = ea2;
        }
    }
    if (rounds_out) *rounds_out = rounds;
    return acc;
}

#ifdef __CUDACC__
// Scratch of one warp group running group_fma_chain (shared memory).
struct ChainScratch {
    uint32_t map_a[8], map_b[8];  // per-warp parity maps
    long long sum[8];             // per-warp integer sums
    uint32_t bad[8];              // per-warp first invalid step
    unsigned long long a_bad;     // running integer at the first invalid step
};

namespace chain_detail {

__device__ __forceinline__ void group_bar(int id, int threads) {
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(threads) : "memory");
}

}  // namespace chain_detail

// CTA-cooperative form: the W warps starting at warp `w0` evaluate the chain
// over x[0..n), w[0..n) from `acc`; every thread of the group returns the
// result.  Steps are split into super-blocks of W*32*E, each thread owning E
// consecutive steps; a round scans the parity maps and the integer steps of
// the whole super-block at once, and a binade change (a new round) shifts the
// thread's cached terms instead of decoding them again.  Synchronises the
// group with named barrier `bar_id` (not 0).
template <int W, int E>
__device__ __forceinline__ double group_fma_chain(const double* x, const double* w, uint32_t n, double acc,
                                                  uint32_t w0, int bar_id, ChainScratch& sc) {
    using namespace chain_detail;
    constexpr uint32_t NT = W * 32, SB = NT * E;
    constexpr uint32_t kNone = 0xFFFFFFFFu;
    const uint32_t tg = threadIdx.x - w0 * 32, lane = tg & 31u, wg = tg >> 5;
    for (uint32_t base = 0; base < n; base += SB) {
        const uint32_t len = n - base < SB ? n - base : SB;
        uint32_t k0 = 0;
        // the first steps change binade every few steps: run them plainly
        const uint32_t early = base == 0 ? (len < 32u ? len : 32u) : 0u;
        while (k0 < early || (k0 < len && !state_ok(acc))) {
            acc = fma(x[base + k0], w[base + k0], acc);
            ++k0;
        }
        if (k0 >= len) continue;
        uint32_t neg;
        uint64_t A0;
        int ea;
        state_split(acc, neg, A0, ea);
        const uint32_t my0 = tg * E;  // first step of this thread within the super-block
        uint64_t tp[E];               // packed terms
#pragma unroll
        for (uint32_t i = 0; i < E; ++i) {
            const uint32_t s = my0 + i;
            tp[i] = (s >= k0 && s < len) ? pack(term(x[base + s], w[base + s], ea, neg)) : 0ull;
        }
        for (;;) {
            // --- parity maps: par' = (a & par) ^ b; steps before k0 are identity
            uint32_t pa = 1u, pb = 0u;
#pragma unroll
            for (uint32_t i = 0; i < E; ++i) {
                const Term t = unpack(tp[i]);
                if (t.flags & kTie) {
                    pa = 0u;
                    pb = 0u;
                } else {
                    pb ^= parity_flip(t);
                }
            }
#pragma unroll
            for (uint32_t o = 1; o < 32; o <<= 1) {
                const uint32_t qa = __shfl_up_sync(0xffffffffu, pa, o), qb = __shfl_up_sync(0xffffffffu, pb, o);
                if (lane >= o) {
                    pb = (pa & qb) ^ pb;
                    pa = qa & pa;
                }
            }
            if (lane == 31) {
                sc.map_a[wg] = pa;
                sc.map_b[wg] = pb;
            }
            uint32_t xa = __shfl_up_sync(0xffffffffu, pa, 1), xb = __shfl_up_sync(0xffffffffu, pb, 1);
            if (lane == 0) {
                xa = 1u;
                xb = 0u;
            }
            group_bar(bar_id, NT);
            // maps of the warps before this one, then this warp's exclusive part
            uint32_t ga = 1u, gb = 0u;
            for (uint32_t v = 0; v < wg; ++v) {
                gb = (sc.map_a[v] & gb) ^ sc.map_b[v];
                ga = sc.map_a[v] & ga;
            }
            const uint32_t ca = xa & ga, cb = (xa & gb) ^ xb;
            const uint32_t par = (ca & (uint32_t)(A0 & 1u)) ^ cb;
            // --- integer steps
            long long lane_sum = 0;
            {
                uint32_t p = par;
#pragma unroll
                for (uint32_t i = 0; i < E; ++i) {
                    const Term t = unpack(tp[i]);
                    const uint64_t mag = t.F + ((t.flags & kGtHalf) ? 1u : 0u) +
                                         ((t.flags & kTie) ? (p ^ (uint32_t)(t.F & 1u)) : 0u);
                    lane_sum += (t.flags & kNeg) ? -(long long)mag : (long long)mag;
                    p = (t.flags & kTie) ? 0u : p ^ parity_flip(t);
                }
            }
            long long incl = lane_sum;
#pragma unroll
            for (uint32_t o = 1; o < 32; o <<= 1) {
                const long long v = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += v;
            }
            if (lane == 31) sc.sum[wg] = incl;
            group_bar(bar_id, NT);
            long long before = 0, total = 0;
            for (uint32_t v = 0; v < (uint32_t)W; ++v) {
                const long long sv = sc.sum[v];
                if (v < wg) before += sv;
                total += sv;
            }
            // --- validity of each step from the exact running integer
            uint64_t A = (uint64_t)((long long)A0 + before + incl - lane_sum);
            uint32_t first_bad = kNone;
            uint64_t A_at_bad = 0;
            {
                uint32_t p = par;
#pragma unroll
                for (uint32_t i = 0; i < E; ++i) {
                    const uint32_t s = my0 + i;
                    const Term t = unpack(tp[i]);
                    if (first_bad == kNone && s >= k0 && s < len) {
                        int64_t q;
                        if (!step(t, A, p, q)) {
                            first_bad = s;
                            A_at_bad = A;
                        } else {
                            A = (uint64_t)((long long)A + q);
                        }
                    }
                    p = (t.flags & kTie) ? 0u : p ^ parity_flip(t);
                }
            }
            const uint32_t wbad = __reduce_min_sync(0xffffffffu, first_bad);
            if (lane == 0) sc.bad[wg] = wbad;
            group_bar(bar_id, NT);
            uint32_t bad = kNone;
            for (uint32_t v = 0; v < (uint32_t)W; ++v) bad = sc.bad[v] < bad ? sc.bad[v] : bad;
            if (bad == kNone) {
                acc = state_join(neg, (uint64_t)((long long)A0 + total), ea);
                group_bar(bar_id, NT);  // the scratch is reused by the next super-block
                break;
            }
            if (first_bad == bad) sc.a_bad = A_at_bad;
            group_bar(bar_id, NT);
            acc = state_join(neg, (uint64_t)sc.a_bad, ea);
            acc = fma(x[base + bad], w[base + bad], acc);
            k0 = bad + 1;
            while (k0 < len && !state_ok(acc)) {
                acc = fma(x[base + k0], w[base + k0], acc);
                ++k0;
            }
            group_bar(bar_id, NT);  // every thread has read the scratch
            if (k0 >= len) break;
            uint32_t neg2;
            uint64_t A2;
            int ea2;
            state_split(acc, neg2, A2, ea2);
            const bool shift = neg2 == neg && ea2 >= ea;
#pragma unroll
            for (uint32_t i = 0; i < E; ++i) {
                const uint32_t s = my0 + i;
                Term t = unpack(tp[i]);
                if (s < k0 || s >= len) {
                    tp[i] = 0ull;
                } else if (shift && !(t.flags & kBad)) {
                    shift_term(t, ea2 - ea);
                    tp[i] = pack(t);
                } else {
                    tp[i] = pack(term(x[base + s], w[base + s], ea2, neg2));
                }
            }
            neg = neg2;
            A0 = A2;
            ea = ea2;
        }
    }
    return acc;
}
#endif

}  // namespace deac
