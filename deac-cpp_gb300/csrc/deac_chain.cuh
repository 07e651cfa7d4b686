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
// device share the per-step code below; the device form scans 32 lanes at a
// time (warp_fma_chain), the host form walks the same blocks sequentially and
// is the CPU check of the arithmetic.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

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

#ifdef __CUDACC__
// Device form: one warp evaluates the chain over x[0..n), w[0..n) (shared or
// global memory) starting from `acc`; every lane returns the result.  Blocks
// of 32*kChainPerLane steps; lane j owns steps j*kChainPerLane + i.
constexpr uint32_t kChainPerLane = 8;

__device__ __forceinline__ double warp_fma_chain(const double* x, const double* w, uint32_t n, double acc) {
    using namespace chain_detail;
    const uint32_t lane = threadIdx.x & 31u;
    constexpr uint32_t E = kChainPerLane, B = 32 * kChainPerLane;
    uint32_t k = 0;
    uint32_t plain_run = 0;  // steps to run plainly before scanning again
    while (k < n) {
        if (plain_run > 0 || !state_ok(acc)) {
            acc = fma(x[k], w[k], acc);
            ++k;
            if (plain_run > 0) --plain_run;
            continue;
        }
        uint32_t neg;
        uint64_t A0;
        int ea;
        state_split(acc, neg, A0, ea);
        const uint32_t L = n - k < B ? n - k : B;
        // this lane's steps: terms, parity map (a, b): par' = (a & par) ^ b
        Term t[E];
        uint32_t pa = 1u, pb = 0u;
#pragma unroll
        for (uint32_t i = 0; i < E; ++i) {
            const uint32_t s = lane * E + i;
            t[i] = s < L ? term(x[k + s], w[k + s], ea, neg) : Term{0ull, 0u};
            if (t[i].flags & kTie) {
                pa = 0u;
                pb = 0u;
            } else {
                pb ^= parity_flip(t[i]);
            }
        }
        // inclusive scan of the maps over lanes, then the exclusive one
#pragma unroll
        for (uint32_t o = 1; o < 32; o <<= 1) {
            const uint32_t qa = __shfl_up_sync(0xffffffffu, pa, o), qb = __shfl_up_sync(0xffffffffu, pb, o);
            if (lane >= o) {
                pb = (pa & qb) ^ pb;
                pa = qa & pa;
            }
        }
        uint32_t ea_map = __shfl_up_sync(0xffffffffu, pa, 1), eb_map = __shfl_up_sync(0xffffffffu, pb, 1);
        if (lane == 0) {
            ea_map = 1u;
            eb_map = 0u;
        }
        uint32_t par = (ea_map & (uint32_t)(A0 & 1u)) ^ eb_map;
        // the integer steps (garbage after an invalid one, never used)
        int64_t q[E];
        int64_t lane_sum = 0;
#pragma unroll
        for (uint32_t i = 0; i < E; ++i) {
            const uint64_t mag = t[i].F + ((t[i].flags & kGtHalf) ? 1u : 0u) +
                                 ((t[i].flags & kTie) ? (par ^ (uint32_t)(t[i].F & 1u)) : 0u);
            q[i] = (t[i].flags & kNeg) ? -(int64_t)mag : (int64_t)mag;
            par = (t[i].flags & kTie) ? 0u : par ^ parity_flip(t[i]);
            lane_sum += q[i];
        }
        int64_t incl = lane_sum;
#pragma unroll
        for (uint32_t o = 1; o < 32; o <<= 1) {
            const int64_t v = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += v;
        }
        // validity of each step from the exact running integer
        uint64_t A = (uint64_t)((int64_t)A0 + incl - lane_sum);
        uint32_t first_bad = 0xFFFFFFFFu;
        uint64_t A_at_bad = 0;
#pragma unroll
        for (uint32_t i = 0; i < E; ++i) {
            const uint32_t s = lane * E + i;
            if (s < L && first_bad == 0xFFFFFFFFu) {
                int64_t qq;
                // the tie parity is already folded into q[i]; step() is used
                // for the range checks only
                if (!step(t[i], A, (uint32_t)(A & 1u), qq)) {
                    first_bad = s;
                    A_at_bad = A;
                } else {
                    A = (uint64_t)((int64_t)A + q[i]);
                }
            }
        }
        const uint32_t bad = __reduce_min_sync(0xffffffffu, first_bad);
        uint64_t A_end;
        if (bad == 0xFFFFFFFFu) {
            A_end = (uint64_t)((int64_t)A0 + __shfl_sync(0xffffffffu, incl, 31));
        } else {
            A_end = __shfl_sync(0xffffffffu, A_at_bad, bad / E);
        }
        acc = state_join(neg, A_end, ea);
        if (bad == 0xFFFFFFFFu) {
            k += L;
        } else {
            acc = fma(x[k + bad], w[k + bad], acc);
            k += bad + 1;
            if (bad < 16) plain_run = 32;  // little progress: step plainly for a while
        }
    }
    return acc;
}
#endif

}  // namespace deac
