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
constexpr uint32_t kBig = 32u;  // with kBad: finite, but 2^54 or more on this grid

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
    mul_wide(mx, mw, hi, lo);  // P < 2^106, |v| = P / 2^r
    const int r = ea - ex - ew;
    if (r >= 51) {
        // the usual case, without 128-bit variable shifts: h = floor(P / 2^42)
        // (P < 2^106 fits), the bits below 2^42 only as a sticky flag; the
        // half bit of |v| is bit r-1-42 >= 8 of h
        const uint64_t h = (lo >> 42) | (hi << 22);
        const uint32_t low = (lo << 22) != 0 ? 1u : 0u;
        const int hb = r - 43;
        uint64_t F;
        uint32_t half, sticky;
        if (hb < 63) {
            F = h >> (hb + 1);
            half = (uint32_t)(h >> hb) & 1u;
            sticky = ((h << (64 - hb)) != 0 ? 1u : 0u) | low;
        } else if (hb == 63) {
            F = 0;
            half = (uint32_t)(h >> 63);
            sticky = ((h << 1) != 0 ? 1u : 0u) | low;
        } else {
            F = 0;
            half = 0;
            sticky = 1;  // 0 < |v| < 1/2 (P > 0)
        }
        if ((F >> 54) != 0) {
            t.flags = kBad | kBig;
            return t;
        }
        t.F = F;
        t.flags = (half && sticky ? kGtHalf : 0u) | (half && !sticky ? kTie : 0u) | (half || sticky ? kGtZero : 0u) |
                  (neg ? kNeg : 0u);
        return t;
    }
    const int sh = -r;
    uint32_t half = 0, sticky = 0;
    if (sh >= 0) {
        if (sh >= 54 || hi != 0 || (lo >> (54 - sh)) != 0) {
            t.flags = kBad | kBig;  // |v| >= 2^54: leaves the binade for sure
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
                t.flags = kBad | kBig;
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

// One pass over the steps [k0, len) of a super-block from the state
// (A0, ea) (positive), with the steps' terms cached relative to ea: predict
// where the running sum crosses into higher binades (from the prefix of the
// integer parts), sum the rounded integer steps of each predicted binade --
// twice, for either parity of the binade's first state, since the ties to
// even make the sum depend on it -- chain the binades with the crossing
// steps run as plain fma, and verify every step's range condition.  Returns
// the position up to which the chain is done, with the state there in *acc;
// the caller continues from it.  This is the sequential statement of the
// device pass in group_fma_chain.
inline uint64_t host_predicted_pass(const double* x, const double* w, const uint64_t* tp, uint64_t k0,
                                    uint64_t len, uint64_t A0, int ea, double* acc) {
    using namespace chain_detail;
    const uint64_t n = len - k0;
    uint64_t ftot = 0;
    for (uint64_t i = 0; i < n; ++i) {
        if (unpack(tp[k0 + i]).flags & (kNeg | kBad)) return k0;  // not a positive run: no prediction
        ftot += unpack(tp[k0 + i]).F;  // each below 2^54: the total is checked before it can overflow
        if (ftot >= (1ull << 60)) return k0;  // every prefix stays below 2^61
    }
    std::vector<uint32_t> cross(n), seg(n);
    std::vector<int> ds(n), dk(n);
    // predicted binade (relative to ea) of the state before each step and of
    // the step's exact sum
    uint64_t prefix = A0;
    for (uint64_t i = 0; i < n; ++i) {
        const Term t = unpack(tp[k0 + i]);
        const uint64_t T = prefix + t.F + ((t.flags & kGtZero) ? 1u : 0u);
        const int bs = 64 - __builtin_clzll(prefix), bt = 64 - __builtin_clzll(T);
        ds[i] = bs - 53 > 0 ? bs - 53 : 0;
        dk[i] = bt - 53 > 0 ? bt - 53 : 0;
        cross[i] = dk[i] > ds[i];
        prefix += t.F;
    }
    // per segment (the steps between crossings, in the grid of their binade)
    // and per parity p0 of its first state: the exclusive prefix P_p0 of the
    // rounded integer steps, and the inclusive one
    std::vector<uint64_t> cpos;
    std::vector<int> cbin;
    std::vector<int64_t> P0(n), P1(n), I0(n), I1(n);
    std::vector<uint64_t> Fs(n);
    uint32_t cnt = 0;
    int64_t r0 = 0, r1 = 0;
    uint32_t ma = 1, mb = 0;  // parity map from the segment start
    for (uint64_t i = 0; i < n; ++i) {
        if (cross[i]) {
            cpos.push_back(k0 + i);
            cbin.push_back(dk[i]);
            ++cnt;
            r0 = r1 = 0;
            ma = 1;
            mb = 0;
            seg[i] = cnt;
            P0[i] = P1[i] = I0[i] = I1[i] = 0;
            continue;
        }
        Term t = unpack(tp[k0 + i]);
        shift_term(t, ds[i]);
        Fs[i] = t.F;
        seg[i] = cnt;
        P0[i] = r0;
        P1[i] = r1;
        for (uint32_t p0 = 0; p0 < 2; ++p0) {
            const uint32_t par = (ma & p0) ^ mb;
            const uint64_t mag = t.F + ((t.flags & kGtHalf) ? 1u : 0u) + ((t.flags & kTie) ? (par ^ (uint32_t)(t.F & 1u)) : 0u);
            (p0 ? r1 : r0) += (int64_t)mag;
        }
        if (t.flags & kTie) {
            ma = 0;
            mb = 0;
        } else {
            mb ^= parity_flip(t);
        }
        I0[i] = r0;
        I1[i] = r1;
    }
    // chain the segments
    const uint32_t nseg = cnt + 1;
    std::vector<uint64_t> Astart(nseg);
    uint64_t fail = len;  // first segment start whose state is not the predicted one
    double fail_acc = 0.0;
    double a = state_join(0, A0, ea);
    for (uint32_t m = 0; m < nseg; ++m) {
        const int j = m == 0 ? 0 : cbin[m - 1];
        const uint64_t start = m == 0 ? k0 : cpos[m - 1] + 1;
        const uint64_t end = m < cnt ? cpos[m] : len;  // exclusive
        uint32_t ng;
        uint64_t A;
        int e;
        if (!state_ok(a) || (state_split(a, ng, A, e), ng != 0 || e != ea + j)) {
            fail = start;
            fail_acc = a;
            break;
        }
        Astart[m] = A;
        const int64_t Q = end > start ? ((A & 1u) ? I1[end - 1 - k0] : I0[end - 1 - k0]) : 0;
        a = state_join(0, A + (uint64_t)Q, e);
        if (m < cnt) a = std::fma(x[cpos[m]], w[cpos[m]], a);
    }
    // verify the steps before the first mismatch
    for (uint64_t i = 0; i < n && k0 + i < fail; ++i) {
        if (cross[i]) continue;
        const uint64_t As = Astart[seg[i]];
        const uint64_t A = As + (uint64_t)((As & 1u) ? P1[i] : P0[i]);
        if (A + Fs[i] > kTwo53 - 1 || A < kTwo52 || A >= kTwo53) {
            const int j = seg[i] == 0 ? 0 : cbin[seg[i] - 1];
            *acc = state_join(0, A, ea + j);  // the state before this step
            return k0 + i;
        }
    }
    *acc = fail < len ? fail_acc : a;
    return fail;
}

// Host form of group_fma_chain: the same super-blocks, plain first steps,
// rounds and term shifts, with the scans walked sequentially.
inline double host_group_fma_chain(const double* x, const double* w, uint64_t n, double acc, uint64_t SB,
                                   uint64_t* rounds_out = nullptr, bool predict = true) {
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
        if (neg == 0 && predict) {
            double a2;
            const uint64_t done = host_predicted_pass(x + base, w + base, tp.data(), k0, len, A0, ea, &a2);
            if (done > k0) {
                acc = a2;
                k0 = done;
                if (k0 >= len) continue;
                uint32_t neg2;
                uint64_t A2;
                int ea2;
                state_split(acc, neg2, A2, ea2);
                if (!state_ok(acc)) {
                    acc = std::fma(x[base + k0], w[base + k0], acc);
                    ++k0;
                    while (k0 < len && !state_ok(acc)) {
                        acc = std::fma(x[base + k0], w[base + k0], acc);
                        ++k0;
                    }
                    if (k0 >= len) continue;
                    state_split(acc, neg2, A2, ea2);
                }
                for (uint64_t s = k0; s < len; ++s) tp[s] = pack(term(x[base + s], w[base + s], ea2, neg2));
                neg = neg2;
                A0 = A2;
                ea = ea2;
            }
        }
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
constexpr uint32_t kMaxCross = 64;  // binade crossings one predicted pass handles
constexpr int kMaxPredictedPasses = 4;  // per super-block, before the rounds take over
constexpr uint32_t kChainMaxWarps = 16;
struct ChainScratch {
    uint32_t map_a[kChainMaxWarps], map_b[kChainMaxWarps];  // per-warp parity maps
    long long sum[kChainMaxWarps];                          // per-warp integer sums
    uint32_t bad[kChainMaxWarps];                           // per-warp first invalid step
    unsigned long long a_bad;     // running integer at the first invalid step
    // predicted pass
    uint32_t cnt[kChainMaxWarps];   // per-warp crossing counts
    long long sum1[kChainMaxWarps]; // per-warp sums for the other start parity
    uint32_t flag[kChainMaxWarps];  // per-warp "not a positive run"
    uint32_t cpos[kMaxCross];     // position of each crossing step
    int32_t cbin[kMaxCross];      // binade (relative) after it
    long long segq[2][kMaxCross + 1];          // per segment and start parity: its integer sum
    unsigned long long astart[kMaxCross + 1];  // state of each segment's first step
    uint8_t first_cross[kChainMaxWarps * 32];  // per thread: its first step is a crossing
    unsigned long long fail_state;
    uint32_t fail_pos;
    int32_t fail_bin;
    // results of the group's one-thread sequential parts
    uint32_t grow[kChainMaxWarps];  // per warp: a term too large for the unit prefix
    double early_acc;      // state after the plain first steps
    uint32_t early_k0;     // steps done plainly
    double pass_acc;       // state where the predicted pass stopped
    uint32_t pass_fail;    // position where the chaining of the segments stopped
    uint32_t pass_ranged;  // every chained segment ended inside its binade
};

namespace chain_detail {

// The non-aligned barrier: the threads of a warp may arrive diverged (after
// a branch taken by one thread, e.g. the group's one-thread sequential
// parts); the aligned form (bar.sync) requires the warp to arrive converged.
__device__ __forceinline__ void group_bar(int id, int threads) {
    asm volatile("barrier.sync %0, %1;" ::"r"(id), "r"(threads) : "memory");
}

}  // namespace chain_detail

namespace chain_detail {

// segmented-scan elements: c crossings in the range; after the last one (or
// from the range start) the parity map (a, b) resp. the sums (s0, s1)
struct SegMap {
    uint32_t c, a, b;
};
struct SegSum {
    uint32_t c;
    long long s0, s1;
};
__device__ __forceinline__ SegMap seg_combine(const SegMap& L, const SegMap& R) {
    if (R.c) return SegMap{L.c + R.c, R.a, R.b};
    return SegMap{L.c, L.a & R.a, (R.a & L.b) ^ R.b};
}
__device__ __forceinline__ SegSum seg_combine(const SegSum& L, const SegSum& R) {
    if (R.c) return SegSum{L.c + R.c, R.s0, R.s1};
    return SegSum{L.c, L.s0 + R.s0, L.s1 + R.s1};
}
// Both at once: c crossings; after the last one (or from the range start)
// the parity map (a, b) and the sums (s0, s1) of the steps for start
// parities 0 and 1.  Composing L then R without a crossing in R, R's start
// parity is L's map applied to L's start parity.
struct SegAll {
    uint32_t c, a, b;
    long long s0, s1;
};
__device__ __forceinline__ SegAll seg_combine(const SegAll& L, const SegAll& R) {
    if (R.c) return SegAll{L.c + R.c, R.a, R.b, R.s0, R.s1};
    const uint32_t p0 = L.b, p1 = L.a ^ L.b;  // R's start parity for L's start parity 0, 1
    return SegAll{L.c, L.a & R.a, (R.a & L.b) ^ R.b, L.s0 + (p0 ? R.s1 : R.s0), L.s1 + (p1 ? R.s1 : R.s0)};
}

// Exclusive group scan of a per-thread aggregate: warp shuffles, then the
// warps' totals through shared memory.  `tot` receives the group total.
template <int W>
__device__ __forceinline__ SegMap group_scan(SegMap v, uint32_t lane, uint32_t wg, int bar_id, ChainScratch& sc,
                                             SegMap& tot) {
    SegMap inc = v;
#pragma unroll
    for (uint32_t o = 1; o < 32; o <<= 1) {
        const SegMap u{__shfl_up_sync(0xffffffffu, inc.c, o), __shfl_up_sync(0xffffffffu, inc.a, o),
                       __shfl_up_sync(0xffffffffu, inc.b, o)};
        if (lane >= o) inc = seg_combine(u, inc);
    }
    SegMap ex{__shfl_up_sync(0xffffffffu, inc.c, 1), __shfl_up_sync(0xffffffffu, inc.a, 1),
              __shfl_up_sync(0xffffffffu, inc.b, 1)};
    if (lane == 0) ex = SegMap{0u, 1u, 0u};
    if (lane == 31) {
        sc.cnt[wg] = inc.c;
        sc.map_a[wg] = inc.a;
        sc.map_b[wg] = inc.b;
    }
    group_bar(bar_id, W * 32);
    SegMap before{0u, 1u, 0u}, all{0u, 1u, 0u};
    for (uint32_t k = 0; k < (uint32_t)W; ++k) {
        const SegMap t{sc.cnt[k], sc.map_a[k], sc.map_b[k]};
        if (k < wg) before = seg_combine(before, t);
        all = seg_combine(all, t);
    }
    group_bar(bar_id, W * 32);
    tot = all;
    return seg_combine(before, ex);
}
template <int W>
__device__ __forceinline__ SegSum group_scan(SegSum v, uint32_t lane, uint32_t wg, int bar_id, ChainScratch& sc) {
    SegSum inc = v;
#pragma unroll
    for (uint32_t o = 1; o < 32; o <<= 1) {
        const SegSum u{__shfl_up_sync(0xffffffffu, inc.c, o), __shfl_up_sync(0xffffffffu, inc.s0, o),
                       __shfl_up_sync(0xffffffffu, inc.s1, o)};
        if (lane >= o) inc = seg_combine(u, inc);
    }
    SegSum ex{__shfl_up_sync(0xffffffffu, inc.c, 1), __shfl_up_sync(0xffffffffu, inc.s0, 1),
              __shfl_up_sync(0xffffffffu, inc.s1, 1)};
    if (lane == 0) ex = SegSum{0u, 0, 0};
    if (lane == 31) {
        sc.cnt[wg] = inc.c;
        sc.sum[wg] = inc.s0;
        sc.sum1[wg] = inc.s1;
    }
    group_bar(bar_id, W * 32);
    SegSum before{0u, 0, 0};
    for (uint32_t k = 0; k < wg; ++k) before = seg_combine(before, SegSum{sc.cnt[k], sc.sum[k], sc.sum1[k]});
    group_bar(bar_id, W * 32);
    return seg_combine(before, ex);
}

template <int W>
__device__ __forceinline__ SegAll group_scan(SegAll v, uint32_t lane, uint32_t wg, int bar_id, ChainScratch& sc,
                                            uint32_t& total_c) {
    SegAll inc = v;
#pragma unroll
    for (uint32_t o = 1; o < 32; o <<= 1) {
        const SegAll u{__shfl_up_sync(0xffffffffu, inc.c, o), __shfl_up_sync(0xffffffffu, inc.a, o),
                       __shfl_up_sync(0xffffffffu, inc.b, o), __shfl_up_sync(0xffffffffu, inc.s0, o),
                       __shfl_up_sync(0xffffffffu, inc.s1, o)};
        if (lane >= o) inc = seg_combine(u, inc);
    }
    SegAll ex{__shfl_up_sync(0xffffffffu, inc.c, 1), __shfl_up_sync(0xffffffffu, inc.a, 1),
              __shfl_up_sync(0xffffffffu, inc.b, 1), __shfl_up_sync(0xffffffffu, inc.s0, 1),
              __shfl_up_sync(0xffffffffu, inc.s1, 1)};
    if (lane == 0) ex = SegAll{0u, 1u, 0u, 0, 0};
    if (lane == 31) {
        sc.cnt[wg] = inc.c;
        sc.map_a[wg] = inc.a;
        sc.map_b[wg] = inc.b;
        sc.sum[wg] = inc.s0;
        sc.sum1[wg] = inc.s1;
    }
    group_bar(bar_id, W * 32);
    SegAll before{0u, 1u, 0u, 0, 0};
    uint32_t tc = 0;
    for (uint32_t k = 0; k < (uint32_t)W; ++k) {
        const uint32_t ck = sc.cnt[k];
        if (k < wg) before = seg_combine(before, SegAll{ck, sc.map_a[k], sc.map_b[k], sc.sum[k], sc.sum1[k]});
        tc += ck;
    }
    group_bar(bar_id, W * 32);
    total_c = tc;
    return seg_combine(before, ex);
}

// binade (relative to the pass's grid) of an integer multiple of the grid
__device__ __forceinline__ int rel_binade(uint64_t v, int c = 0) {  // v in units of 2^c of the grid
    const int b = 64 - __clzll((long long)v) + c;
    return b - 53 > 0 ? b - 53 : 0;
}

}  // namespace chain_detail

// A term decoded on the grid 2^e of a positive state, out of line: the
// predicted pass calls it only for the rare terms beyond its start grid, and
// one copy keeps the unrolled loops small.
static __device__ __noinline__ uint64_t packed_term(double x, double w, int e) {
    return chain_detail::pack(chain_detail::term(x, w, e, 0));
}

// Position of step k in x and w: the plain order, or (kSwz) one super-block
// stored step-major per thread -- step t*E + i at i*(W*32) + t -- so that the
// group's threads read their E steps from consecutive addresses.
template <int W, int E, bool kSwz>
__device__ __forceinline__ uint32_t chain_slot(uint32_t k) {
    return kSwz ? (k % (uint32_t)E) * (uint32_t)(W * 32) + k / (uint32_t)E : k;
}

// The predicted pass of host_predicted_pass, by the W warps of a group, each
// thread over its E cached terms tp (steps tg*E + i of the super-block, the
// ones before k0 and from len_all on are zero).  It covers the steps before
// the first one whose term it cannot place: a negative term, or one beyond
// the grid (at least 2^54 units: a sure binade change, `at_bad` when the pass
// stops there).  Returns the position reached and the state there in acc
// (uniform over the group).
template <int W, int E, bool kSwz>
__device__ __forceinline__ uint32_t group_predicted_pass(const double* x, const double* w, uint64_t (&tp)[E],
                                                          uint32_t k0, uint32_t len_all, uint64_t A0, int ea,
                                                          double& acc, uint32_t tg, int bar_id, ChainScratch& sc,
                                                          bool& rewritten, bool& at_bad) {
    using namespace chain_detail;
    rewritten = false;
    at_bad = false;
    acc = state_join(0, A0, ea);
    constexpr uint32_t NT = W * 32;
    static_assert(W <= (int)kChainMaxWarps, "group larger than its scratch");
    constexpr uint32_t kNone = 0xFFFFFFFFu;
    const uint32_t lane = tg & 31u, wg = tg >> 5, my0 = tg * E;
    // The prefix predicts binades only, in units of 2^c of the start grid
    // (its error near a binade edge is caught by the checks below).  A term
    // beyond the start grid (kBig: a state that grows several-fold within
    // the super-block, a peak after small first steps) is placed on the grid
    // 2^(c + kCoarse) -- its F there, times 2^kCoarse, stands in for it in
    // the prefix -- and decoded again on its predicted binade's grid below.
    // Attempts: units 1, then 2^16 when the prefixes outgrow their budget
    // (a growth beyond 2^8, or one term beyond it), then the old rule: the
    // pass ends at the first term beyond the start grid.
    constexpr int kCoarse = 8, kUnitStep = 16;
    uint32_t len = len_all;
    bool stop_bad = false;
    uint64_t pstart = 0;
    int c = 0;  // prefix units 2^c
    for (int attempt = 0;; ++attempt) {
        c = attempt == 1 ? kUnitStep : 0;
        // --- the first unplaceable step (position * 2 + 1 when negative)
        uint32_t key = kNone, grow = 0;
#pragma unroll
        for (uint32_t i = 0; i < E; ++i) {
            const uint32_t s = my0 + i;
            Term t = unpack(tp[i]);
            if (key != kNone || s < k0 || s >= len_all) continue;
            if (attempt < 2 && (t.flags & kBig)) {
                const uint32_t q = chain_slot<W, E, kSwz>(s);
                t = unpack(packed_term(x[q], w[q], ea + c + kCoarse));
                if (!(t.flags & (kNeg | kBad)) && t.F < (1ull << (57 - kCoarse))) {
                    tp[i] = pack(Term{t.F, kBad | kBig});  // F on the coarse grid
                    continue;
                }
                if (attempt == 0 && !(t.flags & kNeg) && (!(t.flags & kBad) || (t.flags & kBig))) {
                    grow = 1u;  // beyond the unit prefix's budget: coarser units
                    continue;
                }
                key = (s << 1) | ((t.flags & kNeg) ? 1u : 0u);  // beyond the coarse budget too
                continue;
            }
            if (t.flags & (kNeg | kBad)) key = (s << 1) | ((t.flags & kNeg) ? 1u : 0u);
        }
        key = __reduce_min_sync(0xffffffffu, key);
        grow = __any_sync(0xffffffffu, grow != 0);
        if (lane == 0) {
            sc.bad[wg] = key;
            sc.grow[wg] = grow;
        }
        group_bar(bar_id, NT);
        for (uint32_t k = 0; k < (uint32_t)W; ++k) {
            key = sc.bad[k] < key ? sc.bad[k] : key;
            grow |= sc.grow[k];
        }
        if (attempt == 0 && grow) {
            group_bar(bar_id, NT);  // the scratch is reused next
            continue;               // straight to the coarser units
        }
        len = key == kNone ? len_all : key >> 1;
        stop_bad = key != kNone && !(key & 1u);
        if (len <= k0) {
            at_bad = stop_bad;
            group_bar(bar_id, NT);  // the scratch is reused next
            return k0;
        }
        // --- prefix of the integer parts up to len.  Every F below len is
        // under 2^57 (coarse ones scaled), a thread's part is clamped there
        // and a warp's stays below 2^62; warp totals below 2^57 keep every
        // prefix of the group below 2^61.
        long long fsum = 0;
#pragma unroll
        for (uint32_t i = 0; i < E; ++i) {
            const Term t = unpack(tp[i]);
            if (my0 + i < len) fsum += (long long)((t.flags & kBig) ? t.F << kCoarse : t.F >> c);
        }
        fsum = fsum < (1ll << 57) ? fsum : (1ll << 57);
        long long finc = fsum;
#pragma unroll
        for (uint32_t o = 1; o < 32; o <<= 1) {
            const long long v = __shfl_up_sync(0xffffffffu, finc, o);
            if (lane >= o) finc += v;
        }
        if (lane == 31) {
            sc.sum[wg] = finc;
            sc.flag[wg] = finc >= (1ll << 57) ? 1u : 0u;
        }
        group_bar(bar_id, NT);
        long long fbefore = 0;
        uint32_t anybad = 0;
        for (uint32_t k = 0; k < (uint32_t)W; ++k) {
            if (k < wg) fbefore += sc.sum[k];
            anybad |= sc.flag[k];
        }
        group_bar(bar_id, NT);
        if (!anybad) {
            pstart = (A0 >> c) + (uint64_t)(fbefore + finc - fsum);
            break;
        }
        if (attempt == 2) return k0;
        if (attempt == 1) {
            // the last attempt: terms beyond the start grid end the pass
#pragma unroll
            for (uint32_t i = 0; i < E; ++i)
                if (unpack(tp[i]).flags & kBig) tp[i] = pack(Term{0ull, kBad | kBig});
        }
    }
    rewritten = true;
    if (len < len_all) {
        // the steps from the unplaceable one on are not this pass's
#pragma unroll
        for (uint32_t i = 0; i < E; ++i)
            if (my0 + i >= len) tp[i] = 0ull;
    }

    // --- crossings (a step whose exact sum lies in a higher binade than its
    // state) and the parity maps of the segments between them
    // From here on tp[i] holds the step's term in the grid of its predicted
    // binade (a crossing step keeps its binade after the crossing in cbin_of)
    uint32_t cross_bits = 0;
    int cbin_of[E];
    SegAll agg{0u, 1u, 0u, 0, 0};
    {
        // each step's binade before and after it from the prefix (ds, 8 bits
        // a step), its crossing, and the coarse terms to decode again on
        // their step's grid
        uint64_t prefix = pstart, ds_pack = 0;
        uint32_t redo = 0, on_grid = 0;
#pragma unroll
        for (uint32_t i = 0; i < E; ++i) {
            const Term t = unpack(tp[i]);
            const uint32_t s = my0 + i;
            const bool big = (t.flags & kBig) != 0;
            const uint64_t F = big ? t.F << kCoarse : t.F >> c;
            const uint64_t T = prefix + F + ((c == 0 && (t.flags & kGtZero)) ? 1u : 0u);
            const int ds = rel_binade(prefix, c), dk = rel_binade(T, c);
            const bool live = s >= k0 && s < len;
            const bool cr = live && dk > ds;
            cross_bits |= (cr ? 1u : 0u) << i;
            redo |= (big && !cr && live ? 1u : 0u) << i;
            ds_pack |= (uint64_t)(uint32_t)ds << (8 * i);
            cbin_of[i] = dk;
            prefix += F;
        }
        // the coarse term on its own step's grid (a step still beyond it
        // certainly changes binade: a crossing, run plainly); rare, and kept
        // out of the loops around it
        if (__any_sync(0xffffffffu, redo != 0)) {
#pragma unroll
            for (uint32_t i = 0; i < E; ++i) {
                if (!((redo >> i) & 1u)) continue;
                const uint32_t q = chain_slot<W, E, kSwz>(my0 + i);
                const Term t = unpack(packed_term(x[q], w[q], ea + (int)((ds_pack >> (8 * i)) & 0xFFu)));
                if (t.flags & (kNeg | kBad)) {
                    cross_bits |= 1u << i;
                } else {
                    tp[i] = pack(t);
                    on_grid |= 1u << i;
                }
            }
        }
#pragma unroll
        for (uint32_t i = 0; i < E; ++i) {
            if ((cross_bits >> i) & 1u) {
                agg = seg_combine(agg, SegAll{1u, 1u, 0u, 0, 0});
                tp[i] = 0ull;
            } else {
                Term t = unpack(tp[i]);
                if (!((on_grid >> i) & 1u)) shift_term(t, (int)((ds_pack >> (8 * i)) & 0xFFu));
                tp[i] = pack(t);
                // the step for entering parity 0 and 1, and its map
                const long long b0 = (long long)(t.F + ((t.flags & kGtHalf) ? 1u : 0u));
                const bool tie = (t.flags & kTie) != 0;
                const long long f1 = (long long)(t.F & 1u);
                agg = seg_combine(agg, tie ? SegAll{0u, 0u, 0u, b0 + f1, b0 + (f1 ^ 1)}
                                           : SegAll{0u, 1u, parity_flip(t), b0, b0});
            }
        }
    }
    sc.first_cross[tg] = (uint8_t)(cross_bits & 1u);
    for (uint32_t m = tg; m <= kMaxCross; m += NT) {  // empty segments sum to zero
        sc.segq[0][m] = 0;
        sc.segq[1][m] = 0;
    }
    uint32_t ncross;
    const SegAll ex = group_scan<W>(agg, lane, wg, bar_id, sc, ncross);
    if (ncross > kMaxCross) return k0;
    // the map and the sums from the segment's start to this thread's first step
    const SegMap mex{ex.c, ex.a, ex.b};
    const SegSum sex{ex.c, ex.s0, ex.s1};

    // the integer steps of a segment for start parities 0 and 1, given the
    // parity map from the segment's start
    auto steps = [&](Term t, const SegMap& m, long long& q0, long long& q1) {
        const uint64_t base = t.F + ((t.flags & kGtHalf) ? 1u : 0u);
        const uint32_t par0 = m.b, par1 = m.a ^ m.b;
        q0 = (long long)(base + ((t.flags & kTie) ? (par0 ^ (uint32_t)(t.F & 1u)) : 0u));
        q1 = (long long)(base + ((t.flags & kTie) ? (par1 ^ (uint32_t)(t.F & 1u)) : 0u));
    };
    auto next_map = [&](const SegMap& m, const Term& t) {
        return seg_combine(m, (t.flags & kTie) ? SegMap{0u, 0u, 0u} : SegMap{0u, 1u, parity_flip(t)});
    };
    // crossing positions and binades; each segment's sums at its last step
    // (only threads holding a crossing or a segment's last step write)
    const bool next_thread_cross = tg + 1 < NT ? sc.first_cross[tg + 1] != 0 : false;
    if (cross_bits != 0 || next_thread_cross || (len > my0 && len <= my0 + E)) {
        SegMap runm = mex;
        SegSum runs = sex;
#pragma unroll
        for (uint32_t i = 0; i < E; ++i) {
            const Term t = unpack(tp[i]);
            const uint32_t s = my0 + i;
            if ((cross_bits >> i) & 1u) {
                runs = seg_combine(runs, SegSum{1u, 0, 0});
                runm = seg_combine(runm, SegMap{1u, 1u, 0u});
                sc.cpos[runs.c - 1] = s;
                sc.cbin[runs.c - 1] = cbin_of[i];
            } else {
                long long q0, q1;
                steps(t, runm, q0, q1);
                runs = seg_combine(runs, SegSum{0u, q0, q1});
                runm = next_map(runm, t);
                const bool next_cross = i + 1 < E ? ((cross_bits >> (i + 1)) & 1u) != 0 : next_thread_cross;
                if (s >= k0 && s < len && (s + 1 == len || next_cross)) {
                    sc.segq[0][runs.c] = runs.s0;
                    sc.segq[1][runs.c] = runs.s1;
                }
            }
        }
    }
    group_bar(bar_id, NT);

    // --- chain the segments (one thread; the others read the outcome).  A
    // positive run only grows, and each step adds at least its integer part,
    // so a segment whose end state stays below 2^53 had every step inside its
    // binade; only a segment that reaches it needs the step-wise check below.
    if (tg == 0) {
        double a = state_join(0, A0, ea);
        uint32_t fail = len;
        double fail_acc = 0.0;
        uint32_t ranged = 1u;
        for (uint32_t m = 0; m <= ncross; ++m) {
            const int j = m == 0 ? 0 : sc.cbin[m - 1];
            const uint32_t start = m == 0 ? k0 : sc.cpos[m - 1] + 1;
            const uint32_t end = m < ncross ? sc.cpos[m] : len;
            uint32_t ng;
            uint64_t A;
            int e;
            bool ok = state_ok(a);
            if (ok) {
                state_split(a, ng, A, e);
                ok = ng == 0 && e == ea + j;
            }
            if (!ok) {
                fail = start;
                fail_acc = a;
                break;
            }
            sc.astart[m] = A;
            const long long Q = end > start ? sc.segq[A & 1u][m] : 0;
            if (A + (uint64_t)Q > kTwo53 - 1) ranged = 0u;
            a = state_join(0, A + (uint64_t)Q, e);
            if (m < ncross) {
                const uint32_t q = chain_slot<W, E, kSwz>(sc.cpos[m]);
                a = fma(x[q], w[q], a);
            }
        }
        sc.pass_acc = fail < len ? fail_acc : a;
        sc.pass_fail = fail;
        sc.pass_ranged = ranged;
    }
    group_bar(bar_id, NT);
    const uint32_t fail = sc.pass_fail;
    if (sc.pass_ranged) {
        acc = sc.pass_acc;
        at_bad = stop_bad && fail == len;
        return fail;
    }

    // --- verify every step before the first mismatch
    uint32_t first_bad = kNone;
    uint64_t bad_state = 0;
    int bad_bin = 0;
    {
        SegMap runm = mex;
        SegSum runs = sex;
#pragma unroll
        for (uint32_t i = 0; i < E; ++i) {
            const Term t = unpack(tp[i]);
            const uint32_t s = my0 + i;
            if ((cross_bits >> i) & 1u) {
                runs = seg_combine(runs, SegSum{1u, 0, 0});
                runm = seg_combine(runm, SegMap{1u, 1u, 0u});
                continue;
            }
            if (first_bad == kNone && s >= k0 && s < len && s < fail) {
                const uint64_t As = sc.astart[runs.c];
                const uint64_t A = As + (uint64_t)((As & 1u) ? runs.s1 : runs.s0);
                if (A < kTwo52 || A >= kTwo53 || A + t.F > kTwo53 - 1) {
                    first_bad = s;
                    bad_state = A;
                    bad_bin = runs.c == 0 ? 0 : sc.cbin[runs.c - 1];
                }
            }
            long long q0, q1;
            steps(t, runm, q0, q1);
            runs = seg_combine(runs, SegSum{0u, q0, q1});
            runm = next_map(runm, t);
        }
    }
    const uint32_t wmin = __reduce_min_sync(0xffffffffu, first_bad);
    if (lane == 0) sc.bad[wg] = wmin;
    group_bar(bar_id, NT);
    uint32_t bad = kNone;
    for (uint32_t k = 0; k < (uint32_t)W; ++k) bad = sc.bad[k] < bad ? sc.bad[k] : bad;
    if (bad != kNone && first_bad == bad) {
        sc.fail_state = bad_state;
        sc.fail_bin = bad_bin;
    }
    group_bar(bar_id, NT);
    if (bad != kNone) {
        acc = state_join(0, sc.fail_state, ea + sc.fail_bin);
        group_bar(bar_id, NT);  // the scratch is reused next
        return bad;
    }
    acc = sc.pass_acc;
    at_bad = stop_bad && fail == len;
    return fail;
}

// CTA-cooperative form: the W warps starting at warp `w0` evaluate the chain
// over x[0..n), w[0..n) from `acc`; every thread of the group returns the
// result.  Steps are split into super-blocks of W*32*E, each thread owning E
// consecutive steps; a round scans the parity maps and the integer steps of
// the whole super-block at once, and a binade change (a new round) shifts the
// thread's cached terms instead of decoding them again.  Synchronises the
// group with named barrier `bar_id` (not 0).  With kSwz, x and w hold one
// super-block (n <= W*32*E) in the order of chain_slot.
template <int W, int E, bool kPredict = true, bool kSwz = false>
__device__ __forceinline__ double group_fma_chain(const double* x, const double* w, uint32_t n, double acc,
                                                  uint32_t w0, int bar_id, ChainScratch& sc,
                                                  uint32_t early_steps = 32) {
    using namespace chain_detail;
    constexpr uint32_t NT = W * 32, SB = NT * E;
    constexpr uint32_t kNone = 0xFFFFFFFFu;
    const uint32_t tg = threadIdx.x - w0 * 32, lane = tg & 31u, wg = tg >> 5;
    auto xs = [&](uint32_t k) { return x[chain_slot<W, E, kSwz>(k)]; };
    auto ws = [&](uint32_t k) { return w[chain_slot<W, E, kSwz>(k)]; };
    for (uint32_t base = 0; base < n; base += SB) {
        const uint32_t len = n - base < SB ? n - base : SB;
        uint32_t k0 = 0;
        // the first steps change binade every few steps: one thread runs
        // them plainly
        const uint32_t early = base == 0 ? (len < early_steps ? len : early_steps) : 0u;
        if (early > 0 || !state_ok(acc)) {
            if (tg == 0) {
                while (k0 < early || (k0 < len && !state_ok(acc))) {
                    acc = fma(xs(base + k0), ws(base + k0), acc);
                    ++k0;
                }
                sc.early_acc = acc;
                sc.early_k0 = k0;
            }
            group_bar(bar_id, NT);
            acc = sc.early_acc;
            k0 = sc.early_k0;
            if (k0 >= len) {
                group_bar(bar_id, NT);  // every thread has read the scratch
                continue;
            }
        }
        uint32_t neg;
        uint64_t A0;
        int ea;
        state_split(acc, neg, A0, ea);
        const uint32_t my0 = tg * E;  // first step of this thread within the super-block
        uint64_t tp[E];               // packed terms
#pragma unroll
        for (uint32_t i = 0; i < E; ++i) {
            const uint32_t s = my0 + i;
            tp[i] = (s >= k0 && s < len) ? pack(term(xs(base + s), ws(base + s), ea, neg)) : 0ull;
        }
        // predicted passes over the binades of a positive run, each up to
        // the next term beyond its grid (run plainly: a sure binade change)
        for (int pass = 0; kPredict && neg == 0 && pass < kMaxPredictedPasses; ++pass) {
            double a2;
            bool rewritten, at_bad;
            const uint32_t done = group_predicted_pass<W, E, kSwz>(x + base, w + base, tp, k0, len, A0, ea, a2, tg,
                                                                   bar_id, sc, rewritten, at_bad);
            if (!(done > k0 || rewritten || at_bad)) break;  // no progress: the rounds below
            acc = a2;
            k0 = done;
            if (at_bad) {
                acc = fma(xs(base + k0), ws(base + k0), acc);
                ++k0;
            }
            while (k0 < len && !state_ok(acc)) {
                acc = fma(xs(base + k0), ws(base + k0), acc);
                ++k0;
            }
            if (k0 >= len) break;
            // the pass left terms of several grids: decode the rest again
            state_split(acc, neg, A0, ea);
#pragma unroll
            for (uint32_t i = 0; i < E; ++i) {
                const uint32_t s = my0 + i;
                tp[i] = (s >= k0 && s < len) ? pack(term(xs(base + s), ws(base + s), ea, neg)) : 0ull;
            }
        }
        if (k0 >= len) continue;
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
            acc = fma(xs(base + bad), ws(base + bad), acc);
            k0 = bad + 1;
            while (k0 < len && !state_ok(acc)) {
                acc = fma(xs(base + k0), ws(base + k0), acc);
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
                    tp[i] = pack(term(xs(base + s), ws(base + s), ea2, neg2));
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
