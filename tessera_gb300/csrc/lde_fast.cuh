// SPDX-License-Identifier: Apache-2.0 OR MIT
//
// The encoder's four passes with register-resident sub-transforms (2^13 ≤ k ≤ 2^20).
//
// With k = K1·K2 and the codeword interleaving the 2^r cosets s_e·H (symbol q·2^r + e is
// NTT_k(c_e)[q], c_e[i] = s_e^i·(a_i + m_i (s_e^k − 1)), a = iNTT_k(row)):
//
//   pass A   inverse length-K2 transforms down the strided columns t1, × ω_k^{−j2·t1}  → Y[j2][t1]
//   pass M1  per column j2: inverse length-K1 transform; per coset the scale s_e^i/k
//                                                                               → C_e[j1][j2]
//            (mask_fixup then adds the P mask terms of each row into C_e)
//   pass M2  per coset and column j2: forward length-K1 transform, × ω_k^{v2·j2} → Z_e[v2][j2]
//            (written over C_e: a tile reads all of its columns before it writes)
//   pass C   per coset and column v2: forward length-K2 transform, written interleaved into the
//            codeword at (v2 + K1·v1)·2^r + e
//
// A column transform of length L = RA·RB runs in two rounds. Round 1: each thread takes RA/T
// sub-transforms of length RB (T = L/32 threads per column, 32 elements per thread) over the
// strided elements ta + RA·tb, multiplies output kb by w^{ta·kb}, and parks the results in shared
// memory. Round 2: each thread takes RB/T sub-transforms of length RA over ta for its kb. The
// sub-transforms are radix-2 butterflies fully unrolled in registers whose twiddles are powers of
// ω_R for R ≤ 32, which in Goldilocks are powers of two (ω_32 = 2^78, ω_16 = 2^156, ω_8 = 2^120,
// ω_4 = 2^48, ω_2 = 2^96 = −1, exponents mod 192): a twiddle is a shift and a fold, never a 64 x 64
// product. All arithmetic is lazy (tg::lz): values stay any 64-bit word until the codeword is
// written, and every carry is folded with the carry flag.
//
// Columns of 2,048 (k = 2^21..2^22) keep 32 elements per thread too: round 2's length-64
// sub-transforms are split across two threads. Each loads the 64 values of its sub-transform, does
// the first radix-2 stage on load and keeps one half — the even outputs (sums) or the odd ones
// (differences times ω_64^t, a shift) —, then runs the length-32 transform on it; the two halves
// sit in different warps, so the choice never diverges within a warp.
//
// A CTA holds an 8,192-element tile (W = 8192/L columns, 64 KiB of shared memory) with 256
// threads, so that two CTAs share an SM and one's loads overlap the other's arithmetic. Each
// round maps threads to columns so that its global accesses are coalesced: when the column's
// elements are contiguous in memory the warp runs along the column ("q-fast"), when the
// columns are contiguous the warp runs across columns ("c-fast"); Shape::slot keeps both
// mappings free of shared-memory bank conflicts.
#pragma once
#include <stdint.h>

#include <utility>

#include "gl.cuh"

namespace tg {
namespace fast {

constexpr int TILE = 8192;
constexpr int THREADS = 256;

template <typename F, int... Is>
__device__ __forceinline__ void static_for_impl(F&& f, std::integer_sequence<int, Is...>) {
    (f(std::integral_constant<int, Is>{}), ...);
}
template <int N, typename F>
__device__ __forceinline__ void static_for(F&& f) {
    static_for_impl(f, std::make_integer_sequence<int, N>{});
}

constexpr int ilog2(int x) { return x <= 1 ? 0 : 1 + ilog2(x >> 1); }
constexpr int brev_c(int x, int bits) {
    int r = 0;
    for (int b = 0; b < bits; b++) r |= ((x >> b) & 1) << (bits - 1 - b);
    return r;
}

// ω_R = 2^root_exp(R) (mod p), ω_R = 7^((p−1)/R).
constexpr int root_exp(int R) {
    return R == 1 ? 0 : R == 2 ? 96 : R == 4 ? 48 : R == 8 ? 120 : R == 16 ? 156 : R == 32 ? 78 : 39;
}
// The exponent of ω_R^{±m}, in [0, 192).
constexpr int tw_exp(int R, int m, bool inverse) {
    const int e = (m * root_exp(R)) % 192;
    return inverse ? (192 - e) % 192 : e;
}

// Gentleman–Sande butterfly with twiddle 2^E, E in [0, 192): (a, b) → (a + b, (a − b)·2^E).
template <int E>
__device__ __forceinline__ void bf_gs(uint64_t& a, uint64_t& b) {
    const uint64_t s = lz::add(a, b);
    if constexpr (E >= 96)
        b = lz::mulp2<E - 96>(lz::sub(b, a));
    else
        b = lz::mulp2<E>(lz::sub(a, b));
    a = s;
}

// Cooley–Tukey butterfly with twiddle 2^E: (a, b) → (a + b·2^E, a − b·2^E).
template <int E>
__device__ __forceinline__ void bf_ct(uint64_t& a, uint64_t& b) {
    if constexpr (E >= 96) {
        const uint64_t t = lz::mulp2<E - 96>(b);  // b·2^E = −t
        b = lz::add(a, t);
        a = lz::sub(a, t);
    } else {
        const uint64_t t = lz::mulp2<E>(b);
        b = lz::sub(a, t);
        a = lz::add(a, t);
    }
}

// Length-R transform of x[BASE + i], i < R, with root ω_R^{±1}: natural order in, bit-reversed
// order out (position p holds X[rev(p)]).
// Swaps x[BASE .. BASE + H) with x[BASE + H .. BASE + 2H) (register moves).
template <int H, int BASE, int N>
__device__ __forceinline__ void swap_halves(uint64_t (&x)[N]) {
    static_for<H>([&](auto t_) {
        constexpr int t = decltype(t_)::value;
        const uint64_t y = x[BASE + t];
        x[BASE + t] = x[BASE + H + t];
        x[BASE + H + t] = y;
    });
}

template <int R, bool INV, int BASE, int N>
__device__ __forceinline__ void dft_dif(uint64_t (&x)[N]);

template <int R, bool INV, int BASE, int N>
__device__ __forceinline__ void dft_dif(uint64_t (&x)[N]) {
    static_for<ilog2(R)>([&](auto s_) {
        constexpr int s = decltype(s_)::value;
        constexpr int h = R >> (s + 1);
        static_for<R / 2>([&](auto b_) {
            constexpr int b = decltype(b_)::value;
            constexpr int o = b % h, g = b / h;
            constexpr int i0 = g * 2 * h + o;
            bf_gs<tw_exp(R, o << s, INV)>(x[BASE + i0], x[BASE + i0 + h]);
        });
    });
}

// Cache hints: the input rows are read once and the codewords written once, so both stream past
// L2 (evict-first); the group's scratch (Y, C_e/Z_e) is written with evict-last so that it is still
// in L2 when the next pass reads it.
__device__ __forceinline__ uint64_t policy_first() {
    uint64_t pol;
    asm("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
    return pol;
}
__device__ __forceinline__ uint64_t policy_last() {
    uint64_t pol;
    asm("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(pol));
    return pol;
}
__device__ __forceinline__ ulonglong2 ld_hint(const uint64_t* p, uint64_t pol) {
    ulonglong2 v;
    asm("ld.global.L2::cache_hint.v2.u64 {%0, %1}, [%2], %3;" : "=l"(v.x), "=l"(v.y) : "l"(p), "l"(pol));
    return v;
}
__device__ __forceinline__ void st_hint(uint64_t* p, uint64_t v, uint64_t pol) {
    asm volatile("st.global.L2::cache_hint.u64 [%0], %1, %2;" ::"l"(p), "l"(v), "l"(pol) : "memory");
}
__device__ __forceinline__ ulonglong2 ld_stream(const uint64_t* p) { return ld_hint(p, policy_first()); }
__device__ __forceinline__ void st_stream(uint64_t* p, uint64_t v) { st_hint(p, v, policy_first()); }
__device__ __forceinline__ void st_keep(uint64_t* p, uint64_t v) { st_hint(p, v, policy_last()); }

struct Args {
    const uint64_t* rows;
    const uint64_t* masks;
    uint64_t* y;            // k words per row
    uint64_t* z;            // n words per row: C_e, then Z_e in place
    uint64_t* out;
    const uint64_t* pw;     // ω_n^m, m < n
    const uint64_t* pow7k;  // 7^i / k
    uint64_t mk[16];        // k (s_e^k − 1)
    uint64_t sstep[16];     // s_e^{K2·RB1}: the scale's step along a thread's elements in pass M1
    int lgk, lgr, lgk1, lgk2, P;
};

// ω_L^{±m} from pw (n = 2^lgn ≥ L = 2^lg).
__device__ __forceinline__ uint64_t rootp(const uint64_t* pw, int lgn, int lg, uint64_t m, bool inverse) {
    const uint64_t n = 1ull << lgn;
    uint64_t e = (m & ((1ull << lg) - 1)) << (lgn - lg);
    if (inverse) e = (n - e) & (n - 1);
    return pw[e];
}

template <int RA, int RB>
struct Shape {
    static constexpr int L = RA * RB;
    static constexpr int E = 32;                  // elements per thread
    static constexpr int T = L / E;               // threads per column
    static constexpr int W = THREADS / T;         // columns per CTA
    static constexpr int TILE_WORDS = W * L;      // 8,192
    static constexpr int MINB = 2;                // CTAs per SM the registers allow
    static constexpr int NA = RA / T;             // round-1 sub-transforms per thread (length RB)
    // Round 2: RB sub-transforms of length RA over T threads, NB each; with RB < T (columns of
    // 2,048) each is split over two threads, thread q taking kb = q mod RB and half h = q / RB.
    static constexpr bool SPLIT = RB < T;
    static constexpr int NB = SPLIT ? 1 : RB / T;
    static constexpr int KA_N = SPLIT ? RA / 2 : RA;  // round-2 outputs a thread holds per sub-transform
    static constexpr int KA_STEP = SPLIT ? 2 : 1;     // they are ka = h + KA_STEP·j, j < KA_N
    static_assert(L >= 32 && L <= 2048 && NA >= 1 && NA * RB == E && NB * KA_N == E, "column length");
    static_assert(!SPLIT || (RA == 64 && RB == 32), "split only for columns of 2,048");
    static_assert(W >= 4, "at least 4 columns per tile");
    // Exchange slots. With W ≥ 16 columns a row of the tile spans every bank and the column is
    // XORed with ta: a warp along a column (fixed c, 32 ta) and a warp across columns both hit
    // 16 distinct 8-byte bank pairs. With W = 8 a row is half the banks: kb-planes are padded by
    // 8 words so that rows of odd ta + kb take the other half, and the column is XORed with ta/2.
    // With W = 4 (split) a row is a quarter: planes are padded by 4 words, so that four
    // consecutive kb (a half-warp of round 2) take four quarters, and the column is XORed with
    // ta/4, so that sixteen consecutive ta of one column (a half-warp of a q-fast round 1) do.
    static constexpr int PAD = W >= 16 ? 0 : W == 8 ? 8 : 4;
    static constexpr int WORDS = RB * (RA * W + PAD);
    __device__ static __forceinline__ int slot(int c, int ta, int kb) {
        if constexpr (W >= 16)
            return (kb * RA + ta) * W + (c ^ (ta & 15));
        else if constexpr (W == 8)
            return kb * (RA * W + PAD) + ta * W + (c ^ ((ta >> 1) & 7));
        else
            return kb * (RA * W + PAD) + ta * W + (c ^ ((ta >> 2) & 3));
    }
    // Round 2's ownership for thread q (c-fast): sub-transform i's kb, and the half h.
    __device__ static __forceinline__ int kb_of(int q, int i) { return SPLIT ? (q & (RB - 1)) : q + T * i; }
    __device__ static __forceinline__ int h_of(int q) { return SPLIT ? q / RB : 0; }
    // The register of output ka = h + KA_STEP·j of sub-transform i (bit-reversed order).
    static constexpr int reg_of(int i, int j) { return SPLIT ? brev_c(j, ilog2(RA / 2)) : i * RA + brev_c(j, ilog2(RA)); }
};

// tw[kb·RA + ta] = ω_L^{±ta·kb}.
template <int RA, int RB>
__device__ __forceinline__ void fill_inner(uint64_t* tw, const uint64_t* pw, int lgn, bool inverse) {
    constexpr int L = RA * RB;
    for (int i = threadIdx.x; i < L; i += blockDim.x) {
        const int kb = i / RA, ta = i % RA;
        tw[i] = rootp(pw, lgn, ilog2(L), (uint64_t)ta * kb, inverse);
    }
}

// A tile whose columns are adjacent words, copied cooperatively into shared memory as rows of W
// words (element t of column c at sm[t·W + c]) with 16-byte loads, then read by each thread in its
// round-1 pattern: fewer live addresses than loading every strided element into registers.
template <int RA, int RB, bool STREAM, int N>
__device__ __forceinline__ void load_staged(uint64_t (&v)[N], uint64_t* sm, const uint64_t* src, size_t es, int c,
                                            int q) {
    using S = Shape<RA, RB>;
    constexpr int VPR = S::W / 2;                    // 16-byte vectors per row
    constexpr int ITERS = S::L * VPR / THREADS;      // vectors per thread
    constexpr int BATCH = ITERS > 16 ? 16 : ITERS;   // in flight at once
    static_assert(S::L * VPR % THREADS == 0 && ITERS % BATCH == 0, "whole vectors per thread");
    static_for<ITERS / BATCH>([&](auto b_) {
        constexpr int b = decltype(b_)::value;
        ulonglong2 x[BATCH];
        static_for<BATCH>([&](auto it_) {
            constexpr int it = decltype(it_)::value;
            const int i = threadIdx.x + (b * BATCH + it) * THREADS;
            const uint64_t* g = src + (size_t)(i / VPR) * es + 2 * (i % VPR);
            x[it] = STREAM ? ld_stream(g) : *reinterpret_cast<const ulonglong2*>(g);
        });
        static_for<BATCH>([&](auto it_) {
            constexpr int it = decltype(it_)::value;
            const int i = threadIdx.x + (b * BATCH + it) * THREADS;
            *reinterpret_cast<ulonglong2*>(sm + (i / VPR) * S::W + 2 * (i % VPR)) = x[it];
        });
    });
    __syncthreads();
    static_for<S::NA>([&](auto i_) {
        constexpr int i = decltype(i_)::value;
        const int ta = q + S::T * i;
        static_for<RB>([&](auto tb_) {
            constexpr int tb = decltype(tb_)::value;
            v[i * RB + tb] = sm[(ta + RA * tb) * S::W + c];
        });
    });
    __syncthreads();  // the buffer becomes the exchange
}

// A tile of W columns whose elements are adjacent (column c at src + c·cs), copied into shared
// memory as sm[c·L + t] with 16-byte loads, then read by each thread in its round-1 pattern.
template <int RA, int RB, int N>
__device__ __forceinline__ void load_staged_q(uint64_t (&v)[N], uint64_t* sm, const uint64_t* src, size_t cs, int c,
                                              int q) {
    using S = Shape<RA, RB>;
    constexpr int VPC = S::L / 2;                    // 16-byte vectors per column
    constexpr int ITERS = S::W * VPC / THREADS;      // vectors per thread
    constexpr int BATCH = ITERS > 16 ? 16 : ITERS;   // in flight at once
    static_assert(S::W * VPC % THREADS == 0 && ITERS % BATCH == 0, "whole vectors per thread");
    static_for<ITERS / BATCH>([&](auto b_) {
        constexpr int b = decltype(b_)::value;
        ulonglong2 x[BATCH];
        static_for<BATCH>([&](auto it_) {
            constexpr int it = decltype(it_)::value;
            const int i = threadIdx.x + (b * BATCH + it) * THREADS;
            x[it] = *reinterpret_cast<const ulonglong2*>(src + (size_t)(i / VPC) * cs + 2 * (i % VPC));
        });
        static_for<BATCH>([&](auto it_) {
            constexpr int it = decltype(it_)::value;
            const int i = threadIdx.x + (b * BATCH + it) * THREADS;
            *reinterpret_cast<ulonglong2*>(sm + (i / VPC) * S::L + 2 * (i % VPC)) = x[it];
        });
    });
    __syncthreads();
    static_for<S::NA>([&](auto i_) {
        constexpr int i = decltype(i_)::value;
        const int ta = q + S::T * i;
        static_for<RB>([&](auto tb_) {
            constexpr int tb = decltype(tb_)::value;
            v[i * RB + tb] = sm[c * S::L + ta + RA * tb];
        });
    });
    __syncthreads();  // the buffer becomes the exchange
}

// Round-1 loads. q-fast: column c starts at src + c·cs and its elements are adjacent.
template <int RA, int RB, int N>
__device__ __forceinline__ void load_qfast(uint64_t (&v)[N], const uint64_t* src, size_t cs, int c, int q) {
    using S = Shape<RA, RB>;
    const uint64_t* col = src + (size_t)c * cs;
    static_for<S::NA>([&](auto i_) {
        constexpr int i = decltype(i_)::value;
        const int ta = q + S::T * i;
        static_for<RB>([&](auto tb_) {
            constexpr int tb = decltype(tb_)::value;
            v[i * RB + tb] = col[ta + RA * tb];
        });
    });
}

// Round 1: DIF of length RB on each loaded sub-transform, inner twiddle, park in shared memory.
template <int RA, int RB, bool INV, int N>
__device__ __forceinline__ void round1_store(uint64_t (&v)[N], uint64_t* sm, const uint64_t* tw, int c, int q) {
    using S = Shape<RA, RB>;
    if constexpr (S::NA == 2) {
        // two sub-transforms: one copy of the code in a rolled loop, the second half swapped in
#pragma unroll 1
        for (int i = 0; i < 2; i++) {
            dft_dif<RB, INV, 0>(v);
            const int ta = q + S::T * i;
            static_for<RB>([&](auto p_) {
                constexpr int p = decltype(p_)::value;
                constexpr int kb = brev_c(p, ilog2(RB));
                const uint64_t val = kb == 0 ? v[p] : lz::mul(v[p], tw[kb * RA + ta]);
                sm[S::slot(c, ta, kb)] = val;
            });
            swap_halves<RB, 0>(v);
        }
    } else {
        static_for<S::NA>([&](auto i_) {
            constexpr int i = decltype(i_)::value;
            dft_dif<RB, INV, i * RB>(v);
            const int ta = q + S::T * i;
            static_for<RB>([&](auto p_) {
                constexpr int p = decltype(p_)::value;
                constexpr int kb = brev_c(p, ilog2(RB));
                const uint64_t val = kb == 0 ? v[i * RB + p] : lz::mul(v[i * RB + p], tw[kb * RA + ta]);
                sm[S::slot(c, ta, kb)] = val;
            });
        });
    }
}

// Round 2 (c-fast): v[i·RA + ta] = Y[ta][kb_i], kb_i = q + T·i, then DIF of length RA:
// v[i·RA + p] holds output kb_i + RB·rev(p). Split: thread (kb, h) keeps the first stage's half h
// of Y[·][kb] and runs DIF of length RA/2 on it: v[p] holds output kb + RB·(2·rev(p) + h).
template <int RA, int RB, bool INV, int N>
__device__ __forceinline__ void round2(uint64_t (&v)[N], const uint64_t* sm, int c, int q) {
    using S = Shape<RA, RB>;
    if constexpr (S::SPLIT) {
        constexpr int H = RA / 2;
        const int kb = S::kb_of(q, 0);
        if (S::h_of(q) == 0) {  // warp-uniform: h = q / RB and a warp spans 8 consecutive q
            static_for<H>([&](auto t_) {
                constexpr int t = decltype(t_)::value;
                v[t] = lz::add(sm[S::slot(c, t, kb)], sm[S::slot(c, t + H, kb)]);
            });
        } else {
            static_for<H>([&](auto t_) {
                constexpr int t = decltype(t_)::value;
                constexpr int E2 = tw_exp(RA, t, INV);
                const uint64_t a = sm[S::slot(c, t, kb)], b = sm[S::slot(c, t + H, kb)];
                if constexpr (E2 >= 96)
                    v[t] = lz::mulp2<E2 - 96>(lz::sub(b, a));
                else
                    v[t] = lz::mulp2<E2>(lz::sub(a, b));
            });
        }
        dft_dif<H, INV, 0>(v);
        return;
    }
    static_for<S::NB>([&](auto i_) {
        constexpr int i = decltype(i_)::value;
        const int kb = q + S::T * i;
        static_for<RA>([&](auto ta_) {
            constexpr int ta = decltype(ta_)::value;
            v[i * RA + ta] = sm[S::slot(c, ta, kb)];
        });
        dft_dif<RA, INV, i * RA>(v);
    });
}

// ---- pass A ------------------------------------------------------------------------------------
template <int RA, int RB>
__global__ void __launch_bounds__(THREADS, Shape<RA, RB>::MINB) pass_a(Args a) {
    using S = Shape<RA, RB>;
    extern __shared__ uint64_t sm[];
    uint64_t* tw = sm + S::WORDS;
    const int lgn = a.lgk + a.lgr;
    fill_inner<RA, RB>(tw, a.pw, lgn, true);
    const size_t row = blockIdx.y;
    const int t1_0 = blockIdx.x * S::W;
    const int K1 = 1 << a.lgk1;
    const int c = threadIdx.x % S::W, q = threadIdx.x / S::W;  // c-fast throughout
    const uint32_t t1 = t1_0 + c;
    const int h = S::h_of(q);
    // the outer twiddles, fetched before the tile so that their latency hides behind it
    const uint64_t step = rootp(a.pw, lgn, a.lgk, (uint64_t)RB * S::KA_STEP * t1, true);
    uint64_t t0[S::NB];
    static_for<S::NB>([&](auto i_) {
        constexpr int i = decltype(i_)::value;
        t0[i] = rootp(a.pw, lgn, a.lgk, (uint64_t)(S::kb_of(q, i) + RB * h) * t1, true);
    });
    uint64_t v[S::E];
    load_staged<RA, RB, true>(v, sm, a.rows + (row << a.lgk) + t1_0, K1, c, q);  // its syncs cover the twiddles
    round1_store<RA, RB, true>(v, sm, tw, c, q);
    __syncthreads();
    round2<RA, RB, true>(v, sm, c, q);
    uint64_t* y = a.y + (row << a.lgk) + t1;
    static_for<S::NB>([&](auto i_) {
        constexpr int i = decltype(i_)::value;
        const int kb = S::kb_of(q, i);
        // output j2 = kb + RB·ka, ka = h + KA_STEP·j, at v[reg_of(i, j)]; × ω_k^{−j2·t1}; Y[j2][t1]
        uint64_t t = t0[i];
        static_for<S::KA_N>([&](auto j_) {
            constexpr int j = decltype(j_)::value;
            const int ka = h + S::KA_STEP * j;
            st_keep(y + (size_t)(kb + RB * ka) * K1, lz::mul(v[S::reg_of(i, j)], t));
            if constexpr (j + 1 < S::KA_N) t = lz::mul(t, step);
        });
    });
}

// ---- pass M1 -----------------------------------------------------------------------------------
template <int RA, int RB>
__global__ void __launch_bounds__(THREADS, Shape<RA, RB>::MINB) pass_m1(Args a) {
    using S = Shape<RA, RB>;
    extern __shared__ uint64_t sm[];
    uint64_t* tw = sm + S::WORDS;
    const int lgn = a.lgk + a.lgr;
    fill_inner<RA, RB>(tw, a.pw, lgn, true);
    const size_t row = blockIdx.y;
    const int j2_0 = blockIdx.x * S::W;
    const int K2 = 1 << a.lgk2;
    const int c = threadIdx.x % S::W, q = threadIdx.x / S::W;  // c-fast (round 2 and the stores)
    const uint32_t j2 = j2_0 + c;
    const int h = S::h_of(q);
    // the scales' starting points, fetched before the tile so that their latency hides behind it:
    // 7^idx0 / k and ω_n^idx0 (coset 1), idx0 = j2 + K2·(kb + RB·h)
    uint64_t p7[S::NB], w1[S::NB];
    static_for<S::NB>([&](auto i_) {
        constexpr int i = decltype(i_)::value;
        const uint32_t idx0 = j2 + (uint32_t)K2 * (S::kb_of(q, i) + RB * h);
        p7[i] = a.pow7k[idx0];
        w1[i] = a.pw[idx0];
    });
    uint64_t v[S::E];
    {
        const int qq = threadIdx.x % S::T, cc = threadIdx.x / S::T;  // q-fast: a column's t1 are adjacent
        load_staged_q<RA, RB>(v, sm, a.y + (row << a.lgk) + ((size_t)j2_0 << a.lgk1), S::L, cc, qq);
        round1_store<RA, RB, true>(v, sm, tw, cc, qq);
    }
    __syncthreads();
    round2<RA, RB, true>(v, sm, c, q);
    // v[reg_of(i, j)] = k·a_idx, idx = j2 + K2·(kb + RB·ka), ka = h + KA_STEP·j;
    // C_e[j1][j2] = that × s_e^idx / k (mask terms are added afterwards by mask_fixup)
    uint64_t* z = a.z + (row << lgn) + j2;
    for (int e = 0; e < (1 << a.lgr); e++) {
        uint64_t* ce = z + ((size_t)e << a.lgk);
        // the scale's step along j: s_e^{K2·RB·KA_STEP}
        const uint64_t step = S::KA_STEP == 2 ? lz::mul(a.sstep[e], a.sstep[e]) : a.sstep[e];
        static_for<S::NB>([&](auto i_) {
            constexpr int i = decltype(i_)::value;
            const int kb = S::kb_of(q, i);
            const uint32_t idx0 = j2 + (uint32_t)K2 * (kb + RB * h);
            uint64_t t = p7[i];  // s_e^idx0 / k
            if (e == 1)
                t = lz::mul(t, w1[i]);
            else if (e > 1)
                t = lz::mul(t, a.pw[((uint64_t)e * idx0) & ((1ull << lgn) - 1)]);
            static_for<S::KA_N>([&](auto j_) {
                constexpr int j = decltype(j_)::value;
                const int ka = h + S::KA_STEP * j;
                st_keep(ce + (size_t)(kb + RB * ka) * K2, lz::mul(v[S::reg_of(i, j)], t));
                if constexpr (j + 1 < S::KA_N) t = lz::mul(t, step);
            });
        });
    }
}

// Adds the mask terms into C_e after pass M1: C_e[idx] += m_idx·k(s_e^k − 1)·s_e^idx/k for idx < P,
// where C_e[idx] sits at C_e[j1][j2], idx = j2 + K2·j1. One thread per (coset, idx).
static __global__ void mask_fixup(Args a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int R = 1 << a.lgr;
    if (i >= a.P * R) return;
    const int e = i % R;
    const uint32_t idx = (uint32_t)(i / R);
    const size_t row = blockIdx.y;
    const int lgn = a.lgk + a.lgr;
    uint64_t scale = a.pow7k[idx];
    if (e) scale = lz::mul(scale, a.pw[((uint64_t)e * idx) & ((1ull << lgn) - 1)]);
    const uint64_t term = lz::mul(lz::mul(a.masks[row * (size_t)a.P + idx], a.mk[e]), scale);
    const uint32_t j2 = idx & ((1u << a.lgk2) - 1), j1 = idx >> a.lgk2;
    uint64_t* ce = a.z + (row << lgn) + ((size_t)e << a.lgk) + ((size_t)j1 << a.lgk2) + j2;
    *ce = lz::add(*ce, term);
}

// ---- pass M2 -----------------------------------------------------------------------------------
template <int RA, int RB>
__global__ void __launch_bounds__(THREADS, Shape<RA, RB>::MINB) pass_m2(Args a) {
    using S = Shape<RA, RB>;
    extern __shared__ uint64_t sm[];
    uint64_t* tw = sm + S::WORDS;
    const int lgn = a.lgk + a.lgr;
    fill_inner<RA, RB>(tw, a.pw, lgn, false);
    const size_t row = blockIdx.y;
    const int tiles = (1 << a.lgk2) / S::W;
    const int e = blockIdx.x / tiles;
    const int j2_0 = (blockIdx.x % tiles) * S::W;
    const int K2 = 1 << a.lgk2;
    const int c = threadIdx.x % S::W, q = threadIdx.x / S::W;  // c-fast throughout
    uint64_t* z = a.z + (row << lgn) + ((size_t)e << a.lgk) + j2_0;
    const uint32_t j2 = j2_0 + c;
    const int h = S::h_of(q);
    // the outer twiddles, fetched before the tile so that their latency hides behind it
    const uint64_t step = rootp(a.pw, lgn, a.lgk, (uint64_t)RB * S::KA_STEP * j2, false);
    uint64_t t0[S::NB];
    static_for<S::NB>([&](auto i_) {
        constexpr int i = decltype(i_)::value;
        t0[i] = rootp(a.pw, lgn, a.lgk, (uint64_t)(S::kb_of(q, i) + RB * h) * j2, false);
    });
    uint64_t v[S::E];
    load_staged<RA, RB, false>(v, sm, z, K2, c, q);  // every load of this tile is done before any store below
    round1_store<RA, RB, false>(v, sm, tw, c, q);
    __syncthreads();
    round2<RA, RB, false>(v, sm, c, q);
    static_for<S::NB>([&](auto i_) {
        constexpr int i = decltype(i_)::value;
        const int kb = S::kb_of(q, i);
        // output v2 = kb + RB·ka, ka = h + KA_STEP·j; × ω_k^{v2·j2}; Z_e[v2][j2]
        uint64_t t = t0[i];
        static_for<S::KA_N>([&](auto j_) {
            constexpr int j = decltype(j_)::value;
            const int ka = h + S::KA_STEP * j;
            st_keep(z + c + (size_t)(kb + RB * ka) * K2, lz::mul(v[S::reg_of(i, j)], t));
            if constexpr (j + 1 < S::KA_N) t = lz::mul(t, step);
        });
    });
}

// ---- pass C ------------------------------------------------------------------------------------
template <int RA, int RB>
__global__ void __launch_bounds__(THREADS, Shape<RA, RB>::MINB) pass_c(Args a) {
    using S = Shape<RA, RB>;
    extern __shared__ uint64_t sm[];
    uint64_t* tw = sm + S::WORDS;
    const int lgn = a.lgk + a.lgr;
    fill_inner<RA, RB>(tw, a.pw, lgn, false);
    const size_t row = blockIdx.y;
    const int R = 1 << a.lgr;
    const int col0 = blockIdx.x * S::W;  // columns are (v2, e) pairs, e fastest
    const int K1 = 1 << a.lgk1;
    const uint64_t* z = a.z + (row << lgn);
    uint64_t v[S::E];
    {
        const int q = threadIdx.x % S::T, c = threadIdx.x / S::T;  // q-fast
        const int colid = col0 + c;
        const int e = colid & (R - 1), v2 = colid >> a.lgr;
        load_qfast<RA, RB>(v, z + ((size_t)e << a.lgk) + (size_t)v2 * S::L, 0, 0, q);
        __syncthreads();  // the twiddle table
        round1_store<RA, RB, false>(v, sm, tw, c, q);
    }
    __syncthreads();
    const int c = threadIdx.x % S::W, q = threadIdx.x / S::W;  // c-fast
    round2<RA, RB, false>(v, sm, c, q);
    uint64_t* out = a.out + (row << lgn) + col0 + c;
    const int h = S::h_of(q);
    static_for<S::NB>([&](auto i_) {
        constexpr int i = decltype(i_)::value;
        const int kb = S::kb_of(q, i);
        static_for<S::KA_N>([&](auto j_) {
            constexpr int j = decltype(j_)::value;
            // symbol (v2 + K1·v1)·2^r + e with v1 = kb + RB·ka, ka = h + KA_STEP·j
            const int ka = h + S::KA_STEP * j;
            st_stream(out + (((size_t)(kb + RB * ka) * K1) << a.lgr), lz::canon(v[S::reg_of(i, j)]));
        });
    });
}

}  // namespace fast
}  // namespace tg
