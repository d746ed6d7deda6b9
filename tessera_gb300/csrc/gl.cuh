// SPDX-License-Identifier: Apache-2.0 OR MIT
//
// Goldilocks arithmetic on the device: p = 2^64 - 2^32 + 1, canonical representatives in
// [0, p). The reduction uses 2^64 = 2^32 - 1 and 2^96 = -1 (mod p), the identities the reference
// states at crates/tessera-field/src/goldilocks.rs:57-77. Fp2 = Fp[X]/(X^2 - 7), multiplied by
// Karatsuba as at crates/tessera-field/src/ext2.rs:235-249. Results are exact field values, so any
// correct reduction gives the reference's bits.
#pragma once
#include <stdint.h>

namespace tg {

constexpr uint64_t P = 0xFFFFFFFF00000001ull;
constexpr uint64_t EPS = 0xFFFFFFFFull;  // 2^64 mod p

struct fp2 {
    uint64_t c0, c1;
};

__host__ __device__ __forceinline__ uint64_t canon(uint64_t x) { return x >= P ? x - P : x; }

__host__ __device__ __forceinline__ uint64_t add(uint64_t a, uint64_t b) {
    uint64_t s = a + b;
    s += (s < a) ? EPS : 0;  // a carry out adds 2^64 = EPS (mod p); cannot carry twice
    return canon(s);
}

__host__ __device__ __forceinline__ uint64_t sub(uint64_t a, uint64_t b) {
    uint64_t d = a - b;
    return d - ((a < b) ? EPS : 0);  // a borrow added 2^64; take EPS back off
}

__host__ __device__ __forceinline__ uint64_t neg(uint64_t a) { return sub(0, a); }

// lo + 2^64 hi (mod p): lo - hi_hi + hi_lo (2^32 - 1).
__host__ __device__ __forceinline__ uint64_t reduce128(uint64_t lo, uint64_t hi) {
    uint64_t hh = hi >> 32;
    uint64_t hl = hi & EPS;
    uint64_t t0 = lo - hh;
    t0 -= (lo < hh) ? EPS : 0;
    uint64_t t1 = (hl << 32) - hl;  // hl (2^32 - 1) without a multiply
    uint64_t t2 = t0 + t1;
    t2 += (t2 < t1) ? EPS : 0;
    return canon(t2);
}

#ifdef __CUDA_ARCH__
__device__ __forceinline__ uint64_t mul(uint64_t a, uint64_t b) {
    return reduce128(a * b, __umul64hi(a, b));
}
#else
__host__ inline uint64_t mul(uint64_t a, uint64_t b) {
    unsigned __int128 x = (unsigned __int128)a * b;
    return reduce128((uint64_t)x, (uint64_t)(x >> 64));
}
#endif

// x * 2^s for 0 <= s < 64: the 128-bit shift, then one reduction.
__host__ __device__ __forceinline__ uint64_t mul_pow2_lt64(uint64_t x, uint32_t s) {
    if (s == 0) return x;
    return reduce128(x << s, x >> (64 - s));
}

// x * 2^s for 0 <= s < 192 (2^96 = -1, so 2^192 = 1).
__host__ __device__ __forceinline__ uint64_t mul_pow2(uint64_t x, uint32_t s) {
    bool negate = s >= 96;
    if (negate) s -= 96;
    uint64_t y = s >= 64 ? mul_pow2_lt64(mul_pow2_lt64(x, 32), s - 32) : mul_pow2_lt64(x, s);
    return negate ? neg(y) : y;
}

__host__ __device__ __forceinline__ uint64_t mul7(uint64_t x) { return sub(mul_pow2_lt64(x, 3), x); }

__host__ __device__ inline uint64_t pow(uint64_t a, uint64_t e) {
    uint64_t acc = 1;
    while (e) {
        if (e & 1) acc = mul(acc, a);
        a = mul(a, a);
        e >>= 1;
    }
    return acc;
}

__host__ __device__ inline uint64_t inv(uint64_t a) { return pow(a, P - 2); }

// ---- Fp2 ------------------------------------------------------------------------------------

__host__ __device__ __forceinline__ fp2 e_add(fp2 a, fp2 b) { return {add(a.c0, b.c0), add(a.c1, b.c1)}; }
__host__ __device__ __forceinline__ fp2 e_sub(fp2 a, fp2 b) { return {sub(a.c0, b.c0), sub(a.c1, b.c1)}; }
__host__ __device__ __forceinline__ fp2 e_mul(fp2 a, fp2 b) {
    uint64_t v0 = mul(a.c0, b.c0), v1 = mul(a.c1, b.c1);
    uint64_t cross = mul(add(a.c0, a.c1), add(b.c0, b.c1));
    return {add(v0, mul7(v1)), sub(sub(cross, v0), v1)};
}
__host__ __device__ __forceinline__ fp2 e_scale(fp2 a, uint64_t s) { return {mul(a.c0, s), mul(a.c1, s)}; }
__host__ __device__ __forceinline__ fp2 e_lift(uint64_t x) { return {x, 0}; }
// base * ext: two base products
__host__ __device__ __forceinline__ fp2 e_mul_base(fp2 a, uint64_t b) { return {mul(a.c0, b), mul(a.c1, b)}; }

// x * small integer k (k < 2^32), used for the integer nodes 2..7 of a round polynomial.
__host__ __device__ __forceinline__ uint64_t mul_small(uint64_t x, uint32_t k) {
#ifdef __CUDA_ARCH__
    uint64_t lo = x * (uint64_t)k;
    uint64_t hi = __umul64hi(x, (uint64_t)k);
#else
    unsigned __int128 p = (unsigned __int128)x * k;
    uint64_t lo = (uint64_t)p, hi = (uint64_t)(p >> 64);
#endif
    uint64_t t = (hi << 32) - hi;  // hi < 2^32: hi (2^32 - 1) < 2^64
    uint64_t s = lo + t;
    s += (s < t) ? EPS : 0;
    return canon(s);
}

}  // namespace tg

// ---- lazy arithmetic for the transforms --------------------------------------------------------
//
// Values are any 64-bit word x, standing for x mod p (so both x and x − p may appear); sums and
// products fold every carry out of bit 64 back in as 2^64 = 2^32 − 1 with the carry flag, and a
// value is made canonical once, when it leaves a transform. Every function here is exact for all
// 64-bit inputs.
namespace tg {
namespace lz {

// Every multi-instruction asm block below copies its inputs into registers of its own before it
// writes an output: the compiler may give an output (or a read-write operand) the register of an
// input that holds the same value, and a later read of that input would see the output instead.

__device__ __forceinline__ uint32_t lo32(uint64_t x) { return (uint32_t)x; }
__device__ __forceinline__ uint32_t hi32(uint64_t x) { return (uint32_t)(x >> 32); }
__device__ __forceinline__ uint64_t mk64(uint32_t lo, uint32_t hi) { return ((uint64_t)hi << 32) | lo; }
// c·(2^64 mod p) for a carry c ∈ {0, 1}, as a 64-bit word.
__device__ __forceinline__ uint64_t eps_if(uint32_t c) { return (uint64_t)(uint32_t)(-(int32_t)c); }

__device__ __forceinline__ uint64_t add(uint64_t a, uint64_t b) {
    uint64_t s;
    uint32_t c, c2;
    asm("add.cc.u64 %0, %2, %3;\n\taddc.u32 %1, 0, 0;" : "=l"(s), "=r"(c) : "l"(a), "l"(b));
    // a second carry needs a + b ≥ 2^64 + p, possible only for inputs at or above p
    asm("add.cc.u64 %0, %2, %3;\n\taddc.u32 %1, 0, 0;" : "=l"(s), "=r"(c2) : "l"(s), "l"(eps_if(c)));
    return s + eps_if(c2);
}

__device__ __forceinline__ uint64_t sub(uint64_t a, uint64_t b) {
    uint64_t d;
    uint32_t br, br2;  // 0xFFFFFFFF on a borrow, which is 2^64 mod p as a word
    asm("sub.cc.u64 %0, %2, %3;\n\tsubc.u32 %1, 0, 0;" : "=l"(d), "=r"(br) : "l"(a), "l"(b));
    asm("sub.cc.u64 %0, %2, %3;\n\tsubc.u32 %1, 0, 0;" : "=l"(d), "=r"(br2) : "l"(d), "l"((uint64_t)br));
    return d - (uint64_t)br2;
}

// (lo + hl·2^64 + hh·2^96) mod p for hl, hh < 2^32: lo + hl·(2^32 − 1) − hh, the product on the
// multiply pipe with its carry.
__device__ __forceinline__ uint64_t fold(uint64_t lo, uint32_t hl, uint32_t hh) {
    uint32_t r0, r1, c;
    asm("{\n\t.reg .u32 h, l0, l1;\n\tmov.u32 h, %3;\n\tmov.u32 l0, %4;\n\tmov.u32 l1, %5;\n\t"
        "mad.lo.cc.u32 %0, h, 0xFFFFFFFF, l0;\n\t"
        "madc.hi.cc.u32 %1, h, 0xFFFFFFFF, l1;\n\t"
        "addc.u32 %2, 0, 0;\n\t}"
        : "=r"(r0), "=r"(r1), "=r"(c)
        : "r"(hl), "r"(lo32(lo)), "r"(hi32(lo)));
    uint64_t d;
    uint32_t br;
    asm("sub.cc.u64 %0, %2, %3;\n\tsubc.u32 %1, 0, 0;" : "=l"(d), "=r"(br) : "l"(mk64(r0, r1)), "l"((uint64_t)hh));
    // carry and borrow: +2^64 and −2^64 cancel; one alone adds or removes 2^32 − 1 without wrapping
    return d + eps_if(c) - (uint64_t)br;
}

// (lo + h·2^64) mod p for h < 2^32: lo + h·(2^32 − 1).
__device__ __forceinline__ uint64_t fold_lo(uint64_t lo, uint32_t h) {
    uint32_t r0, r1, c;
    asm("{\n\t.reg .u32 h, l0, l1;\n\tmov.u32 h, %3;\n\tmov.u32 l0, %4;\n\tmov.u32 l1, %5;\n\t"
        "mad.lo.cc.u32 %0, h, 0xFFFFFFFF, l0;\n\t"
        "madc.hi.cc.u32 %1, h, 0xFFFFFFFF, l1;\n\t"
        "addc.u32 %2, 0, 0;\n\t}"
        : "=r"(r0), "=r"(r1), "=r"(c)
        : "r"(h), "r"(lo32(lo)), "r"(hi32(lo)));
    // with a carry, the word is below h·(2^32 − 1) < 2^64 − 2^33: adding 2^32 − 1 cannot wrap
    return mk64(r0, r1) + eps_if(c);
}

// x·2^E for 0 ≤ E < 96.
template <int E>
__device__ __forceinline__ uint64_t mulp2(uint64_t x) {
    static_assert(E >= 0 && E < 96, "shift exponent");
    if constexpr (E == 0) {
        return x;
    } else if constexpr (E <= 32) {
        return fold_lo(x << E, (uint32_t)(x >> (64 - E)));
    } else if constexpr (E < 64) {
        const uint64_t hi = x >> (64 - E);
        return fold(x << E, lo32(hi), hi32(hi));
    } else {
        // x·2^64 ≡ x0·2^32 − (x0 + x1), x = x0 + 2^32·x1; then ·2^(E−64)
        const uint32_t x0 = lo32(x), x1 = hi32(x);
        uint64_t y;
        uint32_t br;
        asm("sub.cc.u64 %0, %2, %3;\n\tsubc.u32 %1, 0, 0;"
            : "=l"(y), "=r"(br)
            : "l"((uint64_t)x0 << 32), "l"((uint64_t)x0 + x1));
        return mulp2<E - 64>(y - (uint64_t)br);
    }
}

// a·b: the 128-bit product in 32-bit multiply-add carry chains, then fold.
__device__ __forceinline__ uint64_t mul(uint64_t a, uint64_t b) {
    uint32_t r0, r1, r2, r3;
    asm("{\n\t"
        ".reg .u32 x0, x1, y0, y1;\n\t"
        "mov.u32 x0, %4;\n\tmov.u32 x1, %5;\n\tmov.u32 y0, %6;\n\tmov.u32 y1, %7;\n\t"
        "mul.lo.u32 %0, x0, y0;\n\t"
        "mul.hi.u32 %1, x0, y0;\n\t"
        "mad.lo.cc.u32 %1, x0, y1, %1;\n\t"
        "madc.hi.u32 %2, x0, y1, 0;\n\t"
        "mad.lo.cc.u32 %1, x1, y0, %1;\n\t"
        "madc.hi.cc.u32 %2, x1, y0, %2;\n\t"
        "madc.hi.u32 %3, x1, y1, 0;\n\t"
        "mad.lo.cc.u32 %2, x1, y1, %2;\n\t"
        "addc.u32 %3, %3, 0;\n\t"
        "}"
        : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
        : "r"(lo32(a)), "r"(hi32(a)), "r"(lo32(b)), "r"(hi32(b)));
    return fold(mk64(r0, r1), r2, r3);
}

// The canonical representative.
__device__ __forceinline__ uint64_t canon(uint64_t x) { return x >= P ? x - P : x; }

// lo + h·(2^32 − 1) for h < 2^32 with shifts and adds (no multiply). fold_lo keeps the transforms'
// butterflies off the busier ALU pipe; the unreduced product sums below fill the multiply pipe
// instead, so their folds and 7·x take the ALU (3 % faster tree rounds than on the multiply pipe).
__device__ __forceinline__ uint64_t fold_lo_sh(uint64_t lo, uint32_t h) {
    uint64_t t;
    uint32_t c;
    asm("add.cc.u64 %0, %2, %3;\n\taddc.u32 %1, 0, 0;" : "=l"(t), "=r"(c) : "l"(lo), "l"(((uint64_t)h << 32) - h));
    return t + eps_if(c);
}

// 7·x = 8x − x: the low word (x << 3) − x, its borrow taken from the top bits x >> 61.
__device__ __forceinline__ uint64_t mul7(uint64_t x) {
    uint64_t lo;
    uint32_t br;
    asm("sub.cc.u64 %0, %2, %3;\n\tsubc.u32 %1, 0, 0;" : "=l"(lo), "=r"(br) : "l"(x << 3), "l"(x));
    return fold_lo_sh(lo, (uint32_t)(x >> 61) + br);
}

// An unreduced sum of 64 × 64-bit products (and words) in five 32-bit limbs: exact for fewer than
// 2^32 terms, and folded to one word once, where the sum is used.
struct Acc {
    uint32_t w[5];
};

__device__ __forceinline__ Acc acc_zero() { return {{0, 0, 0, 0, 0}}; }
__device__ __forceinline__ Acc acc_of(uint64_t x) { return {{lo32(x), hi32(x), 0, 0, 0}}; }

// x·y as a sum
__device__ __forceinline__ Acc acc_mul(uint64_t x, uint64_t y) {
    Acc a;
    asm("{\n\t"
        ".reg .u32 x0, x1, y0, y1;\n\t"
        "mov.u32 x0, %4;\n\tmov.u32 x1, %5;\n\tmov.u32 y0, %6;\n\tmov.u32 y1, %7;\n\t"
        "mul.lo.u32 %0, x0, y0;\n\t"
        "mul.hi.u32 %1, x0, y0;\n\t"
        "mad.lo.cc.u32 %1, x0, y1, %1;\n\t"
        "madc.hi.u32 %2, x0, y1, 0;\n\t"
        "mad.lo.cc.u32 %1, x1, y0, %1;\n\t"
        "madc.hi.cc.u32 %2, x1, y0, %2;\n\t"
        "madc.hi.u32 %3, x1, y1, 0;\n\t"
        "mad.lo.cc.u32 %2, x1, y1, %2;\n\t"
        "addc.u32 %3, %3, 0;\n\t"
        "}"
        : "=r"(a.w[0]), "=r"(a.w[1]), "=r"(a.w[2]), "=r"(a.w[3])
        : "r"(lo32(x)), "r"(hi32(x)), "r"(lo32(y)), "r"(hi32(y)));
    a.w[4] = 0;
    return a;
}

// a += x·y: x0·y0 into limbs 0–1, x1·y1 into 2–3, the cross products into 1–2, each carry to limb 4.
__device__ __forceinline__ void mad(Acc& a, uint64_t x, uint64_t y) {
    asm("{\n\t"
        ".reg .u32 x0, x1, y0, y1;\n\t"
        "mov.u32 x0, %5;\n\tmov.u32 x1, %6;\n\tmov.u32 y0, %7;\n\tmov.u32 y1, %8;\n\t"
        "mad.lo.cc.u32 %0, x0, y0, %0;\n\t"
        "madc.hi.cc.u32 %1, x0, y0, %1;\n\t"
        "madc.lo.cc.u32 %2, x1, y1, %2;\n\t"
        "madc.hi.cc.u32 %3, x1, y1, %3;\n\t"
        "addc.u32 %4, %4, 0;\n\t"
        "mad.lo.cc.u32 %1, x0, y1, %1;\n\t"
        "madc.hi.cc.u32 %2, x0, y1, %2;\n\t"
        "addc.cc.u32 %3, %3, 0;\n\t"
        "addc.u32 %4, %4, 0;\n\t"
        "mad.lo.cc.u32 %1, x1, y0, %1;\n\t"
        "madc.hi.cc.u32 %2, x1, y0, %2;\n\t"
        "addc.cc.u32 %3, %3, 0;\n\t"
        "addc.u32 %4, %4, 0;\n\t"
        "}"
        : "+r"(a.w[0]), "+r"(a.w[1]), "+r"(a.w[2]), "+r"(a.w[3]), "+r"(a.w[4])
        : "r"(lo32(x)), "r"(hi32(x)), "r"(lo32(y)), "r"(hi32(y)));
}

// The sum mod p as one word: limbs 0–1 + w2·2^64 + (w3 + w4·2^32)·2^96, with 2^64 ≡ 2^32 − 1 and
// 2^96 ≡ −1.
__device__ __forceinline__ uint64_t reduce(const Acc& a) {
    return sub(fold_lo_sh(mk64(a.w[0], a.w[1]), a.w[2]), mk64(a.w[3], a.w[4]));
}

}  // namespace lz

// Fp2 on lazy words (any 64-bit representative; canonical only where results leave a kernel).
__device__ __forceinline__ fp2 l2_add(fp2 a, fp2 b) { return {lz::add(a.c0, b.c0), lz::add(a.c1, b.c1)}; }
__device__ __forceinline__ fp2 l2_sub(fp2 a, fp2 b) { return {lz::sub(a.c0, b.c0), lz::sub(a.c1, b.c1)}; }
__device__ __forceinline__ fp2 l2_mul(fp2 a, fp2 b) {  // Karatsuba, X^2 = 7
    const uint64_t t0 = lz::mul(a.c0, b.c0), t1 = lz::mul(a.c1, b.c1);
    const uint64_t t2 = lz::mul(lz::add(a.c0, a.c1), lz::add(b.c0, b.c1));
    return {lz::add(t0, lz::sub(lz::mulp2<3>(t1), t1)), lz::sub(lz::sub(t2, t0), t1)};
}
__device__ __forceinline__ fp2 l2_scale(fp2 a, uint64_t b) { return {lz::mul(a.c0, b), lz::mul(a.c1, b)}; }
__device__ __forceinline__ fp2 l2_canon(fp2 a) { return {lz::canon(a.c0), lz::canon(a.c1)}; }

// Fp2 products as unreduced sums, one fold a component: a·b = (a0·b0 + a1·7b1, a0·b1 + a1·b0), the
// 7·b1 passed in where b is a constant of many products (k7 = mul7(k.c1)).
__device__ __forceinline__ fp2 l2_mulk(fp2 a, fp2 k, uint64_t k7) {
    lz::Acc s0 = lz::acc_mul(a.c0, k.c0), s1 = lz::acc_mul(a.c0, k.c1);
    lz::mad(s0, a.c1, k7);
    lz::mad(s1, a.c1, k.c0);
    return {lz::reduce(s0), lz::reduce(s1)};
}
__device__ __forceinline__ fp2 l2_muls(fp2 a, fp2 b) { return l2_mulk(a, b, lz::mul7(b.c1)); }
// a + k·d
__device__ __forceinline__ fp2 l2_fma(fp2 a, fp2 k, uint64_t k7, fp2 d) {
    lz::Acc s0 = lz::acc_of(a.c0), s1 = lz::acc_of(a.c1);
    lz::mad(s0, d.c0, k.c0);
    lz::mad(s0, d.c1, k7);
    lz::mad(s1, d.c0, k.c1);
    lz::mad(s1, d.c1, k.c0);
    return {lz::reduce(s0), lz::reduce(s1)};
}
// a·b + c·d
__device__ __forceinline__ fp2 l2_dot(fp2 a, fp2 b, fp2 c, fp2 d) {
    lz::Acc s0 = lz::acc_mul(a.c0, b.c0), s1 = lz::acc_mul(a.c0, b.c1);
    lz::mad(s0, a.c1, lz::mul7(b.c1));
    lz::mad(s0, c.c0, d.c0);
    lz::mad(s0, c.c1, lz::mul7(d.c1));
    lz::mad(s1, a.c1, b.c0);
    lz::mad(s1, c.c0, d.c1);
    lz::mad(s1, c.c1, d.c0);
    return {lz::reduce(s0), lz::reduce(s1)};
}
// An unreduced Fp2 sum of products: s += k·g (k7 = 7·k.c1), s += k·x for a prime-field x.
struct Acc2 {
    lz::Acc c0, c1;
};
__device__ __forceinline__ Acc2 acc2_zero() { return {lz::acc_zero(), lz::acc_zero()}; }
__device__ __forceinline__ void l2_mad(Acc2& s, fp2 k, uint64_t k7, fp2 g) {
    lz::mad(s.c0, g.c0, k.c0);
    lz::mad(s.c0, g.c1, k7);
    lz::mad(s.c1, g.c0, k.c1);
    lz::mad(s.c1, g.c1, k.c0);
}
__device__ __forceinline__ void l2_mad_base(Acc2& s, fp2 k, uint64_t x) {
    lz::mad(s.c0, x, k.c0);
    lz::mad(s.c1, x, k.c1);
}
__device__ __forceinline__ fp2 l2_reduce(const Acc2& s) { return {lz::reduce(s.c0), lz::reduce(s.c1)}; }
}  // namespace tg
