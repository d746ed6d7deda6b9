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
