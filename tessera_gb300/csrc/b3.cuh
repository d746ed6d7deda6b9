// SPDX-License-Identifier: Apache-2.0 OR MIT
//
// BLAKE3 compression, written from the published BLAKE3 specification, for host and device.
// Every hot-path input is at most one 1024-byte chunk (column-init 40 B, column-step 32 + 8 B
// per row with at most 124 rows, merkle-node 64 B), hashed in derive-key-material mode under a
// domain's 32-byte context key, the way the reference's tessera-hash calls the blake3 crate
// (crates/tessera-hash/src/domain.rs:129-181). The host side also carries the multi-chunk tree
// for the transcript's longer inputs.
#pragma once
#include <stdint.h>
#include <string.h>

namespace tg {
namespace b3 {

enum : uint32_t {
    CHUNK_START = 1,
    CHUNK_END = 2,
    PARENT = 4,
    ROOT = 8,
    KEYED_HASH = 16,
    DERIVE_KEY_CONTEXT = 32,
    DERIVE_KEY_MATERIAL = 64,
};

#define TG_B3_IV0 0x6A09E667u
#define TG_B3_IV1 0xBB67AE85u
#define TG_B3_IV2 0x3C6EF372u
#define TG_B3_IV3 0xA54FF53Au
#define TG_B3_IV4 0x510E527Fu
#define TG_B3_IV5 0x9B05688Cu
#define TG_B3_IV6 0x1F83D9ABu
#define TG_B3_IV7 0x5BE0CD19u

__host__ __device__ __forceinline__ uint32_t rotr(uint32_t x, int n) {
#ifdef __CUDA_ARCH__
    return __funnelshift_r(x, x, n);
#else
    return (x >> n) | (x << (32 - n));
#endif
}

#ifdef __CUDACC__
// The compression is bound by the integer ALU pipe (the XORs and the funnel-shift rotations), so
// on the device its additions go to the otherwise idle multiply-add pipe as x·1 + y with the 1
// read from constant memory, where the compiler cannot fold it away.
static __constant__ uint32_t k_b3_one = 1;
#endif
#ifdef __CUDA_ARCH__
__device__ __forceinline__ uint32_t madd(uint32_t x, uint32_t y) {
    uint32_t r;
    asm("mad.lo.u32 %0, %1, %2, %3;" : "=r"(r) : "r"(x), "r"(k_b3_one), "r"(y));
    return r;
}
#define TG_B3_ADD3(a, b, x) madd(madd(b, x), a)
#define TG_B3_ADD2(a, b) madd(b, a)
#else
#define TG_B3_ADD3(a, b, x) ((a) + (b) + (x))
#define TG_B3_ADD2(a, b) ((a) + (b))
#endif

#define TG_B3_G(a, b, c, d, x, y)  \
    a = TG_B3_ADD3(a, b, (x));     \
    d = rotr(d ^ a, 16);           \
    c = TG_B3_ADD2(c, d);          \
    b = rotr(b ^ c, 12);           \
    a = TG_B3_ADD3(a, b, (y));     \
    d = rotr(d ^ a, 8);            \
    c = TG_B3_ADD2(c, d);          \
    b = rotr(b ^ c, 7);

// One round on the state words s0..s15 with the message words in their permuted order for the
// round; the permutation (2,6,3,10,7,0,4,13,1,11,12,5,9,14,15,8) is applied by the caller's
// index schedule below, so the message never moves in registers.
#define TG_B3_ROUND(m0, m1, m2, m3, m4, m5, m6, m7, m8, m9, m10, m11, m12, m13, m14, m15) \
    TG_B3_G(s0, s4, s8, s12, m0, m1)                                                     \
    TG_B3_G(s1, s5, s9, s13, m2, m3)                                                     \
    TG_B3_G(s2, s6, s10, s14, m4, m5)                                                    \
    TG_B3_G(s3, s7, s11, s15, m6, m7)                                                    \
    TG_B3_G(s0, s5, s10, s15, m8, m9)                                                    \
    TG_B3_G(s1, s6, s11, s12, m10, m11)                                                  \
    TG_B3_G(s2, s7, s8, s13, m12, m13)                                                   \
    TG_B3_G(s3, s4, s9, s14, m14, m15)

// The compression's chaining value: the first 8 output words, cv' = s[0..8] ^ s[8..16].
// m: 16 message words (little-endian), cv: 8 words, updated in place.
__host__ __device__ __forceinline__ void compress_cv(uint32_t cv[8], const uint32_t m[16], uint64_t counter,
                                                     uint32_t block_len, uint32_t flags) {
    uint32_t s0 = cv[0], s1 = cv[1], s2 = cv[2], s3 = cv[3], s4 = cv[4], s5 = cv[5], s6 = cv[6], s7 = cv[7];
    uint32_t s8 = TG_B3_IV0, s9 = TG_B3_IV1, s10 = TG_B3_IV2, s11 = TG_B3_IV3;
    uint32_t s12 = (uint32_t)counter, s13 = (uint32_t)(counter >> 32), s14 = block_len, s15 = flags;
    // Round r reads m[σ^r(i)], σ the message permutation; the schedule is written out.
    TG_B3_ROUND(m[0], m[1], m[2], m[3], m[4], m[5], m[6], m[7], m[8], m[9], m[10], m[11], m[12], m[13], m[14], m[15])
    TG_B3_ROUND(m[2], m[6], m[3], m[10], m[7], m[0], m[4], m[13], m[1], m[11], m[12], m[5], m[9], m[14], m[15], m[8])
    TG_B3_ROUND(m[3], m[4], m[10], m[12], m[13], m[2], m[7], m[14], m[6], m[5], m[9], m[0], m[11], m[15], m[8], m[1])
    TG_B3_ROUND(m[10], m[7], m[12], m[9], m[14], m[3], m[13], m[15], m[4], m[0], m[11], m[2], m[5], m[8], m[1], m[6])
    TG_B3_ROUND(m[12], m[13], m[9], m[11], m[15], m[10], m[14], m[8], m[7], m[2], m[5], m[3], m[0], m[1], m[6], m[4])
    TG_B3_ROUND(m[9], m[14], m[11], m[5], m[8], m[12], m[15], m[1], m[13], m[3], m[0], m[10], m[2], m[6], m[4], m[7])
    TG_B3_ROUND(m[11], m[15], m[5], m[0], m[1], m[9], m[8], m[6], m[14], m[10], m[2], m[12], m[3], m[4], m[7], m[13])
    cv[0] = s0 ^ s8;
    cv[1] = s1 ^ s9;
    cv[2] = s2 ^ s10;
    cv[3] = s3 ^ s11;
    cv[4] = s4 ^ s12;
    cv[5] = s5 ^ s13;
    cv[6] = s6 ^ s14;
    cv[7] = s7 ^ s15;
}

// All 16 output words (for extended output on the host).
__host__ __device__ inline void compress_full(const uint32_t cv_in[8], const uint32_t m[16], uint64_t counter,
                                              uint32_t block_len, uint32_t flags, uint32_t out[16]) {
    uint32_t s0 = cv_in[0], s1 = cv_in[1], s2 = cv_in[2], s3 = cv_in[3], s4 = cv_in[4], s5 = cv_in[5],
             s6 = cv_in[6], s7 = cv_in[7];
    uint32_t s8 = TG_B3_IV0, s9 = TG_B3_IV1, s10 = TG_B3_IV2, s11 = TG_B3_IV3;
    uint32_t s12 = (uint32_t)counter, s13 = (uint32_t)(counter >> 32), s14 = block_len, s15 = flags;
    TG_B3_ROUND(m[0], m[1], m[2], m[3], m[4], m[5], m[6], m[7], m[8], m[9], m[10], m[11], m[12], m[13], m[14], m[15])
    TG_B3_ROUND(m[2], m[6], m[3], m[10], m[7], m[0], m[4], m[13], m[1], m[11], m[12], m[5], m[9], m[14], m[15], m[8])
    TG_B3_ROUND(m[3], m[4], m[10], m[12], m[13], m[2], m[7], m[14], m[6], m[5], m[9], m[0], m[11], m[15], m[8], m[1])
    TG_B3_ROUND(m[10], m[7], m[12], m[9], m[14], m[3], m[13], m[15], m[4], m[0], m[11], m[2], m[5], m[8], m[1], m[6])
    TG_B3_ROUND(m[12], m[13], m[9], m[11], m[15], m[10], m[14], m[8], m[7], m[2], m[5], m[3], m[0], m[1], m[6], m[4])
    TG_B3_ROUND(m[9], m[14], m[11], m[5], m[8], m[12], m[15], m[1], m[13], m[3], m[0], m[10], m[2], m[6], m[4], m[7])
    TG_B3_ROUND(m[11], m[15], m[5], m[0], m[1], m[9], m[8], m[6], m[14], m[10], m[2], m[12], m[3], m[4], m[7], m[13])
    uint32_t s[16] = {s0, s1, s2, s3, s4, s5, s6, s7, s8, s9, s10, s11, s12, s13, s14, s15};
    for (int i = 0; i < 8; i++) {
        out[i] = s[i] ^ s[i + 8];
        out[i + 8] = s[i + 8] ^ cv_in[i];
    }
}

__host__ __device__ __forceinline__ uint32_t le32(const uint8_t *p) {
    return (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
}

}  // namespace b3
}  // namespace tg
