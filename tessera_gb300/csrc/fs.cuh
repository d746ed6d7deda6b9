// SPDX-License-Identifier: Apache-2.0 OR MIT
//
// The Fiat–Shamir transcript on the device (crates/tessera-hash/src/transcript.rs:168-219), for the
// kernels that run a sumcheck's rounds without returning to the host: absorb (state ‖ u64 label
// length ‖ label ‖ value), squeeze (… ‖ u64 counter) and ratchet, BLAKE3 in derive-key-material
// mode under the domains' context keys (derived on the host).
#pragma once
#include <stdint.h>

#include "b3.cuh"
#include "gl.cuh"

namespace tg {

constexpr int FS_MAX_TRIES = 64;  // squeezes per challenge before giving up (each retries with p < 2^-31)

// A job's transcript while it lives on the device.
struct FsState {
    uint8_t state[32];
    uint64_t counter;
    uint64_t r[2];  // the latest challenge
    uint32_t err;   // 1: a challenge found no canonical pair in FS_MAX_TRIES squeezes
    uint32_t pad_;
};

struct FsKeys {
    uint32_t absorb[8], squeeze[8], ratchet[8];
};

struct FsJob {
    char label[168];  // the job's prefix
    int label_len;
    int degree, ninst, n_max, inst0;  // inst0: the job's first instance in the per-instance arrays
    int pad_max;                      // the most padding rounds of any of its instances
    uint64_t rounds_off, chal_off;    // word offsets of the job's rounds and challenges
};
static_assert(sizeof(FsJob) % 8 == 0, "FsJob copies as words");

// A message is built as bytes in a shared-memory buffer and hashed a 64-byte block at a time
// straight from the buffer's words (little-endian, as BLAKE3 reads them).

constexpr int FS_THREADS = 128;  // four warps, one job each
constexpr int FS_BUF_WORDS = 132;  // 512 bytes of message, and 4 words that stagger the threads' banks

// The G function with its additions on the ALU: a transcript is a dependent chain, where the shorter
// latency counts, not the pipe the additions issue on (the column chains, bound by throughput, put
// them on the multiply-add pipe instead; here that form is about 10 % slower).
static __device__ __forceinline__ void b3_g_alu(uint32_t& a, uint32_t& b, uint32_t& c, uint32_t& d, uint32_t x,
                                                uint32_t y) {
    a = a + b + x;
    d = b3::rotr(d ^ a, 16);
    c = c + d;
    b = b3::rotr(b ^ c, 12);
    a = a + b + y;
    d = b3::rotr(d ^ a, 8);
    c = c + d;
    b = b3::rotr(b ^ c, 7);
}

// One compression by one thread with the additions on the ALU and the message in registers: a
// transcript is a chain of dependent compressions, and one thread's chain is shorter than that of
// four lanes running the G functions side by side with shuffles between the column and diagonal
// steps (about 1,250 against 1,450 cycles a compression on GB300).
#define FS_G(a, b, c, d, x, y) b3_g_alu(a, b, c, d, x, y);
#define FS_ROUND(m0, m1, m2, m3, m4, m5, m6, m7, m8, m9, m10, m11, m12, m13, m14, m15) \
    FS_G(s0, s4, s8, s12, m0, m1)                                                       \
    FS_G(s1, s5, s9, s13, m2, m3)                                                       \
    FS_G(s2, s6, s10, s14, m4, m5)                                                      \
    FS_G(s3, s7, s11, s15, m6, m7)                                                      \
    FS_G(s0, s5, s10, s15, m8, m9)                                                      \
    FS_G(s1, s6, s11, s12, m10, m11)                                                    \
    FS_G(s2, s7, s8, s13, m12, m13)                                                     \
    FS_G(s3, s4, s9, s14, m14, m15)
static __device__ __forceinline__ void compress_m(uint32_t cv[8], const uint32_t (&m)[16], uint32_t len, uint32_t flags) {
    uint32_t s0 = cv[0], s1 = cv[1], s2 = cv[2], s3 = cv[3], s4 = cv[4], s5 = cv[5], s6 = cv[6], s7 = cv[7];
    uint32_t s8 = TG_B3_IV0, s9 = TG_B3_IV1, s10 = TG_B3_IV2, s11 = TG_B3_IV3, s12 = 0, s13 = 0, s14 = len, s15 = flags;
    FS_ROUND(m[0], m[1], m[2], m[3], m[4], m[5], m[6], m[7], m[8], m[9], m[10], m[11], m[12], m[13], m[14], m[15])
    FS_ROUND(m[2], m[6], m[3], m[10], m[7], m[0], m[4], m[13], m[1], m[11], m[12], m[5], m[9], m[14], m[15], m[8])
    FS_ROUND(m[3], m[4], m[10], m[12], m[13], m[2], m[7], m[14], m[6], m[5], m[9], m[0], m[11], m[15], m[8], m[1])
    FS_ROUND(m[10], m[7], m[12], m[9], m[14], m[3], m[13], m[15], m[4], m[0], m[11], m[2], m[5], m[8], m[1], m[6])
    FS_ROUND(m[12], m[13], m[9], m[11], m[15], m[10], m[14], m[8], m[7], m[2], m[5], m[3], m[0], m[1], m[6], m[4])
    FS_ROUND(m[9], m[14], m[11], m[5], m[8], m[12], m[15], m[1], m[13], m[3], m[0], m[10], m[2], m[6], m[4], m[7])
    FS_ROUND(m[11], m[15], m[5], m[0], m[1], m[9], m[8], m[6], m[14], m[10], m[2], m[12], m[3], m[4], m[7], m[13])
    cv[0] = s0 ^ s8, cv[1] = s1 ^ s9, cv[2] = s2 ^ s10, cv[3] = s3 ^ s11;
    cv[4] = s4 ^ s12, cv[5] = s5 ^ s13, cv[6] = s6 ^ s14, cv[7] = s7 ^ s15;
}
#undef FS_ROUND
#undef FS_G
static __device__ __forceinline__ void compress_one(uint32_t cv[8], const uint32_t* mp, uint32_t len, uint32_t flags) {
    uint32_t m[16];
#pragma unroll
    for (int i = 0; i < 16; i++) m[i] = mp[i];
    compress_m(cv, m, len, flags);
}

// Eight words passed and returned by value, so that a call keeps them in registers (an array
// passed by address would live in local memory around every call).
struct Fs8 {
    uint32_t w[8];
};
static __device__ __forceinline__ Fs8 fs8(const uint32_t* p) {
    Fs8 v;
#pragma unroll
    for (int i = 0; i < 8; i++) v.w[i] = p[i];
    return v;
}

// BLAKE3 in derive-key-material mode under `key` of the first len bytes of buf (zero from len to
// the next block boundary), by lane 0 of a warp; every lane gets the output. One copy of the
// compression serves every call site.
static __device__ __noinline__ Fs8 fs_hash_warp(Fs8 key, const uint32_t* buf, uint32_t len) {
    Fs8 h = key;
    if ((threadIdx.x & 31) == 0) {
        const uint32_t nb = len == 0 ? 1 : (len + 63) / 64;
        for (uint32_t b = 0; b < nb; b++) {
            const bool last = b + 1 == nb;
            compress_one(h.w, buf + 16 * b, last ? len - 64 * b : 64,
                         b3::DERIVE_KEY_MATERIAL | (b == 0 ? b3::CHUNK_START : 0) | (last ? (b3::CHUNK_END | b3::ROOT) : 0));
        }
    }
    Fs8 out;
#pragma unroll
    for (int i = 0; i < 8; i++) out.w[i] = __shfl_sync(0xFFFFFFFFu, h.w[i], 0);
    return out;
}

// A label tail ("/round/", "/r/") as little-endian bytes of one word, and its length.
constexpr uint64_t fs_pack(const char* t) {
    uint64_t v = 0;
    for (int i = 0; i < 8 && t[i]; i++) v |= (uint64_t)(uint8_t)t[i] << (8 * i);
    return v;
}
constexpr int fs_len(const char* t) {
    int n = 0;
    while (t[n]) n++;
    return n;
}

// Decimal digits of j.
static __device__ __forceinline__ int fs_digits(int j) {
    int nd = 1;
    for (uint32_t q = (uint32_t)j; q >= 10; q /= 10) nd++;
    return nd;
}

// The head of a message by a whole warp: state ‖ u64 len(label) ‖ label into buf's first bytes,
// label = prefix ‖ tail ‖ decimal j (the same state and j in every lane); returns the head's length
// in every lane. Each lane writes its own bytes (the caller syncs the warp before buf is read).
static __device__ __forceinline__ uint32_t fs_head_warp(const uint32_t (&state)[8], const FsJob& jb, uint64_t tail,
                                                        int tail_len, int j, uint32_t* buf) {
    const int lane = threadIdx.x & 31;
    uint8_t* bytes = reinterpret_cast<uint8_t*>(buf);
    const int nd = fs_digits(j);
    const int pre = jb.label_len, L = pre + tail_len + nd;
    if (lane < 10) {  // words 0–9: the state and the label's length
        uint32_t v = lane == 8 ? (uint32_t)L : 0u;
#pragma unroll
        for (int i = 0; i < 8; i++)
            if (lane == i) v = state[i];
        buf[lane] = v;
    }
    for (int k = lane; k < L; k += 32) {
        uint32_t c;
        if (k < pre) {
            c = (uint8_t)jb.label[k];
        } else if (k < pre + tail_len) {
            c = (uint32_t)(tail >> (8 * (k - pre))) & 0xFFu;
        } else {
            uint32_t q = (uint32_t)j;
            for (int t = k - pre - tail_len + 1; t < nd; t++) q /= 10;
            c = '0' + q % 10;
        }
        bytes[40 + k] = (uint8_t)c;
    }
    return 40 + (uint32_t)L;
}

// The payload of a message by a whole warp: np little-endian u64 words (np ≤ NP; the same in every
// lane) from byte off of buf, then zeros to the next block boundary; returns the message's length.
template <int NP>
static __device__ __forceinline__ uint32_t fs_pay_warp(const uint64_t (&pay)[NP], int np, uint32_t off, uint32_t* buf) {
    const int lane = threadIdx.x & 31;
    uint8_t* bytes = reinterpret_cast<uint8_t*>(buf);
    const uint32_t len = off + 8 * (uint32_t)np;
    for (int k = lane; k < 8 * np; k += 32) {
        uint64_t v = 0;
#pragma unroll
        for (int i = 0; i < NP; i++)
            if ((k >> 3) == i) v = pay[i];
        bytes[off + k] = (uint8_t)(v >> (8 * (k & 7)));
    }
    const uint32_t end = (len + 63) / 64 * 64;
    for (uint32_t i = len + lane; i < end; i += 32) bytes[i] = 0;
    return len;
}

// A whole message: state ‖ u64 len(label) ‖ label ‖ payload into buf by a whole warp, label =
// prefix ‖ tail ‖ decimal j and payload np little-endian u64 words, then zeros to the next block
// boundary; returns the length in every lane.
template <int NP>
static __device__ __forceinline__ uint32_t fs_msg_warp(const uint32_t (&state)[8], const FsJob& jb, uint64_t tail,
                                                       int tail_len, int j, const uint64_t (&pay)[NP], int np,
                                                       uint32_t* buf) {
    const uint32_t off = fs_head_warp(state, jb, tail, tail_len, j, buf);
    return fs_pay_warp<NP>(pay, np, off, buf);
}

// Two warps of a block meet (named barrier 1, 64 threads): one has built the other's transcript
// inputs (the absorb's head, the first squeeze's input) while the other formed the message.
static __device__ __forceinline__ void fs_pair_sync() { asm volatile("bar.sync 1, 64;" ::: "memory"); }

// Round j's transcript step by a whole warp, its absorb input (state ‖ label length ‖
// <prefix>/round/j ‖ message) already in buf and zero padded (fs_msg_warp): absorbs it, then
// squeezes <prefix>/r/j until the first two words are a canonical Fp2 (c0, c1), every lane building
// the squeeze and ratchet inputs. state and counter are the same in every lane. False after
// FS_MAX_TRIES squeezes. sq (when given) holds the first squeeze's input, sq_len bytes, built by
// another warp all but its first eight words, the state after the absorb, which are written here.
static __device__ __forceinline__ bool fs_round_warp(const FsKeys& keys, const FsJob& jb, int j, uint32_t* buf,
                                                     uint32_t len, uint32_t (&state)[8], uint64_t* counter,
                                                     uint64_t* c0, uint64_t* c1, uint32_t* sq = nullptr,
                                                     uint32_t sq_len = 0) {
    const int lane = threadIdx.x & 31;
    __syncwarp();
    {
        const Fs8 h = fs_hash_warp(fs8(keys.absorb), buf, len);
#pragma unroll
        for (int i = 0; i < 8; i++) state[i] = h.w[i];
    }
    __syncwarp();
    for (int tries = 0; tries < FS_MAX_TRIES; tries++) {
        const uint32_t* in = buf;
        uint32_t l2;
        if (tries == 0 && sq) {
            if (lane < 8) sq[lane] = state[lane];
            in = sq;
            l2 = sq_len;
        } else {
            const uint64_t pay[1] = {*counter};
            l2 = fs_msg_warp<1>(state, jb, fs_pack("/r/"), fs_len("/r/"), j, pay, 1, buf);
        }
        __syncwarp();
        const Fs8 sqh = fs_hash_warp(fs8(keys.squeeze), in, l2);
        const uint32_t(&out)[8] = sqh.w;
        __syncwarp();
        *counter += 1;
        if (lane < 16) {  // the ratchet's input: state ‖ squeezed block
            uint32_t v = 0;
#pragma unroll
            for (int i = 0; i < 8; i++) {
                if (lane == i) v = state[i];
                if (lane == 8 + i) v = out[i];
            }
            buf[lane] = v;
        }
        __syncwarp();
        {
            const Fs8 h = fs_hash_warp(fs8(keys.ratchet), buf, 64);
#pragma unroll
            for (int i = 0; i < 8; i++) state[i] = h.w[i];
        }
        __syncwarp();
        *c0 = (uint64_t)out[0] | ((uint64_t)out[1] << 32);
        *c1 = (uint64_t)out[2] | ((uint64_t)out[3] << 32);
        if (*c0 < P && *c1 < P) return true;
    }
    return false;
}

}  // namespace tg
