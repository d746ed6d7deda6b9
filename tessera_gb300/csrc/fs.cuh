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
    uint64_t rounds_off, chal_off;    // word offsets of the job's rounds and challenges
};

// A message is built as bytes in a shared-memory buffer and hashed a 64-byte block at a time
// straight from the buffer's words (little-endian, as BLAKE3 reads them).

constexpr int FS_THREADS = 128;  // four warps, one job each
constexpr int FS_BUF_WORDS = 132;  // 512 bytes of message, and 4 words that stagger the threads' banks

// BLAKE3 (derive-key-material mode under `key`) of the first len bytes of buf; the bytes of buf
// past len up to the next block boundary are overwritten with zeros.
static __device__ void fs_hash(const uint32_t key[8], uint32_t* buf, uint32_t len, uint32_t out[8]) {
    uint8_t* bytes = reinterpret_cast<uint8_t*>(buf);
    const uint32_t nb = len == 0 ? 1 : (len + 63) / 64;
    for (uint32_t i = len; i < 64 * nb; i++) bytes[i] = 0;
    uint32_t h[8];
#pragma unroll
    for (int i = 0; i < 8; i++) h[i] = key[i];
    for (uint32_t b = 0; b < nb; b++) {
        uint32_t m[16];
#pragma unroll
        for (int i = 0; i < 16; i++) m[i] = buf[16 * b + i];
        const bool last = b + 1 == nb;
        b3::compress_cv(h, m, 0, last ? len - 64 * b : 64,
                        b3::DERIVE_KEY_MATERIAL | (b == 0 ? b3::CHUNK_START : 0) | (last ? (b3::CHUNK_END | b3::ROOT) : 0));
    }
#pragma unroll
    for (int i = 0; i < 8; i++) out[i] = h[i];
}

// ---- one compression by a warp: the four lanes of each quad run the column and the diagonal
// G functions of a round side by side (lane i holds column i: words i, 4 + i, 8 + i, 12 + i),
// rotating the rows by shuffles for the diagonal step; every lane ends with the whole chaining
// value.

// Word k of round r's message is m[kB3Sched[r][k]] (the message permutation applied r times).
constexpr uint8_t kB3Sched[7][16] = {
    {0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15},  {2, 6, 3, 10, 7, 0, 4, 13, 1, 11, 12, 5, 9, 14, 15, 8},
    {3, 4, 10, 12, 13, 2, 7, 14, 6, 5, 9, 0, 11, 15, 8, 1},  {10, 7, 12, 9, 14, 3, 13, 15, 4, 0, 11, 2, 5, 8, 1, 6},
    {12, 13, 9, 11, 15, 10, 14, 8, 7, 2, 5, 3, 0, 1, 6, 4},  {9, 14, 11, 5, 8, 12, 15, 1, 13, 3, 0, 10, 2, 6, 4, 7},
    {11, 15, 5, 0, 1, 9, 8, 6, 14, 10, 2, 12, 3, 4, 7, 13}};

// The four schedule indices lane i of a quad reads in round r (column words 2i, 2i + 1, diagonal
// words 8 + 2i, 9 + 2i), four bits each; rounds 0–3 in the low word, 4–6 in the high word, so a
// lane keeps its whole schedule in two registers instead of loading lane-divergent table entries.
__host__ __device__ constexpr uint64_t b3_lane_sched(int i, int half) {
    uint64_t v = 0;
    for (int r = 4 * half; r < 7 && r < 4 * half + 4; r++) {
        const uint64_t q = (uint64_t)kB3Sched[r][2 * i] | ((uint64_t)kB3Sched[r][2 * i + 1] << 4) |
                           ((uint64_t)kB3Sched[r][8 + 2 * i] << 8) | ((uint64_t)kB3Sched[r][9 + 2 * i] << 12);
        v |= q << (16 * (r - 4 * half));
    }
    return v;
}

static __device__ __forceinline__ void b3_g(uint32_t& a, uint32_t& b, uint32_t& c, uint32_t& d, uint32_t x, uint32_t y) {
    using namespace b3;
    TG_B3_G(a, b, c, d, x, y)
}

// ROLLED keeps one round's code (the schedule's words are lane-dependent lookups either way): for a
// warp that runs alone on its SM, whose unrolled rounds would miss in the instruction cache.
template <bool ROLLED>
static __device__ __forceinline__ void compress_quad(uint32_t cv[8], const uint32_t* m, uint32_t len, uint32_t flags) {
    const int i = threadIdx.x & 3;
    const uint32_t iv[4] = {TG_B3_IV0, TG_B3_IV1, TG_B3_IV2, TG_B3_IV3};
    uint32_t a = cv[i], b = cv[4 + i], c = iv[i], d = i < 2 ? 0u : i == 2 ? len : flags;
    constexpr uint64_t L0 = b3_lane_sched(0, 0), L1 = b3_lane_sched(1, 0), L2 = b3_lane_sched(2, 0), L3 = b3_lane_sched(3, 0);
    constexpr uint64_t H0 = b3_lane_sched(0, 1), H1 = b3_lane_sched(1, 1), H2 = b3_lane_sched(2, 1), H3 = b3_lane_sched(3, 1);
    uint64_t slo = i == 0 ? L0 : i == 1 ? L1 : i == 2 ? L2 : L3;
    uint64_t shi = i == 0 ? H0 : i == 1 ? H1 : i == 2 ? H2 : H3;
#pragma unroll(ROLLED ? 1 : 7)
    for (int r = 0; r < 7; r++) {
        const uint32_t q = (uint32_t)slo & 0xFFFFu;  // this round's four indices
        slo = (slo >> 16) | (shi << 48);
        shi >>= 16;
        b3_g(a, b, c, d, m[q & 15], m[(q >> 4) & 15]);
        b = __shfl_sync(0xFFFFFFFFu, b, (i + 1) & 3, 4);
        c = __shfl_sync(0xFFFFFFFFu, c, (i + 2) & 3, 4);
        d = __shfl_sync(0xFFFFFFFFu, d, (i + 3) & 3, 4);
        b3_g(a, b, c, d, m[(q >> 8) & 15], m[q >> 12]);
        b = __shfl_sync(0xFFFFFFFFu, b, (i + 3) & 3, 4);
        c = __shfl_sync(0xFFFFFFFFu, c, (i + 2) & 3, 4);
        d = __shfl_sync(0xFFFFFFFFu, d, (i + 1) & 3, 4);
    }
    const uint32_t lo = a ^ c, hi = b ^ d;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        cv[k] = __shfl_sync(0xFFFFFFFFu, lo, k, 4);
        cv[4 + k] = __shfl_sync(0xFFFFFFFFu, hi, k, 4);
    }
}

// fs_hash by a whole warp; the caller has zeroed buf from len to the next block boundary (one copy
// of the code for the absorb, squeeze and ratchet calls).
template <bool ROLLED>
static __device__ __noinline__ void fs_hash_warp(const uint32_t key[8], const uint32_t* buf, uint32_t len, uint32_t out[8]) {
    const uint32_t nb = len == 0 ? 1 : (len + 63) / 64;
    uint32_t h[8];
#pragma unroll
    for (int i = 0; i < 8; i++) h[i] = key[i];
    for (uint32_t b = 0; b < nb; b++) {
        const bool last = b + 1 == nb;
        compress_quad<ROLLED>(h, buf + 16 * b, last ? len - 64 * b : 64,
                      b3::DERIVE_KEY_MATERIAL | (b == 0 ? b3::CHUNK_START : 0) | (last ? (b3::CHUNK_END | b3::ROOT) : 0));
    }
#pragma unroll
    for (int i = 0; i < 8; i++) out[i] = h[i];
}

static __device__ __forceinline__ void zero_to_block(uint32_t* buf, uint32_t len) {
    uint8_t* bytes = reinterpret_cast<uint8_t*>(buf);
    const uint32_t end = (len == 0 ? 1 : (len + 63) / 64) * 64;
    for (uint32_t i = len; i < end; i++) bytes[i] = 0;
}

// zero_to_block by a whole warp (the caller syncs the warp after it).
static __device__ __forceinline__ void zero_to_block_warp(uint32_t* buf, uint32_t len) {
    uint8_t* bytes = reinterpret_cast<uint8_t*>(buf);
    const uint32_t end = (len == 0 ? 1 : (len + 63) / 64) * 64;
    for (uint32_t i = len + (threadIdx.x & 31); i < end; i += 32) bytes[i] = 0;
}

static __device__ __forceinline__ void put64(uint8_t* p, uint64_t v) {
    for (int i = 0; i < 8; i++) p[i] = (uint8_t)(v >> (8 * i));
}

// state ‖ u64 len(label) ‖ label, label = prefix ‖ tail ‖ decimal j, into buf; returns the length.
static __device__ uint32_t fs_begin(const uint32_t state[8], const FsJob& jb, const char* tail, int j, uint32_t* buf) {
    uint8_t* b = reinterpret_cast<uint8_t*>(buf);
#pragma unroll
    for (int i = 0; i < 8; i++) buf[i] = state[i];
    uint32_t n = 40;
    for (int i = 0; i < jb.label_len; i++) b[n++] = (uint8_t)jb.label[i];
    for (const char* c = tail; *c; c++) b[n++] = (uint8_t)*c;
    char digits[12];
    int nd = 0;
    do {
        digits[nd++] = (char)('0' + j % 10);
        j /= 10;
    } while (j > 0);
    while (nd > 0) b[n++] = (uint8_t)digits[--nd];
    buf[8] = n - 40;  // the label's length as a u64
    buf[9] = 0;
    return n;
}

// Round j's transcript step by a whole warp: lane 0 has written the round's absorb input (state ‖
// label length ‖ <prefix>/round/j ‖ message, len bytes) into buf; every lane absorbs it, then
// squeezes <prefix>/r/j until the first two words are a canonical Fp2 (c0, c1). state and counter
// are the same in every lane. False after FS_MAX_TRIES squeezes.
template <bool ROLLED = false>
static __device__ bool fs_round_warp(const FsKeys& keys, const FsJob& jb, int j, uint32_t* buf, uint32_t len,
                                     uint32_t state[8], uint64_t* counter, uint64_t* c0, uint64_t* c1) {
    const int lane = threadIdx.x & 31;
    zero_to_block_warp(buf, len);
    __syncwarp();
    fs_hash_warp<ROLLED>(keys.absorb, buf, len, state);
    __syncwarp();
    for (int tries = 0; tries < FS_MAX_TRIES; tries++) {
        uint32_t l2 = 0;
        if (lane == 0) {
            l2 = fs_begin(state, jb, "/r/", j, buf);
            put64(reinterpret_cast<uint8_t*>(buf) + l2, *counter);
        }
        l2 = __shfl_sync(0xFFFFFFFFu, l2, 0);
        __syncwarp();
        zero_to_block_warp(buf, l2 + 8);
        __syncwarp();
        uint32_t out[8];
        fs_hash_warp<ROLLED>(keys.squeeze, buf, l2 + 8, out);
        __syncwarp();
        *counter += 1;
        if (lane == 0)
            for (int i = 0; i < 8; i++) buf[i] = state[i], buf[8 + i] = out[i];
        __syncwarp();
        fs_hash_warp<ROLLED>(keys.ratchet, buf, 64, state);
        __syncwarp();
        *c0 = (uint64_t)out[0] | ((uint64_t)out[1] << 32);
        *c1 = (uint64_t)out[2] | ((uint64_t)out[3] << 32);
        if (*c0 < P && *c1 < P) return true;
    }
    return false;
}

}  // namespace tg
