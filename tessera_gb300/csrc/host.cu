// SPDX-License-Identifier: Apache-2.0 OR MIT
//
// Host side of the library: BLAKE3 over inputs of any length (the transcript's messages can
// span many chunks), the domain hash H(domain, x), and the Fiat–Shamir transcript of the
// reference (crates/tessera-hash/src/transcript.rs:127-250): absorb, squeeze with ratchet,
// challenge_fp2 / challenge_fp by rejection, challenge_indices, and proof-of-work grinding.
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <array>
#include <string>
#include <vector>

#include "b3.cuh"
#include "gl.cuh"
#include "internal.h"

namespace tg {

static const uint32_t IV[8] = {TG_B3_IV0, TG_B3_IV1, TG_B3_IV2, TG_B3_IV3,
                               TG_B3_IV4, TG_B3_IV5, TG_B3_IV6, TG_B3_IV7};

static void words16(const uint8_t* p, size_t len, uint32_t m[16]) {
    uint8_t buf[64] = {0};
    memcpy(buf, p, len);
    for (int i = 0; i < 16; i++) m[i] = b3::le32(buf + 4 * i);
}

struct Node {
    uint32_t cv[8];
    uint32_t m[16];
    uint64_t counter;
    uint32_t len, flags;
};

static void node_cv(const Node& n, uint32_t out[8]) {
    memcpy(out, n.cv, 32);
    b3::compress_cv(out, n.m, n.counter, n.len, n.flags);
}

// The chunk's last block, with the blocks before it compressed into its chaining value.
static Node chunk_node(const uint32_t key[8], const uint8_t* in, size_t len, uint64_t chunk, uint32_t mode) {
    Node n;
    memcpy(n.cv, key, 32);
    const size_t nb = len == 0 ? 1 : (len + 63) / 64;
    for (size_t b = 0; b + 1 < nb; b++) {
        uint32_t m[16];
        words16(in + 64 * b, 64, m);
        b3::compress_cv(n.cv, m, chunk, 64, mode | (b == 0 ? (uint32_t)b3::CHUNK_START : 0u));
    }
    const size_t last = len - 64 * (nb - 1);
    words16(in + 64 * (nb - 1), last, n.m);
    n.counter = chunk;
    n.len = (uint32_t)last;
    n.flags = mode | b3::CHUNK_END | (nb == 1 ? (uint32_t)b3::CHUNK_START : 0u);
    return n;
}

static Node parent_node(const uint32_t key[8], const uint32_t l[8], const uint32_t r[8], uint32_t mode) {
    Node n;
    memcpy(n.cv, key, 32);
    memcpy(n.m, l, 32);
    memcpy(n.m + 8, r, 32);
    n.counter = 0;
    n.len = 64;
    n.flags = mode | b3::PARENT;
    return n;
}

// BLAKE3 with chaining-value key `key` and mode flags, 32 bytes of output.
static void b3_hash(const uint32_t key[8], uint32_t mode, const uint8_t* in, size_t len, uint8_t out[32]) {
    const size_t nchunks = len == 0 ? 1 : (len + 1023) / 1024;
    std::vector<std::array<uint32_t, 8>> stack;
    for (size_t c = 0; c + 1 < nchunks; c++) {
        Node n = chunk_node(key, in + 1024 * c, 1024, c, mode);
        std::array<uint32_t, 8> cv;
        node_cv(n, cv.data());
        uint64_t total = c + 1;
        while ((total & 1) == 0) {
            Node p = parent_node(key, stack.back().data(), cv.data(), mode);
            stack.pop_back();
            node_cv(p, cv.data());
            total >>= 1;
        }
        stack.push_back(cv);
    }
    const size_t off = 1024 * (nchunks - 1);
    Node node = chunk_node(key, in + off, len - off, nchunks - 1, mode);
    while (!stack.empty()) {
        uint32_t cv[8];
        node_cv(node, cv);
        node = parent_node(key, stack.back().data(), cv, mode);
        stack.pop_back();
    }
    uint32_t o[16];
    b3::compress_full(node.cv, node.m, 0, node.len, node.flags | b3::ROOT, o);
    for (int i = 0; i < 32; i++) out[i] = (uint8_t)(o[i / 4] >> (8 * (i % 4)));
}

void context_key(const char* name, uint32_t key[8]) {
    std::string ctx = std::string("tessera/v1/") + name;
    uint8_t k[32];
    b3_hash(IV, b3::DERIVE_KEY_CONTEXT, (const uint8_t*)ctx.data(), ctx.size(), k);
    for (int i = 0; i < 8; i++) key[i] = b3::le32(k + 4 * i);
}

void host_hash(const uint32_t key[8], const uint8_t* in, size_t len, uint8_t out[32]) {
    b3_hash(key, b3::DERIVE_KEY_MATERIAL, in, len, out);
}

struct Domains {
    uint32_t init[8], absorb[8], squeeze[8], ratchet[8], pow[8];
    Domains() {
        context_key("transcript-init", init);
        context_key("transcript-absorb", absorb);
        context_key("transcript-squeeze", squeeze);
        context_key("transcript-ratchet", ratchet);
        context_key("pow", pow);
    }
};
static const Domains& domains() {
    static const Domains d;
    return d;
}

static void put64(std::vector<uint8_t>& v, uint64_t x) {
    for (int i = 0; i < 8; i++) v.push_back((uint8_t)(x >> (8 * i)));
}
static uint64_t get64(const uint8_t* p) {
    uint64_t v = 0;
    for (int i = 7; i >= 0; i--) v = (v << 8) | p[i];
    return v;
}

// state ‖ u64 len(label) ‖ label (the reference's begin(), transcript.rs:154-161)
static std::vector<uint8_t> begin(const tg_transcript* t, const char* label) {
    std::vector<uint8_t> v(t->state, t->state + 32);
    const size_t n = strlen(label);
    put64(v, n);
    v.insert(v.end(), label, label + n);
    return v;
}

static bool printable(const char* label) {
    for (const char* p = label; *p; p++)
        if (*p < 0x20 || *p > 0x7E) return false;
    return true;
}

}  // namespace tg

using namespace tg;

extern "C" {

int tg_hash(const char* domain, const uint8_t* in, size_t len, uint8_t out[32]) {
    if (!domain || (!in && len) || !out) return fail(TG_ERR_INVALID, "tg_hash: null argument");
    uint32_t key[8];
    context_key(domain, key);
    host_hash(key, in, len, out);
    return TG_OK;
}

int tg_transcript_init(tg_transcript* t, const uint8_t* context_tce, size_t len) {
    if (!t || (!context_tce && len)) return fail(TG_ERR_INVALID, "tg_transcript_init: null argument");
    host_hash(domains().init, context_tce, len, t->state);
    t->counter = 0;
    return TG_OK;
}

int tg_transcript_absorb(tg_transcript* t, const char* label, const uint8_t* value, size_t len) {
    if (!t || !label || (!value && len)) return fail(TG_ERR_INVALID, "tg_transcript_absorb: null argument");
    if (!printable(label)) return fail(TG_ERR_INVALID, "a transcript label is printable ASCII");
    std::vector<uint8_t> in = begin(t, label);
    in.insert(in.end(), value, value + len);
    host_hash(domains().absorb, in.data(), in.size(), t->state);
    return TG_OK;
}

int tg_transcript_squeeze(tg_transcript* t, const char* label, uint8_t out[32]) {
    if (!t || !label || !out) return fail(TG_ERR_INVALID, "tg_transcript_squeeze: null argument");
    if (!printable(label)) return fail(TG_ERR_INVALID, "a transcript label is printable ASCII");
    if (t->counter == UINT64_MAX) return fail(TG_ERR_STATE, "a transcript makes fewer than 2^64 squeezes");
    std::vector<uint8_t> in = begin(t, label);
    put64(in, t->counter);
    host_hash(domains().squeeze, in.data(), in.size(), out);
    t->counter += 1;
    uint8_t r[64];
    memcpy(r, t->state, 32);
    memcpy(r + 32, out, 32);
    host_hash(domains().ratchet, r, 64, t->state);
    return TG_OK;
}

int tg_transcript_challenge_fp2(tg_transcript* t, const char* label, uint64_t out[2]) {
    for (;;) {
        uint8_t d[32];
        int rc = tg_transcript_squeeze(t, label, d);
        if (rc) return rc;
        const uint64_t c0 = get64(d), c1 = get64(d + 8);
        if (c0 < P && c1 < P) {
            out[0] = c0;
            out[1] = c1;
            return TG_OK;
        }
    }
}

int tg_transcript_challenge_fp(tg_transcript* t, const char* label, uint64_t* out) {
    for (;;) {
        uint8_t d[32];
        int rc = tg_transcript_squeeze(t, label, d);
        if (rc) return rc;
        for (int i = 0; i < 4; i++) {
            const uint64_t w = get64(d + 8 * i);
            if (w < P) {
                *out = w;
                return TG_OK;
            }
        }
    }
}

int tg_transcript_challenge_indices(tg_transcript* t, const char* label, uint32_t log_n, uint32_t count,
                                    uint64_t* out) {
    if (log_n > 64) return fail(TG_ERR_INVALID, "an index domain of 2^%u exceeds u64", log_n);
    const uint64_t mask = log_n >= 64 ? ~0ull : ((1ull << log_n) - 1);
    uint32_t have = 0;
    while (have < count) {
        uint8_t d[32];
        int rc = tg_transcript_squeeze(t, label, d);
        if (rc) return rc;
        for (int i = 0; i < 4 && have < count; i++) out[have++] = get64(d + 8 * i) & mask;
    }
    return TG_OK;
}

// Absorbs TCE Vec<Fp2>: u64 LE length, then c0 ‖ c1 of each element (8 bytes LE each).
int tg_transcript_absorb_fp2s(tg_transcript* t, const char* label, const uint64_t* values, size_t count) {
    std::vector<uint8_t> v;
    v.reserve(8 + 16 * count);
    put64(v, count);
    for (size_t i = 0; i < 2 * count; i++) put64(v, values[i]);
    return tg_transcript_absorb(t, label, v.data(), v.size());
}

static bool pow_meets(const tg_transcript* t, const char* label, uint32_t bits, uint64_t nonce) {
    std::vector<uint8_t> in = begin(t, label);
    put64(in, nonce);
    uint8_t d[32];
    host_hash(domains().pow, in.data(), in.size(), d);
    uint32_t zeros = 0;
    for (int i = 0; i < 32; i++) {
        if (d[i]) {
            zeros += __builtin_clz((unsigned)d[i]) - 24;
            break;
        }
        zeros += 8;
    }
    return zeros >= bits;
}

int tg_transcript_check_grind(tg_transcript* t, const char* label, uint32_t bits, uint64_t nonce, int* valid) {
    if (!t || !label || !valid) return fail(TG_ERR_INVALID, "tg_transcript_check_grind: null argument");
    *valid = pow_meets(t, label, bits, nonce);
    if (*valid) {
        uint8_t v[8];
        for (int i = 0; i < 8; i++) v[i] = (uint8_t)(nonce >> (8 * i));
        return tg_transcript_absorb(t, label, v, 8);
    }
    return TG_OK;
}

}  // extern "C"
