/* SPDX-License-Identifier: Apache-2.0 OR MIT
 *
 * TEST INFRASTRUCTURE ONLY: the CPU oracle of the proving hot path, a plain-C restatement of
 * the reference's Rust algorithms. The test suite uses it as the checker of the CUDA path and
 * the benchmark times it as the CPU baseline; the product library never links or calls it.
 * Parity is pinned against the reference's golden vectors (see tests/test_oracle_golden.py).
 *
 * Paths in citations are relative to the reference repository (AbdelStark/tessera).
 */
#include "tessera_oracle.h"

#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

typedef unsigned __int128 u128;

/* ======================================================================================== */
/* Goldilocks: crates/tessera-field/src/goldilocks.rs:23-108                                */
/* ======================================================================================== */

#define FP_P 0xFFFFFFFF00000001ULL
#define FP_EPS 0xFFFFFFFFULL

static inline uint64_t canon(uint64_t x) { return x >= FP_P ? x - FP_P : x; }

/* add: goldilocks.rs:40-47 */
static inline uint64_t fadd(uint64_t a, uint64_t b) {
    uint64_t s = a + b;
    s += (s < a) ? FP_EPS : 0;
    return canon(s);
}
/* sub: goldilocks.rs:49-55 */
static inline uint64_t fsub(uint64_t a, uint64_t b) {
    uint64_t d = a - b;
    return d - ((a < b) ? FP_EPS : 0);
}
/* reduce128: goldilocks.rs:57-77; 2^64 = 2^32 - 1 and 2^96 = -1 (mod p) */
static inline uint64_t reduce128(u128 x) {
    uint64_t lo = (uint64_t)x, hi = (uint64_t)(x >> 64);
    uint64_t hh = hi >> 32, hl = hi & FP_EPS;
    uint64_t t0 = lo - hh;
    if (lo < hh) t0 -= FP_EPS;
    uint64_t t1 = hl * FP_EPS;
    uint64_t t2 = t0 + t1;
    if (t2 < t1) t2 += FP_EPS;
    return canon(t2);
}
static inline uint64_t fmul(uint64_t a, uint64_t b) { return reduce128((u128)a * b); }
static uint64_t fpow(uint64_t a, uint64_t e) {
    uint64_t acc = 1;
    while (e) {
        if (e & 1) acc = fmul(acc, a);
        a = fmul(a, a);
        e >>= 1;
    }
    return acc;
}
static inline uint64_t finv(uint64_t a) { return fpow(a, FP_P - 2); }

uint64_t or_fp_add(uint64_t a, uint64_t b) { return fadd(a, b); }
uint64_t or_fp_sub(uint64_t a, uint64_t b) { return fsub(a, b); }
uint64_t or_fp_mul(uint64_t a, uint64_t b) { return fmul(a, b); }
uint64_t or_fp_pow(uint64_t a, uint64_t e) { return fpow(a, e); }
uint64_t or_fp_inv(uint64_t a) { return finv(a); }
uint64_t or_fp_reduce(uint64_t x) { return canon(x); }

/* two_adic_generator: ROOT_2_32 = 7^((p-1)/2^32), ROOTS[k] = ROOT_2_32^(2^(32-k))
 * (goldilocks.rs:167-179, 397-403). */
uint64_t or_root_of_unity(uint32_t log_n) { return fpow(7, (FP_P - 1) >> log_n); }

/* Fp2 = Fp[X]/(X^2 - 7), Karatsuba (crates/tessera-field/src/ext2.rs:41, 235-249) */
typedef struct {
    uint64_t c0, c1;
} fp2;
static inline fp2 e_add(fp2 a, fp2 b) { return (fp2){fadd(a.c0, b.c0), fadd(a.c1, b.c1)}; }
static inline fp2 e_sub(fp2 a, fp2 b) { return (fp2){fsub(a.c0, b.c0), fsub(a.c1, b.c1)}; }
static inline fp2 e_mul(fp2 a, fp2 b) {
    uint64_t v0 = fmul(a.c0, b.c0), v1 = fmul(a.c1, b.c1);
    uint64_t cross = fmul(fadd(a.c0, a.c1), fadd(b.c0, b.c1));
    return (fp2){fadd(v0, fmul(v1, 7)), fsub(fsub(cross, v0), v1)};
}
static inline fp2 e_scale(fp2 a, uint64_t s) { return (fp2){fmul(a.c0, s), fmul(a.c1, s)}; }
static inline fp2 e_lift(uint64_t x) { return (fp2){x, 0}; }
static const fp2 E_ZERO = {0, 0};
static const fp2 E_ONE = {1, 0};

void or_fp2_mul(const uint64_t a[2], const uint64_t b[2], uint64_t out[2]) {
    fp2 r = e_mul((fp2){a[0], a[1]}, (fp2){b[0], b[1]});
    out[0] = r.c0;
    out[1] = r.c1;
}
/* (a0 + a1 X)^-1 = (a0 - a1 X) / (a0^2 - 7 a1^2) (ext2.rs inverse) */
void or_fp2_inv(const uint64_t a[2], uint64_t out[2]) {
    uint64_t norm = fsub(fmul(a[0], a[0]), fmul(7, fmul(a[1], a[1])));
    uint64_t ni = finv(norm);
    out[0] = fmul(a[0], ni);
    out[1] = fmul(fsub(0, a[1]), ni);
}
void or_fp_vec(int op, const uint64_t *a, const uint64_t *b, uint64_t *out, size_t n) {
    for (size_t i = 0; i < n; i++)
        out[i] = op == 0 ? fadd(a[i], b[i]) : op == 1 ? fsub(a[i], b[i]) : fmul(a[i], b[i]);
}
void or_fp2_vec_mul(const uint64_t *a, const uint64_t *b, uint64_t *out, size_t n) {
    for (size_t i = 0; i < n; i++) or_fp2_mul(a + 2 * i, b + 2 * i, out + 2 * i);
}

/* ======================================================================================== */
/* A small parallel-for over pthreads (the baseline's "all cores" mode).                     */
/* ======================================================================================== */

typedef void (*range_fn)(void *ctx, size_t lo, size_t hi);
typedef struct {
    range_fn fn;
    void *ctx;
    size_t lo, hi;
} range_job;
static void *range_run(void *p) {
    range_job *j = (range_job *)p;
    j->fn(j->ctx, j->lo, j->hi);
    return NULL;
}
static void parallel_for(size_t n, int threads, range_fn fn, void *ctx) {
    if (threads <= 1 || n < 2) {
        fn(ctx, 0, n);
        return;
    }
    if ((size_t)threads > n) threads = (int)n;
    pthread_t tid[256];
    range_job jobs[256];
    if (threads > 256) threads = 256;
    for (int i = 0; i < threads; i++) {
        jobs[i] = (range_job){fn, ctx, n * i / threads, n * (i + 1) / threads};
        if (i > 0 && pthread_create(&tid[i], NULL, range_run, &jobs[i]) != 0) {
            jobs[i].fn(ctx, jobs[i].lo, jobs[i].hi); /* no thread: run it here */
            tid[i] = 0;
        }
    }
    fn(ctx, jobs[0].lo, jobs[0].hi);
    for (int i = 1; i < threads; i++)
        if (tid[i]) pthread_join(tid[i], NULL);
}

/* ======================================================================================== */
/* BLAKE3, from the published specification (the reference calls the blake3 crate 1.8.7:     */
/* crates/tessera-hash/src/domain.rs:129-181).                                               */
/* ======================================================================================== */

enum {
    B3_CHUNK_START = 1,
    B3_CHUNK_END = 2,
    B3_PARENT = 4,
    B3_ROOT = 8,
    B3_KEYED_HASH = 16,
    B3_DERIVE_KEY_CONTEXT = 32,
    B3_DERIVE_KEY_MATERIAL = 64,
};
static const uint32_t B3_IV[8] = {0x6A09E667, 0xBB67AE85, 0x3C6EF372, 0xA54FF53A,
                                  0x510E527F, 0x9B05688C, 0x1F83D9AB, 0x5BE0CD19};
static const uint8_t B3_PERM[16] = {2, 6, 3, 10, 7, 0, 4, 13, 1, 11, 12, 5, 9, 14, 15, 8};

static inline uint32_t rotr32(uint32_t x, int n) { return (x >> n) | (x << (32 - n)); }
static inline void b3_g(uint32_t *s, int a, int b, int c, int d, uint32_t x, uint32_t y) {
    s[a] = s[a] + s[b] + x;
    s[d] = rotr32(s[d] ^ s[a], 16);
    s[c] = s[c] + s[d];
    s[b] = rotr32(s[b] ^ s[c], 12);
    s[a] = s[a] + s[b] + y;
    s[d] = rotr32(s[d] ^ s[a], 8);
    s[c] = s[c] + s[d];
    s[b] = rotr32(s[b] ^ s[c], 7);
}
static void b3_compress(const uint32_t cv[8], const uint32_t block[16], uint64_t counter,
                        uint32_t block_len, uint32_t flags, uint32_t out[16]) {
    uint32_t s[16], m[16], t[16];
    memcpy(s, cv, 32);
    memcpy(s + 8, B3_IV, 16);
    s[12] = (uint32_t)counter;
    s[13] = (uint32_t)(counter >> 32);
    s[14] = block_len;
    s[15] = flags;
    memcpy(m, block, 64);
    for (int r = 0; r < 7; r++) {
        b3_g(s, 0, 4, 8, 12, m[0], m[1]);
        b3_g(s, 1, 5, 9, 13, m[2], m[3]);
        b3_g(s, 2, 6, 10, 14, m[4], m[5]);
        b3_g(s, 3, 7, 11, 15, m[6], m[7]);
        b3_g(s, 0, 5, 10, 15, m[8], m[9]);
        b3_g(s, 1, 6, 11, 12, m[10], m[11]);
        b3_g(s, 2, 7, 8, 13, m[12], m[13]);
        b3_g(s, 3, 4, 9, 14, m[14], m[15]);
        if (r < 6) {
            for (int i = 0; i < 16; i++) t[i] = m[B3_PERM[i]];
            memcpy(m, t, 64);
        }
    }
    for (int i = 0; i < 8; i++) {
        out[i] = s[i] ^ s[i + 8];
        out[i + 8] = s[i + 8] ^ cv[i];
    }
}
static void b3_words(const uint8_t *bytes, size_t len, uint32_t block[16]) {
    uint8_t buf[64] = {0};
    memcpy(buf, bytes, len);
    for (int i = 0; i < 16; i++)
        block[i] = (uint32_t)buf[4 * i] | ((uint32_t)buf[4 * i + 1] << 8) |
                   ((uint32_t)buf[4 * i + 2] << 16) | ((uint32_t)buf[4 * i + 3] << 24);
}

/* The node whose compression yields the output: its inputs are kept for XOF output. */
typedef struct {
    uint32_t cv[8];
    uint32_t block[16];
    uint64_t counter;
    uint32_t block_len, flags;
} b3_node;

/* Compresses one chunk up to (not including) its last block; returns the last block's node. */
static b3_node b3_chunk(const uint32_t key[8], const uint8_t *in, size_t len, uint64_t chunk,
                        uint32_t mode) {
    uint32_t cv[8], block[16], out[16];
    memcpy(cv, key, 32);
    size_t nblocks = len == 0 ? 1 : (len + 63) / 64;
    for (size_t b = 0; b + 1 < nblocks; b++) {
        b3_words(in + 64 * b, 64, block);
        b3_compress(cv, block, chunk, 64, mode | (b == 0 ? B3_CHUNK_START : 0), out);
        memcpy(cv, out, 32);
    }
    b3_node node;
    memcpy(node.cv, cv, 32);
    size_t last = len - 64 * (nblocks - 1);
    b3_words(in + 64 * (nblocks - 1), last, node.block);
    node.counter = chunk;
    node.block_len = (uint32_t)last;
    node.flags = mode | B3_CHUNK_END | (nblocks == 1 ? B3_CHUNK_START : 0);
    return node;
}
static void b3_node_cv(const b3_node *n, uint32_t cv[8]) {
    uint32_t out[16];
    b3_compress(n->cv, n->block, n->counter, n->block_len, n->flags, out);
    memcpy(cv, out, 32);
}
static b3_node b3_parent(const uint32_t key[8], const uint32_t l[8], const uint32_t r[8],
                         uint32_t mode) {
    b3_node n;
    memcpy(n.cv, key, 32);
    memcpy(n.block, l, 32);
    memcpy(n.block + 8, r, 32);
    n.counter = 0;
    n.block_len = 64;
    n.flags = mode | B3_PARENT;
    return n;
}
/* The root node of the tree over `len` bytes: chunks merged left to right with a CV stack,
 * the left subtree always the largest complete power of two. */
static b3_node b3_root_node(const uint32_t key[8], const uint8_t *in, size_t len, uint32_t mode) {
    size_t nchunks = len == 0 ? 1 : (len + 1023) / 1024;
    uint32_t stack[64][8];
    int depth = 0;
    for (size_t c = 0; c + 1 < nchunks; c++) {
        b3_node n = b3_chunk(key, in + 1024 * c, 1024, c, mode);
        uint32_t cv[8];
        b3_node_cv(&n, cv);
        uint64_t total = c + 1;
        while ((total & 1) == 0) {
            b3_node p = b3_parent(key, stack[--depth], cv, mode);
            b3_node_cv(&p, cv);
            total >>= 1;
        }
        memcpy(stack[depth++], cv, 32);
    }
    size_t off = 1024 * (nchunks - 1);
    b3_node node = b3_chunk(key, in + off, len - off, nchunks - 1, mode);
    while (depth > 0) {
        uint32_t cv[8];
        b3_node_cv(&node, cv);
        node = b3_parent(key, stack[--depth], cv, mode);
    }
    return node;
}
static void b3_output(const b3_node *root, uint8_t *out, size_t out_len) {
    uint32_t w[16];
    for (uint64_t blk = 0; out_len > 0; blk++) {
        b3_compress(root->cv, root->block, blk, root->block_len, root->flags | B3_ROOT, w);
        for (int i = 0; i < 64 && out_len > 0; i++, out_len--) *out++ = (uint8_t)(w[i / 4] >> (8 * (i % 4)));
    }
}
static void b3_hash_with(const uint32_t key[8], uint32_t mode, const uint8_t *in, size_t len,
                         uint8_t *out, size_t out_len) {
    b3_node root = b3_root_node(key, in, len, mode);
    b3_output(&root, out, out_len);
}
static void b3_key_words(const uint8_t k[32], uint32_t w[8]) {
    for (int i = 0; i < 8; i++)
        w[i] = (uint32_t)k[4 * i] | ((uint32_t)k[4 * i + 1] << 8) | ((uint32_t)k[4 * i + 2] << 16) |
               ((uint32_t)k[4 * i + 3] << 24);
}
void or_blake3(int mode, const void *key, const uint8_t *in, size_t len, uint8_t *out,
               size_t out_len) {
    uint32_t kw[8];
    if (mode == 0) {
        b3_hash_with(B3_IV, 0, in, len, out, out_len);
    } else if (mode == 1) {
        b3_key_words((const uint8_t *)key, kw);
        b3_hash_with(kw, B3_KEYED_HASH, in, len, out, out_len);
    } else {
        const char *ctx = (const char *)key;
        uint8_t ck[32];
        b3_hash_with(B3_IV, B3_DERIVE_KEY_CONTEXT, (const uint8_t *)ctx, strlen(ctx), ck, 32);
        b3_key_words(ck, kw);
        b3_hash_with(kw, B3_DERIVE_KEY_MATERIAL, in, len, out, out_len);
    }
}

/* CONTEXT_KEYS: the key of "tessera/v1/<name>" (crates/tessera-hash/src/domain.rs:134-158) */
void or_context_key(const char *name, uint8_t key[32]) {
    char ctx[128];
    size_t n = strlen(name);
    if (n > 100) n = 100;
    memcpy(ctx, "tessera/v1/", 11);
    memcpy(ctx + 11, name, n);
    ctx[11 + n] = 0;
    b3_hash_with(B3_IV, B3_DERIVE_KEY_CONTEXT, (const uint8_t *)ctx, 11 + n, key, 32);
}

/* A domain hasher with its context key derived once (domain.rs:160-181). */
typedef struct {
    uint32_t key[8];
} dom;
static dom dom_new(const char *name) {
    uint8_t k[32];
    dom d;
    or_context_key(name, k);
    b3_key_words(k, d.key);
    return d;
}
static void dom_hash(const dom *d, const uint8_t *in, size_t len, uint8_t out[32]) {
    b3_hash_with(d->key, B3_DERIVE_KEY_MATERIAL, in, len, out, 32);
}
void or_hash(const char *name, const uint8_t *in, size_t len, uint8_t out[32]) {
    dom d = dom_new(name);
    dom_hash(&d, in, len, out);
}

/* ======================================================================================== */
/* Column chains: crates/tessera-hash/src/columns.rs:72-104                                  */
/* ======================================================================================== */

static inline void le64(uint8_t *p, uint64_t v) {
    for (int i = 0; i < 8; i++) p[i] = (uint8_t)(v >> (8 * i));
}

typedef struct {
    dom d;
    const uint8_t *id;
    uint8_t *chains;
} init_ctx;
static void init_range(void *c, size_t lo, size_t hi) {
    init_ctx *x = (init_ctx *)c;
    uint8_t in[40];
    memcpy(in, x->id, 32);
    for (size_t j = lo; j < hi; j++) {
        le64(in + 32, j);
        dom_hash(&x->d, in, 40, x->chains + 32 * j);
    }
}
/* ColumnChains::new, columns.rs:72-88: d_j = H("column-init", id || u64 j) */
void or_column_init(const uint8_t id[32], uint64_t ncols, uint8_t *chains, int threads) {
    init_ctx c = {dom_new("column-init"), id, chains};
    parallel_for(ncols, threads, init_range, &c);
}

typedef struct {
    dom d;
    uint8_t *chains;
    uint64_t ncols;
    const uint64_t *rows;
    size_t count;
} absorb_ctx;
static void absorb_range(void *c, size_t lo, size_t hi) {
    absorb_ctx *x = (absorb_ctx *)c;
    size_t len = 32 + 8 * x->count;
    uint8_t *in = (uint8_t *)malloc(len);
    for (size_t j = lo; j < hi; j++) {
        memcpy(in, x->chains + 32 * j, 32);
        for (size_t r = 0; r < x->count; r++) le64(in + 32 + 8 * r, x->rows[r * x->ncols + j]);
        dom_hash(&x->d, in, len, x->chains + 32 * j);
    }
    free(in);
}
/* ColumnChains::absorb_block, columns.rs:90-104: d_j = H("column-step", d_j || symbols) */
void or_column_absorb(uint8_t *chains, uint64_t ncols, const uint64_t *rows, size_t count,
                      int threads) {
    absorb_ctx c = {dom_new("column-step"), chains, ncols, rows, count};
    parallel_for(ncols, threads, absorb_range, &c);
}

/* ======================================================================================== */
/* Merkle tree: crates/tessera-hash/src/merkle.rs:10-16, 93-113                              */
/* ======================================================================================== */

void or_merkle_node(const uint8_t l[32], const uint8_t r[32], uint8_t out[32]) {
    uint8_t in[64];
    memcpy(in, l, 32);
    memcpy(in + 32, r, 32);
    or_hash("merkle-node", in, 64, out);
}
typedef struct {
    dom d;
    const uint8_t *src;
    uint8_t *dst;
} level_ctx;
static void level_range(void *c, size_t lo, size_t hi) {
    level_ctx *x = (level_ctx *)c;
    for (size_t i = lo; i < hi; i++) dom_hash(&x->d, x->src + 64 * i, 64, x->dst + 32 * i);
}
void or_merkle_tree(const uint8_t *leaves, size_t n, uint8_t *nodes, int threads) {
    memcpy(nodes, leaves, 32 * n);
    size_t start = 0, width = n;
    level_ctx c = {dom_new("merkle-node"), NULL, NULL};
    while (width > 1) {
        c.src = nodes + 32 * start;
        c.dst = nodes + 32 * (start + width);
        parallel_for(width / 2, threads, level_range, &c);
        start += width;
        width /= 2;
    }
}
void or_merkle_root(const uint8_t *leaves, size_t n, uint8_t root[32], int threads) {
    uint8_t *nodes = (uint8_t *)malloc(32 * (2 * n - 1));
    or_merkle_tree(leaves, n, nodes, threads);
    memcpy(root, nodes + 32 * (2 * n - 2), 32);
    free(nodes);
}

/* ======================================================================================== */
/* Transcript: crates/tessera-hash/src/transcript.rs:127-219, label_prefix :294-300           */
/* ======================================================================================== */

void or_transcript_init(or_transcript *t, const uint8_t *ctx, size_t len) {
    or_hash("transcript-init", ctx, len, t->state);
    t->counter = 0;
}
static void tr_begin(const or_transcript *t, const char *label, uint8_t *buf, size_t *off) {
    size_t n = strlen(label);
    memcpy(buf, t->state, 32);
    le64(buf + 32, n);
    memcpy(buf + 40, label, n);
    *off = 40 + n;
}
void or_transcript_absorb(or_transcript *t, const char *label, const uint8_t *value, size_t len) {
    size_t n = strlen(label), off;
    uint8_t *buf = (uint8_t *)malloc(40 + n + len);
    tr_begin(t, label, buf, &off);
    memcpy(buf + off, value, len);
    or_hash("transcript-absorb", buf, off + len, t->state);
    free(buf);
}
void or_transcript_squeeze(or_transcript *t, const char *label, uint8_t out[32]) {
    size_t n = strlen(label), off;
    uint8_t *buf = (uint8_t *)malloc(48 + n);
    tr_begin(t, label, buf, &off);
    le64(buf + off, t->counter);
    or_hash("transcript-squeeze", buf, off + 8, out);
    free(buf);
    t->counter += 1;
    uint8_t r[64];
    memcpy(r, t->state, 32);
    memcpy(r + 32, out, 32);
    or_hash("transcript-ratchet", r, 64, t->state);
}
static uint64_t rd64(const uint8_t *p) {
    uint64_t v = 0;
    for (int i = 7; i >= 0; i--) v = (v << 8) | p[i];
    return v;
}
/* challenge_fp2: transcript.rs:205-219, squeezing again until both words are below p */
void or_transcript_challenge_fp2(or_transcript *t, const char *label, uint64_t out[2]) {
    for (;;) {
        uint8_t d[32];
        or_transcript_squeeze(t, label, d);
        uint64_t c0 = rd64(d), c1 = rd64(d + 8);
        if (c0 < FP_P && c1 < FP_P) {
            out[0] = c0;
            out[1] = c1;
            return;
        }
    }
}
/* challenge_fp: the first of a squeeze's four words below p (transcript.rs:190-202) */
uint64_t or_transcript_challenge_fp(or_transcript *t, const char *label) {
    for (;;) {
        uint8_t d[32];
        or_transcript_squeeze(t, label, d);
        for (int i = 0; i < 4; i++) {
            uint64_t w = rd64(d + 8 * i);
            if (w < FP_P) return w;
        }
    }
}
/* challenge_indices: words masked to log_n bits, four per squeeze (transcript.rs:221-239) */
void or_transcript_challenge_indices(or_transcript *t, const char *label, uint32_t log_n,
                                     uint32_t count, uint64_t *out) {
    uint64_t mask = log_n >= 64 ? ~0ULL : ((1ULL << log_n) - 1);
    uint32_t have = 0;
    while (have < count) {
        uint8_t d[32];
        or_transcript_squeeze(t, label, d);
        for (int i = 0; i < 4 && have < count; i++) out[have++] = rd64(d + 8 * i) & mask;
    }
}
static uint32_t leading_zero_bits(const uint8_t d[32]) { /* transcript.rs:367-377 */
    uint32_t z = 0;
    for (int i = 0; i < 32; i++) {
        if (d[i]) return z + (uint32_t)__builtin_clz((unsigned)d[i]) - 24;
        z += 8;
    }
    return z;
}
/* pow_meets: H("pow", state || u64 len || label || u64 nonce) starts with `bits` zero bits
 * (transcript.rs:270-292) */
int or_transcript_pow_meets(const or_transcript *t, const char *label, uint32_t bits, uint64_t nonce) {
    size_t n = strlen(label), off;
    uint8_t *buf = (uint8_t *)malloc(48 + n);
    tr_begin(t, label, buf, &off);
    le64(buf + off, nonce);
    uint8_t d[32];
    or_hash("pow", buf, off + 8, d);
    free(buf);
    return leading_zero_bits(d) >= bits;
}
/* grind: the smallest nonce that meets `bits`, then absorbed (transcript.rs:241-250) */
uint64_t or_transcript_grind(or_transcript *t, const char *label, uint32_t bits) {
    uint64_t nonce = 0;
    while (!or_transcript_pow_meets(t, label, bits, nonce)) nonce++;
    uint8_t v[8];
    le64(v, nonce);
    or_transcript_absorb(t, label, v, 8);
    return nonce;
}
/* TCE Vec<Fp2>: crates/tessera-sumcheck/src/transcript.rs:35-44 */
void or_transcript_absorb_fp2s(or_transcript *t, const char *label, const uint64_t *v, size_t count) {
    uint8_t *buf = (uint8_t *)malloc(8 + 16 * count);
    le64(buf, count);
    for (size_t i = 0; i < 2 * count; i++) le64(buf + 8 + 8 * i, v[i]);
    or_transcript_absorb(t, label, buf, 8 + 16 * count);
    free(buf);
}

/* ======================================================================================== */
/* NTT: crates/tessera-pcs/src/ntt.rs                                                        */
/* ======================================================================================== */

#define NTT_LEAF 4096 /* ntt.rs:58 */

static inline size_t rev_bits(size_t i, uint32_t bits) {
    size_t r = 0;
    for (uint32_t b = 0; b < bits; b++) r |= ((i >> b) & 1) << (bits - 1 - b);
    return r;
}
/* bit_reversed_powers: out[t] = scale * base^rev(t), t < 2^bits (ntt.rs:96-115) */
static uint64_t *bit_reversed_powers(uint64_t base, uint32_t bits, uint64_t scale) {
    size_t n = (size_t)1 << bits;
    uint64_t *out = (uint64_t *)malloc(8 * n);
    uint64_t sq[64];
    uint64_t s = base;
    for (uint32_t e = 0; e < bits; e++) {
        sq[e] = s;
        s = fmul(s, s);
    }
    out[0] = scale;
    size_t len = 1;
    for (int e = (int)bits - 1; e >= 0; e--) {
        for (size_t i = 0; i < len; i++) out[len + i] = fmul(out[i], sq[e]);
        len *= 2;
    }
    return out;
}
/* twiddles: Z[t] = ω^rev(t), t < n/2, ω = ω_n or ω_n^-1 (ntt.rs:117-132) */
static uint64_t *twiddles(uint32_t log_n, int inverse) {
    if (log_n == 0) return (uint64_t *)malloc(8);
    uint64_t root = or_root_of_unity(log_n);
    uint64_t base = inverse ? fpow(root, ((uint64_t)1 << log_n) - 1) : root;
    return bit_reversed_powers(base, log_n - 1, 1);
}
/* The Shift of ntt.rs:139-186: subgroup (unit first group), or coset powers s^(2^e). */
typedef struct {
    int coset;
    uint64_t powers[33];
} shift_t;
static shift_t shift_subgroup(void) {
    shift_t s;
    memset(&s, 0, sizeof s);
    return s;
}
static shift_t shift_coset(uint64_t sh) {
    shift_t s;
    s.coset = 1;
    s.powers[0] = sh;
    for (int e = 1; e < 33; e++) s.powers[e] = fmul(s.powers[e - 1], s.powers[e - 1]);
    return s;
}
static inline uint64_t tw_of(const shift_t *s, uint64_t z, uint32_t log_half) {
    return s->coset ? fmul(z, s->powers[log_half]) : z;
}
static inline uint32_t ilog2z(size_t x) { return (uint32_t)__builtin_ctzll((unsigned long long)x); }

/* ct_butterflies (u, v) -> (u + c v, u - c v): ntt.rs:188-209 */
static void ct_bf(uint64_t *lo, uint64_t *hi, size_t h, uint64_t c, int unit) {
    for (size_t i = 0; i < h; i++) {
        uint64_t t = unit ? hi[i] : fmul(hi[i], c);
        hi[i] = fsub(lo[i], t);
        lo[i] = fadd(lo[i], t);
    }
}
/* gs_butterflies (u, v) -> (u + v, c (u - v)): ntt.rs:211-232 */
static void gs_bf(uint64_t *lo, uint64_t *hi, size_t h, uint64_t c, int unit) {
    for (size_t i = 0; i < h; i++) {
        uint64_t a = lo[i], b = hi[i];
        lo[i] = fadd(a, b);
        hi[i] = unit ? fsub(a, b) : fmul(fsub(a, b), c);
    }
}
/* ct_leaf: ntt.rs:262-285 */
static void ct_leaf(uint64_t *v, size_t n, const uint64_t *tw, const shift_t *s, size_t group) {
    size_t half = n / 2, first = group, count = 1;
    while (half > 0) {
        uint32_t lh = ilog2z(half);
        for (size_t g = 0; g < count; g++) {
            int unit = !s->coset && first + g == 0;
            ct_bf(v + 2 * half * g, v + 2 * half * g + half, half, tw_of(s, tw[first + g], lh), unit);
        }
        half /= 2;
        first *= 2;
        count *= 2;
    }
}
/* cooley_tukey / ct_group: ntt.rs:234-260, natural in, bit-reversed out */
static void ct_group(uint64_t *v, size_t n, const uint64_t *tw, const shift_t *s, size_t group) {
    if (n <= NTT_LEAF) {
        ct_leaf(v, n, tw, s, group);
        return;
    }
    size_t half = n / 2;
    int unit = !s->coset && group == 0;
    ct_bf(v, v + half, half, tw_of(s, tw[group], ilog2z(half)), unit);
    ct_group(v, half, tw, s, 2 * group);
    ct_group(v + half, half, tw, s, 2 * group + 1);
}
/* gs_leaf: ntt.rs:318-340 */
static void gs_leaf(uint64_t *v, size_t n, const uint64_t *tw, const shift_t *s, size_t group) {
    size_t half = 1, count = n / 2, first = group * count;
    while (count > 0) {
        uint32_t lh = ilog2z(half);
        for (size_t g = 0; g < count; g++) {
            int unit = !s->coset && first + g == 0;
            gs_bf(v + 2 * half * g, v + 2 * half * g + half, half, tw_of(s, tw[first + g], lh), unit);
        }
        half *= 2;
        first /= 2;
        count /= 2;
    }
}
/* gentleman_sande / gs_group: ntt.rs:287-316, bit-reversed in, natural out */
static void gs_group(uint64_t *v, size_t n, const uint64_t *tw, const shift_t *s, size_t group) {
    if (n <= NTT_LEAF) {
        gs_leaf(v, n, tw, s, group);
        return;
    }
    size_t half = n / 2;
    gs_group(v, half, tw, s, 2 * group);
    gs_group(v + half, half, tw, s, 2 * group + 1);
    int unit = !s->coset && group == 0;
    gs_bf(v, v + half, half, tw_of(s, tw[group], ilog2z(half)), unit);
}
/* bit_reverse_scaled (ntt.rs:349-395), the plain swap form */
static void bit_reverse_scaled(uint64_t *v, uint32_t bits, int has_scale, uint64_t scale) {
    size_t n = (size_t)1 << bits;
    for (size_t i = 0; i < n; i++) {
        size_t j = rev_bits(i, bits);
        if (i < j) {
            uint64_t x = v[i], y = v[j];
            v[i] = has_scale ? fmul(y, scale) : y;
            v[j] = has_scale ? fmul(x, scale) : x;
        } else if (i == j && has_scale) {
            v[i] = fmul(v[i], scale);
        }
    }
}
static uint64_t inverse_of_power_of_two(uint32_t log_n) { /* ntt.rs:134-137 */
    return fpow(FP_P / 2 + 1, log_n);
}
/* NttPlan::{ntt,intt,coset_ntt,coset_intt}: ntt.rs:461-516 */
void or_ntt(uint64_t *v, uint32_t log_n) {
    uint64_t *tw = twiddles(log_n, 0);
    shift_t s = shift_subgroup();
    ct_group(v, (size_t)1 << log_n, tw, &s, 0);
    bit_reverse_scaled(v, log_n, 0, 0);
    free(tw);
}
void or_intt(uint64_t *v, uint32_t log_n) {
    uint64_t *tw = twiddles(log_n, 1);
    shift_t s = shift_subgroup();
    bit_reverse_scaled(v, log_n, 1, inverse_of_power_of_two(log_n));
    gs_group(v, (size_t)1 << log_n, tw, &s, 0);
    free(tw);
}
void or_coset_ntt(uint64_t *v, uint32_t log_n, uint64_t shift) {
    uint64_t *tw = twiddles(log_n, 0);
    shift_t s = shift_coset(shift);
    ct_group(v, (size_t)1 << log_n, tw, &s, 0);
    bit_reverse_scaled(v, log_n, 0, 0);
    free(tw);
}
void or_coset_intt(uint64_t *v, uint32_t log_n, uint64_t shift) {
    uint64_t *tw = twiddles(log_n, 1);
    shift_t s = shift_coset(finv(shift));
    bit_reverse_scaled(v, log_n, 1, inverse_of_power_of_two(log_n));
    gs_group(v, (size_t)1 << log_n, tw, &s, 0);
    free(tw);
}

/* ======================================================================================== */
/* RowEncoder: crates/tessera-pcs/src/encoding.rs:126-161 (tables), 292-313 (encode),        */
/* 323-340 (spread)                                                                          */
/* ======================================================================================== */

typedef struct {
    uint32_t log_k, log_r, P;
    uint64_t *inverse, *forward, *spread, shift_pow_k;
    const uint64_t *rows, *masks;
    uint64_t *codewords;
} enc_ctx;

static void encode_one(const enc_ctx *e, const uint64_t *row, const uint64_t *mask, uint64_t *cw) {
    size_t k = (size_t)1 << e->log_k, n = k << e->log_r, stride = (size_t)1 << e->log_r;
    shift_t sub = shift_subgroup();
    /* 1. k f in bit-reversed order, in the first k positions */
    memcpy(cw, row, 8 * k);
    ct_group(cw, k, e->inverse, &sub, 0);
    /* 2. spread, top down: position stride*t receives entry t times 7^rev(t)/k */
    for (size_t t = k; t-- > 0;) {
        uint64_t y = fmul(cw[t], e->spread[t]);
        for (size_t z = 1; z < stride; z++) cw[stride * t + z] = 0;
        cw[stride * t] = y;
    }
    /* 3. the mask */
    uint64_t power = 1;
    for (uint32_t i = 0; i < e->P; i++) {
        uint64_t scaled = fmul(mask[i], power);
        size_t low = stride * rev_bits(i, e->log_k);
        cw[low] = fsub(cw[low], scaled);
        cw[low + stride / 2] = fmul(scaled, e->shift_pow_k);
        power = fmul(power, 7);
    }
    /* 4. the values of g at 7 ω_n^j, natural order */
    gs_group(cw, n, e->forward, &sub, 0);
}
static void enc_range(void *c, size_t lo, size_t hi) {
    enc_ctx *e = (enc_ctx *)c;
    size_t k = (size_t)1 << e->log_k, n = k << e->log_r;
    for (size_t r = lo; r < hi; r++)
        encode_one(e, e->rows + r * k, e->masks ? e->masks + r * e->P : NULL, e->codewords + r * n);
}
int or_encode_rows(uint32_t log_k, uint32_t log_r, uint32_t P, const uint64_t *rows, size_t nrows,
                   const uint64_t *masks, uint64_t *codewords, int threads) {
    if (log_r == 0 || log_k + log_r > 32 || P > (1u << log_k)) return -1;
    enc_ctx e = {log_k, log_r, P, NULL, NULL, NULL, 0, rows, masks, codewords};
    e.forward = twiddles(log_k + log_r, 0);
    e.inverse = twiddles(log_k, 1);
    e.spread = bit_reversed_powers(7, log_k, inverse_of_power_of_two(log_k));
    e.shift_pow_k = fpow(7, (uint64_t)1 << log_k);
    parallel_for(nrows, threads, enc_range, &e);
    free(e.forward);
    free(e.inverse);
    free(e.spread);
    return 0;
}

/* ======================================================================================== */
/* Commitments: crates/tessera-pcs/src/commitment.rs:343-458, streaming.rs:382-438          */
/* ======================================================================================== */

/* from_encoded's per-segment chains (commitment.rs:425-437): blocks of B rows of n symbols. */
void or_segment_chains(const uint8_t id[32], uint64_t n, uint32_t row_block,
                       const uint64_t *codewords, size_t nrows, uint8_t *chains, int threads) {
    or_column_init(id, n, chains, threads);
    for (size_t r = 0; r < nrows; r += row_block) {
        size_t count = nrows - r < row_block ? nrows - r : row_block;
        or_column_absorb(chains, n, codewords + r * n, count, threads);
    }
}
int or_commit_unmasked(uint32_t log_k, uint32_t log_r, uint32_t row_block, const uint8_t id[32],
                       const uint64_t *rows, size_t npolys, uint64_t *codewords, uint8_t *leaves,
                       uint8_t root[32], int threads) {
    size_t n = (size_t)1 << (log_k + log_r);
    if (row_block == 0) return -1;
    uint64_t *cw = codewords ? codewords : (uint64_t *)malloc(8 * n * (npolys ? npolys : 1));
    int rc = or_encode_rows(log_k, log_r, 0, rows, npolys, NULL, cw, threads);
    if (rc == 0) {
        or_segment_chains(id, n, row_block, cw, npolys, leaves, threads);
        or_merkle_root(leaves, n, root, threads);
    }
    if (!codewords) free(cw);
    return rc;
}
/* merge_segments + merged_column: streaming.rs:382-404, 432-438 */
void or_merge_segments(const uint8_t *seg, size_t S, uint64_t n, uint8_t *leaves, uint8_t root[32]) {
    dom d = dom_new("column-merge");
    uint8_t *in = (uint8_t *)malloc(32 * (S ? S : 1));
    for (uint64_t j = 0; j < n; j++) {
        for (size_t s = 0; s < S; s++) memcpy(in + 32 * s, seg + 32 * (s * n + j), 32);
        dom_hash(&d, in, 32 * S, leaves + 32 * j);
    }
    free(in);
    or_merkle_root(leaves, n, root, 1);
}

/* ======================================================================================== */
/* Sumcheck: crates/tessera-sumcheck/src/prover.rs:1122-1421 (prove_batch, prove_checked),   */
/* kernel.rs:90-101 (line), 292-355 (product_sums), 591-633 (bind)                           */
/* ======================================================================================== */

typedef struct {
    int is_ext; /* the working table: base words until the first bind */
    uint64_t *base;
    fp2 *ext;
    int is_public;
} wtable;

/* Σ_x Π_k T_k[x] over an instance's whole hypercube, in Fp2. */
static fp2 instance_sum(const or_instance *in) {
    size_t len = (size_t)1 << in->vars;
    fp2 acc = E_ZERO;
    for (size_t x = 0; x < len; x++) {
        fp2 p = E_ONE;
        for (int k = 0; k < in->ntables; k++) {
            const or_table *t = &in->tables[k];
            fp2 v = t->is_ext ? (fp2){t->values[2 * x], t->values[2 * x + 1]} : e_lift(t->values[x]);
            p = e_mul(p, v);
        }
        acc = e_add(acc, p);
    }
    return acc;
}

int or_prove_batch(or_transcript *t, const char *prefix, int degree, const or_instance *inst,
                   int ninst, uint64_t *gamma_out, uint64_t *rounds, uint64_t *challenges,
                   uint64_t *final_evals, size_t *n_evals) {
    /* check_batch: prover.rs:1196-1218 */
    if (degree < 1 || degree > 7) return -1;
    if (ninst < 1) return -2;
    int n_max = 0;
    for (int i = 0; i < ninst; i++) {
        if (inst[i].ntables < 1 || inst[i].ntables > degree) return -3;
        if (inst[i].vars < 0 || inst[i].vars > 40) return -4;
        if (inst[i].vars > n_max) n_max = inst[i].vars;
    }
    char label[256];
    snprintf(label, sizeof label, "%s/gamma", prefix);
    uint64_t g[2];
    or_transcript_challenge_fp2(t, label, g);
    fp2 gamma = {g[0], g[1]};
    gamma_out[0] = g[0];
    gamma_out[1] = g[1];

    /* weights γ^i and working tables */
    fp2 *w = (fp2 *)malloc(sizeof(fp2) * ninst);
    fp2 *padsum = (fp2 *)malloc(sizeof(fp2) * ninst);
    wtable **tabs = (wtable **)malloc(sizeof(wtable *) * ninst);
    fp2 acc = E_ONE;
    for (int i = 0; i < ninst; i++) {
        w[i] = acc;
        acc = e_mul(acc, gamma);
        size_t len = (size_t)1 << inst[i].vars;
        tabs[i] = (wtable *)calloc(inst[i].ntables, sizeof(wtable));
        for (int k = 0; k < inst[i].ntables; k++) {
            const or_table *src = &inst[i].tables[k];
            wtable *d = &tabs[i][k];
            d->is_public = src->is_public;
            d->is_ext = src->is_ext;
            if (src->is_ext) {
                d->ext = (fp2 *)malloc(sizeof(fp2) * len);
                memcpy(d->ext, src->values, 16 * len);
            } else {
                d->base = (uint64_t *)malloc(8 * len);
                memcpy(d->base, src->values, 8 * len);
            }
        }
        padsum[i] = inst[i].vars < n_max ? instance_sum(&inst[i]) : E_ZERO;
    }

    fp2 nodes_val[8];
    for (int j = 0; j < n_max; j++) {
        fp2 msg[8];
        for (int d = 0; d < degree; d++) msg[d] = E_ZERO;
        for (int i = 0; i < ninst; i++) {
            int pad = n_max - inst[i].vars;
            if (j < pad) {
                /* a padding round: 2^(pad - j - 1) S_i at every node (prover.rs:1414-1421) */
                fp2 v = e_mul(w[i], e_scale(padsum[i], (uint64_t)1 << (pad - j - 1)));
                for (int d = 0; d < degree; d++) msg[d] = e_add(msg[d], v);
                continue;
            }
            size_t half = (size_t)1 << (inst[i].vars - (j - pad) - 1);
            int nt = inst[i].ntables;
            int all_base = 1;
            for (int k = 0; k < nt; k++) all_base &= !tabs[i][k].is_ext;
            for (int d = 0; d < degree; d++) nodes_val[d] = E_ZERO;
            if (all_base) {
                /* the first own round in the prime subfield, lifted once (kernel.rs:292-355) */
                uint64_t sums[8] = {0};
                for (size_t p = 0; p < half; p++) {
                    for (int d = 0; d < degree; d++) {
                        uint64_t x = d == 0 ? 0 : (uint64_t)(d + 1), prod = 1;
                        for (int k = 0; k < nt; k++) {
                            uint64_t a = tabs[i][k].base[2 * p], b = tabs[i][k].base[2 * p + 1];
                            prod = fmul(prod, fadd(a, fmul(x, fsub(b, a))));
                        }
                        sums[d] = fadd(sums[d], prod);
                    }
                }
                for (int d = 0; d < degree; d++) nodes_val[d] = e_lift(sums[d]);
            } else {
                for (size_t p = 0; p < half; p++) {
                    for (int d = 0; d < degree; d++) {
                        uint64_t x = d == 0 ? 0 : (uint64_t)(d + 1);
                        fp2 prod = E_ONE;
                        for (int k = 0; k < nt; k++) {
                            fp2 a, b;
                            if (tabs[i][k].is_ext) {
                                a = tabs[i][k].ext[2 * p];
                                b = tabs[i][k].ext[2 * p + 1];
                            } else {
                                a = e_lift(tabs[i][k].base[2 * p]);
                                b = e_lift(tabs[i][k].base[2 * p + 1]);
                            }
                            prod = e_mul(prod, e_add(a, e_scale(e_sub(b, a), x)));
                        }
                        nodes_val[d] = e_add(nodes_val[d], prod);
                    }
                }
            }
            for (int d = 0; d < degree; d++) msg[d] = e_add(msg[d], e_mul(w[i], nodes_val[d]));
        }
        uint64_t words[16];
        for (int d = 0; d < degree; d++) {
            words[2 * d] = msg[d].c0;
            words[2 * d + 1] = msg[d].c1;
            rounds[(size_t)j * 2 * degree + 2 * d] = msg[d].c0;
            rounds[(size_t)j * 2 * degree + 2 * d + 1] = msg[d].c1;
        }
        snprintf(label, sizeof label, "%s/round/%d", prefix, j);
        or_transcript_absorb_fp2s(t, label, words, (size_t)degree);
        snprintf(label, sizeof label, "%s/r/%d", prefix, j);
        uint64_t rr[2];
        or_transcript_challenge_fp2(t, label, rr);
        challenges[2 * j] = rr[0];
        challenges[2 * j + 1] = rr[1];
        fp2 r = {rr[0], rr[1]};
        /* bind: t'[i] = t[2i] + r (t[2i+1] - t[2i]) (kernel.rs:591-633) */
        for (int i = 0; i < ninst; i++) {
            int pad = n_max - inst[i].vars;
            if (j < pad) continue;
            size_t half = (size_t)1 << (inst[i].vars - (j - pad) - 1);
            for (int k = 0; k < inst[i].ntables; k++) {
                wtable *tb = &tabs[i][k];
                if (!tb->is_ext) {
                    fp2 *e = (fp2 *)malloc(sizeof(fp2) * (half ? half : 1));
                    for (size_t p = 0; p < half; p++) {
                        uint64_t a = tb->base[2 * p], diff = fsub(tb->base[2 * p + 1], a);
                        e[p] = (fp2){fadd(a, fmul(r.c0, diff)), fmul(r.c1, diff)};
                    }
                    free(tb->base);
                    tb->base = NULL;
                    tb->ext = e;
                    tb->is_ext = 1;
                } else {
                    for (size_t p = 0; p < half; p++) {
                        fp2 a = tb->ext[2 * p], b = tb->ext[2 * p + 1];
                        tb->ext[p] = e_add(a, e_mul(r, e_sub(b, a)));
                    }
                }
            }
        }
    }
    /* final evaluations, instance by instance, public factors left out (prover.rs:1387-1399) */
    size_t ne = 0;
    for (int i = 0; i < ninst; i++) {
        for (int k = 0; k < inst[i].ntables; k++) {
            wtable *tb = &tabs[i][k];
            if (tb->is_public) continue;
            fp2 v = tb->is_ext ? tb->ext[0] : e_lift(tb->base[0]);
            final_evals[2 * ne] = v.c0;
            final_evals[2 * ne + 1] = v.c1;
            ne++;
        }
    }
    snprintf(label, sizeof label, "%s/evals", prefix);
    or_transcript_absorb_fp2s(t, label, final_evals, ne);
    *n_evals = ne;
    for (int i = 0; i < ninst; i++) {
        for (int k = 0; k < inst[i].ntables; k++) {
            free(tabs[i][k].base);
            free(tabs[i][k].ext);
        }
        free(tabs[i]);
    }
    free(tabs);
    free(w);
    free(padsum);
    return 0;
}

/* ======================================================================================== */
/* Tree-level rounds: crates/tessera-sumcheck/src/offload.rs:27-48 (DeviceLevel contract)    */
/* ======================================================================================== */

void or_level_sums(int shape, const uint64_t lambda[2], const uint64_t *const *tables, size_t len,
                   const uint64_t *low, const uint64_t *high, uint32_t low_bits, uint64_t out[6]) {
    fp2 s[3] = {E_ZERO, E_ZERO, E_ZERO};
    fp2 lam = {lambda[0], lambda[1]};
    int nt = shape == 0 ? 4 : 2;
    size_t mask = ((size_t)1 << low_bits) - 1;
    for (size_t p = 0; p < len / 2; p++) {
        fp2 wl = {low[2 * (p & mask)], low[2 * (p & mask) + 1]};
        size_t hi = p >> low_bits;
        fp2 wh = {high[2 * hi], high[2 * hi + 1]};
        fp2 w = e_mul(wl, wh);
        for (int xi = 0; xi < 3; xi++) {
            uint64_t x = xi == 0 ? 0 : (uint64_t)(xi + 1);
            fp2 v[4];
            for (int k = 0; k < nt; k++) {
                fp2 a = {tables[k][4 * p], tables[k][4 * p + 1]};
                fp2 b = {tables[k][4 * p + 2], tables[k][4 * p + 3]};
                v[k] = e_add(a, e_scale(e_sub(b, a), x));
            }
            fp2 val;
            if (shape == 0)
                val = e_add(e_add(e_mul(v[0], v[3]), e_mul(v[1], v[2])), e_mul(lam, e_mul(v[2], v[3])));
            else
                val = e_mul(v[0], v[1]);
            s[xi] = e_add(s[xi], e_mul(w, val));
        }
    }
    for (int i = 0; i < 3; i++) {
        out[2 * i] = s[i].c0;
        out[2 * i + 1] = s[i].c1;
    }
}
void or_level_bind(uint64_t *const *tables, int ntables, size_t len, const uint64_t r[2]) {
    fp2 rr = {r[0], r[1]};
    for (int k = 0; k < ntables; k++) {
        fp2 *t = (fp2 *)tables[k];
        for (size_t i = 0; i < len / 2; i++) t[i] = e_add(t[2 * i], e_mul(rr, e_sub(t[2 * i + 1], t[2 * i])));
    }
}

/* ======================================================================================== */
/* SplitMix64 inputs: crates/tessera-bench/benches/primitives.rs:52-69                       */
/* ======================================================================================== */

void or_splitmix_fill(uint64_t seed, uint64_t *out, size_t n) {
    uint64_t s = seed;
    for (size_t i = 0; i < n; i++) {
        s += 0x9E3779B97F4A7C15ULL;
        uint64_t z = s;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
        out[i] = canon(z ^ (z >> 31));
    }
}

/* ---- multilinear extension at a point (verifier side) ---------------------------------- */
/* Σ_x values[x]·eq(point, x) over x < 2^log_n, x_1 the index's lowest bit: the eq table is built
 * one coordinate at a time (eq over the first t coordinates doubled by (1 − r_t, r_t)), then one
 * dot product — not the prover's variable-by-variable binding. values: prime-field words
 * (is_ext = 0) or interleaved Fp2 pairs (is_ext = 1); point: log_n Fp2 pairs. */
void or_mle(const uint64_t *values, int is_ext, uint32_t log_n, const uint64_t *point, uint64_t out[2]) {
    const size_t n = (size_t)1 << log_n;
    fp2 *eqt = (fp2 *)malloc(n * sizeof(fp2));
    eqt[0] = E_ONE;
    for (uint32_t t = 0; t < log_n; t++) {
        const fp2 r = {point[2 * t], point[2 * t + 1]};
        const fp2 one_minus = e_sub(E_ONE, r);
        const size_t half = (size_t)1 << t;
        for (size_t x = 0; x < half; x++) {
            const fp2 e = eqt[x];
            eqt[x + half] = e_mul(e, r);
            eqt[x] = e_mul(e, one_minus);
        }
    }
    fp2 acc = E_ZERO;
    for (size_t x = 0; x < n; x++) {
        const fp2 v = is_ext ? (fp2){values[2 * x], values[2 * x + 1]} : e_lift(values[x]);
        acc = e_add(acc, e_mul(v, eqt[x]));
    }
    free(eqt);
    out[0] = acc.c0;
    out[1] = acc.c1;
}
