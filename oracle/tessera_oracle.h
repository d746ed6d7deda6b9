/* SPDX-License-Identifier: Apache-2.0 OR MIT
 *
 * TEST INFRASTRUCTURE ONLY. The CPU oracle of the Tessera proving hot path: a plain-C
 * restatement of the reference's Rust algorithms (tessera-field, tessera-pcs, tessera-hash,
 * tessera-sumcheck), used by the test suite as the checker of the CUDA path and by the
 * benchmark as the timed CPU baseline. Nothing in the product library links or calls it.
 *
 * Parity is pinned: the oracle reproduces the reference's golden vectors (spec/vectors/
 * {field,encoding,hash,blake3,transcript,sumcheck,pcs-streaming}) byte for byte; the committed
 * fixtures under tests/golden/ carry those vectors.
 *
 * Conventions: an Fp element is a canonical uint64_t in [0, p); an Fp2 element is two
 * consecutive words (c0, c1) for c0 + c1*X, X^2 = 7; digests are 32 bytes.
 */
#ifndef TESSERA_ORACLE_H
#define TESSERA_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- field (tessera-field/src/goldilocks.rs, ext2.rs) ---------------------------------- */
uint64_t or_fp_add(uint64_t a, uint64_t b);
uint64_t or_fp_sub(uint64_t a, uint64_t b);
uint64_t or_fp_mul(uint64_t a, uint64_t b);
uint64_t or_fp_pow(uint64_t a, uint64_t e);
uint64_t or_fp_inv(uint64_t a);
uint64_t or_fp_reduce(uint64_t x);
/* ω_{2^log_n} = 7^((p-1)/2^log_n) */
uint64_t or_root_of_unity(uint32_t log_n);
void or_fp2_mul(const uint64_t a[2], const uint64_t b[2], uint64_t out[2]);
void or_fp2_inv(const uint64_t a[2], uint64_t out[2]);
/* Batch element-wise ops over n values, for vector tests. op: 0 add, 1 sub, 2 mul. */
void or_fp_vec(int op, const uint64_t *a, const uint64_t *b, uint64_t *out, size_t n);
void or_fp2_vec_mul(const uint64_t *a, const uint64_t *b, uint64_t *out, size_t n);

/* ---- BLAKE3 (full tree mode, from the public specification) ---------------------------- */
/* mode: 0 hash, 1 keyed (key 32 B), 2 derive-key (key = NUL-terminated context string). */
void or_blake3(int mode, const void *key, const uint8_t *in, size_t len, uint8_t *out, size_t out_len);
/* H(domain, bytes): BLAKE3 derive-key with context "tessera/v1/<name>" (tessera-hash/src/domain.rs). */
void or_context_key(const char *name, uint8_t key[32]);
void or_hash(const char *name, const uint8_t *in, size_t len, uint8_t out[32]);

/* ---- column chains and Merkle (tessera-hash/src/columns.rs, merkle.rs) ---------------- */
void or_column_init(const uint8_t id[32], uint64_t ncols, uint8_t *chains, int threads);
/* Absorbs `count` rows (row-major, count x ncols symbols) as one block. */
void or_column_absorb(uint8_t *chains, uint64_t ncols, const uint64_t *rows, size_t count, int threads);
/* All 2n-1 nodes, leaves first, root last (tessera-hash/src/merkle.rs:93). */
void or_merkle_tree(const uint8_t *leaves, size_t n, uint8_t *nodes, int threads);
void or_merkle_root(const uint8_t *leaves, size_t n, uint8_t root[32], int threads);
void or_merkle_node(const uint8_t l[32], const uint8_t r[32], uint8_t out[32]);

/* ---- transcript (tessera-hash/src/transcript.rs) -------------------------------------- */
typedef struct {
    uint8_t state[32];
    uint64_t counter;
} or_transcript;
void or_transcript_init(or_transcript *t, const uint8_t *context_tce, size_t len);
void or_transcript_absorb(or_transcript *t, const char *label, const uint8_t *value, size_t len);
void or_transcript_squeeze(or_transcript *t, const char *label, uint8_t out[32]);
void or_transcript_challenge_fp2(or_transcript *t, const char *label, uint64_t out[2]);
uint64_t or_transcript_challenge_fp(or_transcript *t, const char *label);
void or_transcript_challenge_indices(or_transcript *t, const char *label, uint32_t log_n,
                                     uint32_t count, uint64_t *out);
int or_transcript_pow_meets(const or_transcript *t, const char *label, uint32_t bits, uint64_t nonce);
uint64_t or_transcript_grind(or_transcript *t, const char *label, uint32_t bits);
/* Absorbs TCE Vec<Fp2>: u64 length, then c0, c1 of each element. */
void or_transcript_absorb_fp2s(or_transcript *t, const char *label, const uint64_t *values, size_t count);

/* ---- NTT and encoding (tessera-pcs/src/ntt.rs, encoding.rs) --------------------------- */
void or_ntt(uint64_t *values, uint32_t log_n);              /* f(ω^j), natural order both sides */
void or_intt(uint64_t *values, uint32_t log_n);
void or_coset_ntt(uint64_t *values, uint32_t log_n, uint64_t shift);
void or_coset_intt(uint64_t *values, uint32_t log_n, uint64_t shift);
/* RowEncoder::encode_rows: nrows rows of k values -> nrows codewords of n = 2^r k symbols,
 * masks: nrows x P coefficients (m_0 first). Rows are encoded in parallel over `threads`. */
int or_encode_rows(uint32_t log_k, uint32_t log_inv_rate, uint32_t mask_coeffs,
                   const uint64_t *rows, size_t nrows, const uint64_t *masks,
                   uint64_t *codewords, int threads);
/* ReferenceCommitment::commit_unmasked: codewords (npolys x n, may be NULL), leaves (n x 32),
 * root. */
int or_commit_unmasked(uint32_t log_k, uint32_t log_inv_rate, uint32_t row_block,
                       const uint8_t id[32], const uint64_t *rows, size_t npolys,
                       uint64_t *codewords, uint8_t *leaves, uint8_t root[32], int threads);
/* Column chains of one segment from its codewords (blocks of B rows). */
void or_segment_chains(const uint8_t id[32], uint64_t n, uint32_t row_block,
                       const uint64_t *codewords, size_t nrows, uint8_t *chains, int threads);
/* merge_segments: leaves_j = H("column-merge", d_j^(1..S)), then the Merkle root. */
void or_merge_segments(const uint8_t *segment_chains, size_t nsegments, uint64_t n,
                       uint8_t *leaves, uint8_t root[32]);

/* ---- sumcheck (tessera-sumcheck/src/prover.rs) ---------------------------------------- */
typedef struct {
    const uint64_t *values; /* 2^vars entries: words (base) or pairs of words (ext) */
    int is_ext;
    int is_public;
} or_table;
typedef struct {
    const or_table *tables;
    int ntables;
    int vars;
} or_instance;
/* prove_batch for product instances. Outputs: gamma[2]; rounds: n_max x degree Fp2 (p(0),
 * p(2..d)); challenges: n_max Fp2; final_evals: Fp2 list (count written to *n_evals).
 * Returns 0, or a negative code for a refused batch (nothing absorbed). */
int or_prove_batch(or_transcript *t, const char *prefix, int degree, const or_instance *inst,
                   int ninst, uint64_t *gamma, uint64_t *rounds, uint64_t *challenges,
                   uint64_t *final_evals, size_t *n_evals);

/* ---- tree-level rounds (tessera-sumcheck/src/offload.rs DeviceLevel) ------------------ */
/* shape 0: fraction N0 D1 + N1 D0 + λ D0 D1 over 4 tables; shape 1: product V0 V1 over 2.
 * tables: ntables pointers to len Fp2 entries. out: 3 Fp2 (x = 0, 2, 3). */
void or_level_sums(int shape, const uint64_t lambda[2], const uint64_t *const *tables, size_t len,
                   const uint64_t *low, const uint64_t *high, uint32_t low_bits, uint64_t out[6]);
void or_level_bind(uint64_t *const *tables, int ntables, size_t len, const uint64_t r[2]);

/* ---- multilinear extension Σ_x values[x]·eq(point, x) (eq table, then one dot product) ---- */
void or_mle(const uint64_t *values, int is_ext, uint32_t log_n, const uint64_t *point, uint64_t out[2]);

/* ---- synthetic inputs (tessera-bench/benches/primitives.rs:52-69) --------------------- */
void or_splitmix_fill(uint64_t seed, uint64_t *out, size_t n); /* from_u64_reduced of each */

#ifdef __cplusplus
}
#endif
#endif
