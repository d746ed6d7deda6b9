/* SPDX-License-Identifier: Apache-2.0 OR MIT
 *
 * libtessera_gb300: the GB300 (sm_103a) proving hot path of Tessera behind a C ABI.
 *
 * The entry points replace the device seams of the reference prover (AbdelStark/tessera);
 * each declaration cites the reference interface it stands in for. Field elements are
 * canonical Goldilocks words (uint64_t in [0, p), p = 2^64 - 2^32 + 1, little-endian in memory
 * as the reference's repr(transparent) Goldilocks); an Fp2 element is two words (c0, c1) for
 * c0 + c1 X, X^2 = 7, laid out as the reference's repr(C) QuadraticExt; digests are 32 bytes.
 * Matrices are row-major by polynomial: row r (one polynomial of k values) at rows + r*k, its
 * codeword at codewords + r*n.
 *
 * Every function returns TG_OK (0) or a negative status, with the reason in tg_last_error()
 * (per thread). "_dev" entry points take device pointers and an optional cudaStream_t (NULL:
 * the device handle's own stream) and return once the work is queued; the others take host
 * memory and return when the results are in it. A handle may be used from one thread at a
 * time unless its comment says otherwise.
 */
#ifndef TESSERA_GB300_H
#define TESSERA_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    TG_OK = 0,
    TG_DECLINED = 1,        /* an offload declined the work (the host does it) */
    TG_ERR_INVALID = -1,    /* a shape or argument the reference would refuse */
    TG_ERR_CUDA = -2,       /* a CUDA call failed */
    TG_ERR_NOMEM = -3,      /* device memory exhausted */
    TG_ERR_STATE = -4,      /* a call out of order (absorb after finish, after a short block) */
};

typedef struct tg_device tg_device;
typedef struct tg_sink tg_sink;
typedef struct tg_matrix tg_matrix;
typedef struct tg_level tg_level;

/* Device configuration; zero fields take their defaults. The level fields are the reference's
 * TESSERA_GPU_LEVEL_GIB / TESSERA_GPU_LEVEL_MIN (crates/tessera-prover/src/gpu.rs:121-134). */
typedef struct {
    uint64_t level_budget_bytes; /* default 16 GiB */
    uint64_t level_min_entries;  /* default 2^14 (gpu.rs:89 LEVEL_MIN_ENTRIES) */
    uint64_t lde_group_bytes;    /* encoder scratch per group of rows; default 768 MiB */
    uint64_t tree_flags;         /* TG_TREE_* below; default 0 */
} tg_config;

/* Tree levels: sum each round's q(1) on the device and use it, instead of deriving q(1) from the
 * round's claim (the reference prover's derivation, crates/tessera-sumcheck/src/level.rs:317-347).
 * The proof is the same either way; the summing path is otherwise taken only where a point
 * coordinate is 0, so this flag exists to check it. Slower. */
#define TG_TREE_SUM_Q1 1u

/* Library version, and the message of the calling thread's last failure. */
int tg_version(void);
const char *tg_last_error(void);

/* Opens one GPU (replaces Gpu::open / Device::new, crates/tessera-prover/src/gpu.rs:111-146,
 * crates/tessera-gpu/src/device.rs:125-146). */
int tg_device_open(int ordinal, const tg_config *cfg, tg_device **out);
int tg_device_close(tg_device *dev);
int tg_device_sync(tg_device *dev);
/* The handle's own CUDA stream (a cudaStream_t), where calls given a NULL stream run. */
int tg_device_stream(tg_device *dev, void **stream);
/* Kernels launched through this handle so far (the library's own, counted at launch). */
int tg_device_launches(tg_device *dev, uint64_t *launches);
/* Returns the workspace memory that closed leaf stages left for reuse (levels and bound tables,
 * pooled as the reference's ForestWorkspace is, crates/tessera-gpu/src/trees.rs:124-160) to the
 * driver, zeroed first. tg_device_close does the same. */
int tg_device_trim(tg_device *dev);

/* Reads one byte of every page of a host buffer on the calling thread. On the GB300's Arm host a
 * copy to the device from host memory that the CPU has not read or written for some seconds can
 * run at a small fraction of the link's speed (measured: 64 MiB requests at 7-13 GB/s instead of
 * about 190 GB/s); reading its pages first restores the full speed, for well under a millisecond
 * per 64 MiB. The proof server does this for each request's rows and tables on submission. */
int tg_host_prefault(const void *p, size_t bytes);

/* Integer-pipe peaks of the device, measured with register-only microbenchmarks (no reference
 * counterpart: these are the denominators of the integer-bound kernels' rooflines). Rates per
 * second over the whole GPU: mad.wide.u32 operations, Goldilocks products, radix-2 butterflies
 * inside radix-32 shift-twiddle transforms, and BLAKE3 compressions. Takes about 0.1 s. */
typedef struct tg_int_peaks {
    double imad_wide_per_s;
    double mulmod_per_s;
    double butterflies_per_s;
    double blake3_compressions_per_s;
} tg_int_peaks;
int tg_measure_int_peaks(tg_device *dev, tg_int_peaks *out);

/* Self-check of the device's lazy Goldilocks arithmetic, the field code of the hot kernels (no
 * reference counterpart; its results are checked against exact integer arithmetic). Inputs are any
 * 64-bit words, standing for their value mod p. For i < n, with a = words[i], b = words[(i+1) % n],
 * c = words[(i+2) % n], d = words[(i+3) % n], out[TG_LAZY_CHECK_OUTS·i + t] is the canonical value
 * of: t = 0 a + b; 1 a − b; 2 a·b; 3 7·a; 4 a·2^5; 5 a·2^40; 6 a·2^70; 7 a·b + c·d as one unreduced
 * sum; 8 a + b·c + d·a, a sum seeded with a word; 9–10 (a + bX)(c + dX) in Fp2 = Fp[X]/(X^2 − 7);
 * 11–12 (a + bX) + (c + dX)(b + aX); 13–14 (a + bX)(c + dX) + (b + dX)(a + cX); 15
 * Σ_{k<64} words[(i+k) % n]·words[(i+2k+1) % n] as one unreduced sum. n ≥ 4; host buffers. */
#define TG_LAZY_CHECK_OUTS 16
int tg_check_lazy_arith(tg_device *dev, const uint64_t *words, size_t n, uint64_t *out);
/* A self-check of the bounded meetings between the persistent sumcheck rounds' blocks: `blocks`
 * co-resident blocks (at most one per SM) meet `meetings` times, except block `absent` (-1: none),
 * which leaves first; the others then give up after `polls` polls each (at least 256) instead of
 * waiting for it. *met = the blocks that met every time, *gave_up = whether the meeting point
 * recorded a give-up. */
int tg_check_grid_meet(tg_device *dev, int blocks, int meetings, int absent, uint32_t polls, int *met, int *gave_up);

/* Synthetic inputs on the device (no reference counterpart; the reference benchmark draws the
 * same words on the host, crates/tessera-bench/benches/primitives.rs:52-69): out[i] is the
 * (i + 1)-th SplitMix64 output from `seed`, reduced once below p. Enqueued on `stream` (NULL:
 * the device's stream). */
int tg_fill_splitmix(tg_device *dev, uint64_t *out, size_t n, uint64_t seed, void *stream);
/* Replaces Device::fill_counter (crates/tessera-gpu/src/commit.rs:401-414): out[i] = counter(base + i),
 * counter(c) the SplitMix64 output for state (c + 1)·0x9E3779B97F4A7C15 reduced once below p. */
int tg_fill_counter(tg_device *dev, uint64_t *out, size_t n, uint64_t base, void *stream);
/* Per-kernel timing (no counterpart in the reference; its GPU timing lives in benchmark
 * harnesses, crates/tessera-bench/examples/gpu_unit_costs.rs): while enabled, every launch is
 * bracketed by CUDA events on its own stream. tg_profile_read sums the elapsed times by kernel
 * name since the last read: names come newline-separated in `names`; ms, launches and units
 * (work items) fill the first `cap` entries; *count is the number of kernels seen. */
int tg_profile_enable(tg_device *dev, int on);
int tg_profile_read(tg_device *dev, char *names, size_t names_len, double *ms, uint64_t *launches, uint64_t *units,
                    size_t cap, size_t *count);

/* ---- Reed–Solomon encoding: RowEncoder::encode_rows (crates/tessera-pcs/src/encoding.rs:257)
 * nrows rows of k = 2^log_k values -> codewords of n = 2^(log_k + log_inv_rate) symbols,
 * symbol j = g(7 ω_n^j), g = f + (X^k - 1) m, masks: nrows x mask_coeffs (m_0 first) or NULL
 * for mask_coeffs = 0. 1 <= log_inv_rate <= 4, log_k <= 24, mask_coeffs <= k. */
int tg_encode_rows_dev(tg_device *dev, uint32_t log_k, uint32_t log_inv_rate, uint32_t mask_coeffs,
                       const uint64_t *rows, size_t nrows, const uint64_t *masks, uint64_t *codewords,
                       void *stream);
int tg_encode_rows(tg_device *dev, uint32_t log_k, uint32_t log_inv_rate, uint32_t mask_coeffs,
                   const uint64_t *rows, size_t nrows, const uint64_t *masks, uint64_t *codewords);
/* tg_encode_rows_dev without any device allocation, for callers that cannot call cudaMalloc
 * (device memory owned by another allocator, or a loop that must not synchronize the device as
 * cudaMalloc/cudaFree do). No counterpart in the reference. Tables and scratch live in one fixed
 * 32 MiB device array that every GPU loading the library holds until exit; shapes need
 * 2 (k + n) <= 2^22 words (k <= 2^19 at rate 1/2) and larger ones are refused. The first call on a
 * device looks up the array's address, so make it before any stream capture. Calls share the
 * array: calls that overlap on the GPU race, so order them on one stream. The handle's device
 * must be the current device (TG_ERR_INVALID otherwise). */
int tg_encode_rows_noalloc_dev(tg_device *dev, uint32_t log_k, uint32_t log_inv_rate, uint32_t mask_coeffs,
                               const uint64_t *rows, size_t nrows, const uint64_t *masks, uint64_t *codewords,
                               void *stream);

/* ---- Standalone transforms: NttPlan::{ntt, intt, coset_ntt, coset_intt}
 * (crates/tessera-pcs/src/ntt.rs:461-516), over nrows rows of n = 2^log_n values each, in place,
 * natural order on both sides: ntt gives values[j] = f(ω_n^j) from the coefficients, coset_ntt
 * values[j] = f(shift·ω_n^j), intt and coset_intt their inverses. log_n <= 22; a zero or
 * non-canonical shift is refused (PcsError::ZeroShift). The _dev forms work on device memory
 * and are enqueued on `stream` (NULL: the device's stream); the others take host memory. */
int tg_ntt_dev(tg_device *dev, uint32_t log_n, uint64_t *values, size_t nrows, void *stream);
int tg_intt_dev(tg_device *dev, uint32_t log_n, uint64_t *values, size_t nrows, void *stream);
int tg_coset_ntt_dev(tg_device *dev, uint32_t log_n, uint64_t shift, uint64_t *values, size_t nrows, void *stream);
int tg_coset_intt_dev(tg_device *dev, uint32_t log_n, uint64_t shift, uint64_t *values, size_t nrows, void *stream);
int tg_ntt(tg_device *dev, uint32_t log_n, uint64_t *values, size_t nrows);
int tg_intt(tg_device *dev, uint32_t log_n, uint64_t *values, size_t nrows);
int tg_coset_ntt(tg_device *dev, uint32_t log_n, uint64_t shift, uint64_t *values, size_t nrows);
int tg_coset_intt(tg_device *dev, uint32_t log_n, uint64_t shift, uint64_t *values, size_t nrows);

/* ---- The advice mask stream: ProverDomain::AdviceMasks (crates/tessera-hash/src/domain.rs:83-127)
 * out[i] is the (first + i)-th word below p of BLAKE3's extended output of
 * H("advice-masks", seed) in derive-key mode (eight little-endian words per 64-byte output block,
 * words at or above p skipped), i < count: the masks a prover draws for its advice commitment,
 * P per row, m_0 first, in row order. seed: at most 64 bytes (a proof seed is 32). The _dev form
 * writes device memory on `stream` and returns once the values are written; the other host
 * memory. The values are secret-class: the host form clears its device copy. */
int tg_advice_masks_dev(tg_device *dev, const uint8_t *seed, size_t seed_len, uint64_t first, size_t count,
                        uint64_t *out, void *stream);
int tg_advice_masks(tg_device *dev, const uint8_t *seed, size_t seed_len, uint64_t first, size_t count, uint64_t *out);

/* ---- Column chains and Merkle trees (crates/tessera-hash/src/columns.rs:72-104,
 * crates/tessera-hash/src/merkle.rs:93-113). chains: ncols x 32 bytes. */
int tg_column_init_dev(tg_device *dev, const uint8_t commitment_id[32], uint64_t ncols, uint8_t *chains,
                       void *stream);
/* Absorbs `count` rows (count x ncols symbols, row-major) in blocks of `row_block` rows
 * (1 <= row_block <= 124, each step one BLAKE3 chunk). */
int tg_column_absorb_dev(tg_device *dev, uint8_t *chains, uint64_t ncols, const uint64_t *rows, size_t count,
                         uint32_t row_block, void *stream);
/* Every node of the tree over n (a power of two) leaves: nodes holds 2n - 1 digests, leaves
 * first, the root last (the reference's level order). */
int tg_merkle_tree_dev(tg_device *dev, const uint8_t *leaves, size_t n, uint8_t *nodes, void *stream);
/* leaf_j = H("column-merge", d_j^(1) || ... || d_j^(S)) over S x n segment chains
 * (crates/tessera-pcs/src/streaming.rs:432-438). */
int tg_column_merge_dev(tg_device *dev, const uint8_t *segment_chains, size_t nsegments, uint64_t n,
                        uint8_t *leaves, void *stream);

/* ---- Resident unmasked commitment: ReferenceCommitment::commit_unmasked
 * (crates/tessera-pcs/src/commitment.rs:343-458): encode, one chain per column over blocks of
 * row_block rows (leaf = last chain), Merkle tree. Device form: codewords (npolys x n) and
 * nodes (2n - 1 digests) are caller device buffers; the root is copied to host `root`. */
int tg_commit_unmasked_dev(tg_device *dev, uint32_t log_k, uint32_t log_inv_rate, uint32_t row_block,
                           const uint8_t commitment_id[32], const uint64_t *rows, size_t npolys,
                           uint64_t *codewords, uint8_t *nodes, uint8_t root[32], void *stream);
/* Host form: rows in host memory; leaves (n x 32, may be NULL) and root returned to the host. */
int tg_commit_unmasked(tg_device *dev, uint32_t log_k, uint32_t log_inv_rate, uint32_t row_block,
                       const uint8_t commitment_id[32], const uint64_t *rows, size_t npolys, uint8_t *leaves,
                       uint8_t root[32]);

/* Many unmasked commitments of uneven shapes at once (the batched pattern; each job is what one
 * tg_commit_unmasked_dev call takes, all buffers on the device). The jobs run on `workers`
 * streams (0: the library's default), longest first onto the least loaded stream; roots and
 * nodes are byte-identical to committing the jobs one at a time. */
typedef struct {
    uint32_t log_k, log_inv_rate, row_block;
    uint8_t commitment_id[32];
    const uint64_t *rows;  /* device: npolys x 2^log_k */
    size_t npolys;
    uint64_t *codewords;   /* device out: npolys x n */
    uint8_t *nodes;        /* device out: 2n - 1 digests, leaves first, root last */
    uint8_t root[32];      /* out (tg_commit_many) */
} tg_commit_job;
int tg_commit_many(tg_device *dev, tg_commit_job *jobs, int njobs, int workers);

/* A batch of commitments captured once into a CUDA graph and replayed. Creating the plan
 * builds the twiddle tables, allocates the encoder scratch the graph keeps, and autotunes on the
 * batch itself: (1) for each encoder shape (k, rate, rows) with 2^13 <= k <= 2^22, the split of
 * the row transform k = K1 x K2 (K1 = 2^split_log) and the rows per group, by timing each
 * candidate's encode of the first job of that shape (or read from the cache file named by the
 * environment variable TESSERA_GB300_TUNE_CACHE, written after tuning, for a GPU of the same SM
 * count); (2) with workers = 0, the worker count over {1, 2, 4, 8}, by timing a replay of each
 * candidate graph. Every launch then re-reads the jobs' row buffers (same addresses, new
 * contents) and writes the codewords, nodes, and the njobs x 32 roots to host `roots`. */
typedef struct tg_commit_plan tg_commit_plan;
int tg_commit_plan_create(tg_device *dev, const tg_commit_job *jobs, int njobs, int workers, tg_commit_plan **out);
int tg_commit_plan_launch(tg_commit_plan *plan, uint8_t *roots);
/* The chosen worker count, kernels per replay, and the autotuner's replay times (ms) at
 * 1, 2, 4 and 8 workers (0 where not tried). */
int tg_commit_plan_info(const tg_commit_plan *plan, int *workers, uint64_t *kernels, double tuned_ms[4]);
/* The encoder configuration the plan chose for one shape. */
typedef struct {
    uint32_t log_k, log_inv_rate;
    uint64_t npolys;
    int32_t split_log;   /* log2 K1, the length of passes M1/M2's columns */
    int32_t candidates;  /* configurations timed (0: read from the cache) */
    uint64_t group;      /* rows per group */
    double ms_default;   /* one encode of the shape with the default split and group */
    double ms_tuned;     /* ... with the chosen ones */
    int32_t from_cache;
    int32_t reserved;
} tg_encode_tuning;
/* Writes up to cap shapes to out; *count = the plan's number of tuned shapes. */
int tg_commit_plan_tuning(const tg_commit_plan *plan, tg_encode_tuning *out, int cap, int *count);
int tg_commit_plan_destroy(tg_commit_plan *plan);

/* merge_segments on host buffers (crates/tessera-pcs/src/streaming.rs:382-404). */
int tg_merge_segments(tg_device *dev, const uint8_t *segment_chains, size_t nsegments, uint64_t n,
                      uint8_t *leaves, uint8_t root[32]);

/* ---- BlockSink: the advice sink (crates/tessera-pcs/src/streaming.rs:24-37; the reference's
 * AdviceSink, crates/tessera-prover/src/gpu.rs:570-667). Opened with the commitment's k, rate,
 * P and B; starts from the chains of commitment_id over n columns. absorb takes one block of
 * 1..B whole rows (k values each) and their masks (P per row, m_0 first); a block shorter than
 * B must be the last. finish writes the n chains (n x 32). Device copies of rows, masks and
 * codewords are zeroed before their memory is released. */
int tg_advice_sink_open(tg_device *dev, uint32_t log_k, uint32_t log_inv_rate, uint32_t mask_coeffs,
                        uint32_t row_block, const uint8_t commitment_id[32], tg_sink **out);
int tg_sink_absorb(tg_sink *sink, const uint64_t *rows, size_t nrows, const uint64_t *masks);
int tg_sink_finish(tg_sink *sink, uint8_t *chains);
int tg_sink_close(tg_sink *sink);

/* ---- MatrixSink / WeightEncoding (crates/tessera-pcs/src/weights/regenerated.rs:24-58):
 * unmasked rows at any rate 1/2^r, chained leaves, answering `queries` (codeword columns,
 * distinct and increasing). absorb writes nrows x nqueries answers, row by row. */
int tg_matrix_open(tg_device *dev, uint32_t log_k, uint32_t log_inv_rate, uint32_t row_block,
                   const uint8_t commitment_id[32], const uint64_t *queries, size_t nqueries, tg_matrix **out);
int tg_matrix_absorb(tg_matrix *m, const uint64_t *rows, size_t nrows, uint64_t *answers);
int tg_matrix_finish(tg_matrix *m, uint8_t *chains);
int tg_matrix_close(tg_matrix *m);

/* ---- ColumnSink (crates/tessera-pcs/src/streaming/opening.rs:845-884; the reference's GPU
 * ColumnsSink, crates/tessera-prover/src/gpu.rs:196-398): P5 re-encodes blocks of whole rows
 * (mask_coeffs masks per row, m_0 first) and returns each row's symbols at `columns`
 * (out: nrows x ncolumns, row by row; a column at or past n reads 0). select_combining also adds
 * P4's combined rows Σ_r coefficients[g][r]·rows[r] (coefficients: groups x nrows Fp2) to sums
 * kept on the device, with one group count per opening; combined adds those sums into `out`
 * (groups x k Fp2) and clears them (a no-op before any combining block). Device copies of rows,
 * masks, codewords and sums are zeroed when the sink closes. */
typedef struct tg_column_sink tg_column_sink;
int tg_column_sink_open(tg_device *dev, uint32_t log_k, uint32_t log_inv_rate, uint32_t mask_coeffs, uint32_t block,
                        const uint64_t *columns, size_t ncolumns, tg_column_sink **out);
int tg_column_sink_select(tg_column_sink *sink, const uint64_t *rows, size_t nrows, const uint64_t *masks,
                          uint64_t *out);
int tg_column_sink_select_combining(tg_column_sink *sink, const uint64_t *rows, size_t nrows, const uint64_t *masks,
                                    const uint64_t *coefficients, size_t groups, uint64_t *out);
int tg_column_sink_combined(tg_column_sink *sink, uint64_t *out, size_t groups);
int tg_column_sink_close(tg_column_sink *sink);

/* ---- Fiat–Shamir transcript (crates/tessera-hash/src/transcript.rs:127-250), host side.
 * context_tce is TCE(SessionContext). */
typedef struct {
    uint8_t state[32];
    uint64_t counter;
} tg_transcript;
int tg_hash(const char *domain, const uint8_t *in, size_t len, uint8_t out[32]);
int tg_transcript_init(tg_transcript *t, const uint8_t *context_tce, size_t len);
int tg_transcript_absorb(tg_transcript *t, const char *label, const uint8_t *value, size_t len);
int tg_transcript_absorb_fp2s(tg_transcript *t, const char *label, const uint64_t *values, size_t count);
int tg_transcript_squeeze(tg_transcript *t, const char *label, uint8_t out[32]);
int tg_transcript_challenge_fp(tg_transcript *t, const char *label, uint64_t *out);
int tg_transcript_challenge_fp2(tg_transcript *t, const char *label, uint64_t out[2]);
int tg_transcript_challenge_indices(tg_transcript *t, const char *label, uint32_t log_n, uint32_t count,
                                    uint64_t *out);
int tg_transcript_check_grind(tg_transcript *t, const char *label, uint32_t bits, uint64_t nonce, int *valid);
/* grind (transcript.rs:241-250): the smallest nonce meeting `bits`, searched on the GPU,
 * then absorbed. */
int tg_transcript_grind(tg_device *dev, tg_transcript *t, const char *label, uint32_t bits, uint64_t *nonce);

/* ---- Batched sumcheck: prove_batch (crates/tessera-sumcheck/src/prover.rs:1122) for
 * product instances, Protocol One (degree 1..7). A table is 2^vars entries: words (is_ext = 0,
 * Table::base) or Fp2 pairs (is_ext = 1, Table::ext); is_public leaves it out of the final
 * evaluations (Table::public). Tables are device pointers when tables_on_device, else host.
 * Outputs: gamma; rounds: n_max x degree Fp2 (p(0), p(2), ..., p(d)); challenges: n_max Fp2;
 * final_evals: the evaluations (count in *n_evals). The transcript advances exactly as the
 * reference's does. */
typedef struct {
    const uint64_t *values;
    int is_ext;
    int is_public;
} tg_table;
typedef struct {
    const tg_table *tables;
    int ntables;
    int vars;
} tg_instance;
int tg_prove_batch(tg_device *dev, tg_transcript *t, const char *prefix, int degree, const tg_instance *instances,
                   int ninstances, int tables_on_device, uint64_t gamma[2], uint64_t *rounds, uint64_t *challenges,
                   uint64_t *final_evals, size_t *n_evals);

/* Many independent prove_batch calls at once (the batched pattern of uneven sumcheck instances;
 * each job is what one tg_prove_batch call takes, with its own transcript). The jobs' rounds run
 * in lockstep: round j of every job is one fused launch of round sums plus one launch that
 * advances every job's transcript on the device, so a batch of J jobs of up to n variables costs
 * about 2n launches instead of 2·Σ n_i. Results, transcripts included, are byte-identical to calling
 * tg_prove_batch on the jobs one after another. On any error every transcript is left as it was. */
typedef struct {
    tg_transcript *transcript; /* this job's transcript, advanced in place */
    const char *prefix;
    int degree;
    const tg_instance *instances;
    int ninstances;
    uint64_t gamma[2];      /* out */
    uint64_t *rounds;       /* out (may be NULL): n_max x degree Fp2 */
    uint64_t *challenges;   /* out (may be NULL): n_max Fp2 */
    uint64_t *final_evals;  /* out (may be NULL): one Fp2 per non-public table */
    size_t n_evals;         /* out */
} tg_sumcheck_job;
int tg_prove_many(tg_device *dev, tg_sumcheck_job *jobs, int njobs, int tables_on_device);

/* ---- LevelOffload / DeviceLevel (crates/tessera-sumcheck/src/offload.rs:17-79; the
 * reference's GpuLevels, crates/tessera-gpu/src/level.rs:52-146). shape 0: fraction
 * N0 D1 + N1 D0 + λ D0 D1 over [N0, N1, D0, D1]; shape 1: product V0 V1 over [V0, V1].
 * tables: ntables host pointers to len Fp2 entries each. Returns TG_DECLINED with *out = NULL
 * when the level is below the minimum size, over the budget or malformed, as load() declines.
 * Handles are safe to use from several threads. */
int tg_level_load(tg_device *dev, int shape, const uint64_t lambda[2], const uint64_t *const *tables, int ntables,
                  size_t len, tg_level **out);
/* Σ_p w(p) P(line_x(p)) for x = 0, 2, 3 over the current pairs, w(p) = low[p mod 2^low_bits]
 * high[p >> low_bits]; low has 2^low_bits Fp2, high nhigh Fp2. out: 3 Fp2. */
int tg_level_sums(tg_level *l, const uint64_t *low, const uint64_t *high, size_t nhigh, uint32_t low_bits,
                  uint64_t out[6]);
int tg_level_bind(tg_level *l, const uint64_t r[2]);
/* Each table's first entry, in table order (ntables Fp2). */
int tg_level_firsts(tg_level *l, uint64_t *out);
int tg_level_free(tg_level *l);

/* ---- Tree levels: product forests and LogUp fraction trees (RFC-0010 'Tree levels'; the
 * reference's FractionTree, crates/tessera-sumcheck/src/trees.rs:260-345, prove_trees :761, and
 * LogUp's leaf stage, crates/tessera-logup/src/prover.rs:361). Trees are listed in schedule order.
 * kind 0: a forest of 2^s product trees of height `height` (a single tree: s = 0) from its
 * 2^(s+height) stacked leaves (Fp2, or prime-field words with base_leaves, as the reference's GPU
 * forest takes them, crates/tessera-gpu/src/trees.rs:163-185); kind 1: a fraction tree (s = 0) from 2^height numerators
 * (Fp2; NULL: all 1) and denominators (Fp2), entering the schedule with `sent` (n, d) when given
 * (as the roots message carried it), else its own root. Every level is built on the device when
 * the stage opens; each tg_leaf_stage_prove_level call proves the next level on the transcript,
 * byte for byte as the reference does, and moves every present tree's claim one level down.
 * With on_device, the leaves are read in place (they must stay unchanged until the stage closes);
 * the other levels and the bound tables come from the device's workspace cache. */
/* Generated LogUp leaves, as tg_logup_leaves writes them: leaf j is (n_j, α − (k_j + β·v_j)) with
 * k_j = counter(key_seed + j), v_j = counter(value_seed + j) and n_j = 1 (unit) or −m_j,
 * m_j = counter(mult_seed + j) mod 2^16 (the reference benchmark's inputs,
 * crates/tessera-gpu/src/fraction.rs:61-105). */
typedef struct {
    uint64_t key_seed, value_seed, mult_seed;
    int unit;
    uint64_t alpha[2], beta[2];
} tg_leaf_gen;

typedef struct {
    int kind;
    uint32_t s, height;
    const uint64_t *leaves;        /* forest leaves, or fraction numerators */
    const uint64_t *denominators;  /* fraction trees */
    const uint64_t *sent;          /* fraction trees: 2 Fp2, or NULL */
    uint32_t base_leaves;          /* forests: 1 when the leaves are prime-field words (one per leaf) */
    const tg_leaf_gen *gen;        /* fraction trees, or NULL: the stage generates the leaves into
                                      `denominators` (and `leaves` unless gen->unit; NULL then), 16-byte
                                      aligned device buffers of 2^height Fp2 (on_device), in the same pass
                                      as the two levels above them */
} tg_tree;
typedef struct {
    int level;
    int n_root_challenges;     /* s_max of the joining forests */
    uint64_t *root_challenges; /* caller buffer, >= 40 Fp2 (may be NULL) */
    uint64_t gamma[2];
    int has_lambda;
    uint64_t lambda[2];
    int n_max;                 /* rounds */
    uint64_t *rounds;          /* caller buffer: n_max x 3 Fp2 (p(0), p(2), p(3)) */
    uint64_t *challenges;      /* n_max Fp2 */
    uint64_t *claims;          /* n_max + 1 Fp2, as a verifier derives them */
    int n_evals;
    uint64_t *evals;           /* caller buffer: 2 Fp2 per forest, 4 per fraction tree */
    uint64_t rho[2];
    int n_present;
    int *present;              /* caller buffer: the trees present at the level, in order */
} tg_tree_level_proof;
typedef struct tg_leaf_stage tg_leaf_stage;
int tg_leaf_stage_open(tg_device *dev, const tg_tree *trees, int ntrees, int on_device, tg_leaf_stage **out);
/* H, the tallest height (the number of levels), and the next level to prove. */
int tg_leaf_stage_height(const tg_leaf_stage *stage, int *height, int *level);
/* A forest's root level (2^s Fp2) or a fraction tree's root (n, d). */
int tg_leaf_stage_root(const tg_leaf_stage *stage, int tree, uint64_t *out);
int tg_leaf_stage_prove_level(tg_leaf_stage *stage, tg_transcript *t, tg_tree_level_proof *out);
/* A tree's current claim: its point (npoint Fp2), the claim (a forest's value, then 0; a fraction
 * tree's (p, q)) and its level (−1 before it joins). */
int tg_leaf_stage_claim(const tg_leaf_stage *stage, int tree, uint64_t *point, int *npoint, uint64_t *claim, int *own);
int tg_leaf_stage_close(tg_leaf_stage *stage);
/* Generated LogUp leaves on the device (the reference benchmark's fraction-tree inputs,
 * crates/tessera-gpu/src/fraction.rs:61-105): leaf j is (n_j, α − (k_j + β·v_j)) with
 * k_j = counter(key_seed + j), v_j = counter(value_seed + j), counter(c) the SplitMix64 output for
 * state (c + 1)·0x9E3779B97F4A7C15 reduced once below p, and n_j = 1 (unit) or −m_j,
 * m_j = counter(mult_seed + j) mod 2^16. numerators and denominators: count Fp2 each, device
 * (numerators may be NULL with unit: numerators of 1 need no table). */
int tg_logup_leaves(tg_device *dev, uint64_t key_seed, uint64_t value_seed, int unit, uint64_t mult_seed,
                    const uint64_t alpha[2], const uint64_t beta[2], size_t count, uint64_t *numerators,
                    uint64_t *denominators);

/* ---- Serving: a proof server with continuous batching (no reference counterpart: the serving
 * pattern around the hot path). A request's proof is the resident unmasked commitment of its rows
 * (commit_unmasked, crates/tessera-pcs/src/commitment.rs:343-458), the root absorbed into the
 * request's transcript under "<prefix>/root", then prove_batch of one instance, the product of its
 * prime-field tables, under <prefix> (crates/tessera-sumcheck/src/prover.rs:1122). Requests are
 * admitted first come first served while a stream slot is free and their device footprint fits
 * the HBM budget (a request larger than the budget runs alone); admitted requests run on their own
 * streams with stream-ordered device memory, so their work overlaps on the GPU, and a scheduler
 * thread advances each one, woken by the streams' completions; when requests overlap, the oldest
 * in flight runs on high-priority streams. Results are byte-identical to proving the request
 * alone. Host rows and tables must stay valid until the request completes (pinned memory lets
 * their copies overlap).
 * With queries > 0 the proof ends with an opening round on the still-resident commitment: after
 * the sumcheck, `queries` column indices are drawn from the transcript under "<prefix>/queries"
 * (Transcript::challenge_indices over log2 n bits, crates/tessera-hash/src/transcript.rs), and the
 * answer is read from the codewords and Merkle nodes the commitment left on the device: each
 * distinct queried column's symbols (one per row, in row order, the columns in increasing index
 * order) and the canonical multiproof of those indices (the siblings the verifier cannot compute,
 * level by level from the leaves up, left to right within a level; the verifier's
 * verify_multiproof, verifier/crates/tv-hash/src/merkle.rs:137). A request's answer must fit
 * 1 MiB of staging: queries · (8·npolys + 32·log2 n) bytes, about. */
typedef struct {
    uint32_t log_k, log_inv_rate, row_block;
    uint8_t commitment_id[32];
    const uint64_t *rows;          /* host: npolys x 2^log_k */
    size_t npolys;
    int degree, ntables, vars;     /* the sumcheck: ntables prime-field tables of 2^vars entries */
    const uint64_t *const *tables; /* host */
    tg_transcript transcript;      /* the proof's transcript at its start */
    const char *prefix;
    uint32_t queries;              /* column queries answered after the proof (0: none) */
} tg_proof_request;
typedef struct {
    int status;                    /* TG_OK once done */
    uint8_t root[32];
    uint64_t gamma[2];
    uint64_t *rounds;              /* caller buffers: vars x degree Fp2 */
    uint64_t *challenges;          /* vars Fp2 */
    uint64_t *final_evals;         /* ntables Fp2 */
    tg_transcript transcript;      /* at the end of the proof */
    double queued_ms, latency_ms;  /* submission to admission, submission to completion */
    /* the opening round (caller buffers, used when queries > 0): */
    uint64_t *query_indices;       /* queries indices, in draw order */
    uint64_t *columns;             /* n_distinct x npolys symbols (room for queries x npolys) */
    uint8_t *siblings;             /* n_siblings digests (room for queries x log2 n) */
    uint32_t n_distinct, n_siblings;
    /* when the scheduler saw each stage end (commit, sumcheck, opening), ms after submission */
    double stage_ms[3];
} tg_proof_result;
typedef struct {
    uint64_t submitted, completed, peak_inflight;
    size_t peak_bytes;
} tg_server_stats;
typedef struct tg_server tg_server;
int tg_server_open(tg_device *dev, size_t hbm_budget_bytes, int max_inflight, tg_server **out);
/* Queues a request; *out is filled when it completes (collect it with tg_server_wait). */
int tg_server_submit(tg_server *server, const tg_proof_request *request, tg_proof_result *out, uint64_t *ticket);
/* Waits for a ticket (timeout_ms < 0: no limit): TG_OK, the request's error, or TG_DECLINED on
 * timeout. Each ticket is collected once. */
int tg_server_wait(tg_server *server, uint64_t ticket, int timeout_ms);
int tg_server_stats_read(tg_server *server, tg_server_stats *out);
/* Finishes every queued and running request, then releases the server. */
int tg_server_close(tg_server *server);

#ifdef __cplusplus
}
#endif
#endif
