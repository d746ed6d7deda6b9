// SPDX-License-Identifier: Apache-2.0 OR MIT
//
// Batched sumcheck of products of multilinear tables on the device: the reference's prove_batch
// (crates/tessera-sumcheck/src/prover.rs:1122-1421) with its round sums and binds
// (crates/tessera-sumcheck/src/kernel.rs:90-101, 292-355, 591-633). Conventions (RFC-0010 as the
// reference applies them): x_1 is the index's least significant bit; round j binds x_j; the
// message is p(0), p(2), …, p(d); instance i weighs γ^i; an instance on fewer variables than the
// batch is front-padded and contributes 2^{n_max − n_i − j − 1}·S_i to each of its padding rounds.
//
// Many independent proofs ("jobs", each a prove_batch with its own transcript) advance in
// lockstep: a large round j of every job is ONE launch of sc_rounds, whose blocks are split among
// the (job, instance) segments of that round in proportion to their pairs, and ONE launch of
// sc_fs_many, one warp per job, which forms the job's message, absorbs it into the job's
// Fiat–Shamir transcript and squeezes its challenge with BLAKE3 on the device
// (crates/tessera-hash/src/transcript.rs:168-219); the rounds of at most SC_PERSIST_PAIRS pairs
// run in one persistent launch of sc_persist. A segment binds the previous challenge into its
// tables (t'[i] = t[2i] + r·(t[2i+1] − t[2i])) in the same pass that accumulates the d node sums
// of the new table, and the last of its blocks to finish reduces the blocks' partial sums. The
// rounds never return to the host: γ is drawn on the host before them, and the final evaluations
// are absorbed on the host after them; each transcript travels to the device and back once.
// tg_prove_batch is the one-job case.
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <string>
#include <vector>

#include "b3.cuh"
#include "gl.cuh"
#include "fs.cuh"
#include "internal.h"

namespace tg {

constexpr int SC_MAX_TABLES = 7;
constexpr int SC_MAX_DEGREE = 7;
constexpr int SC_THREADS = 256;
constexpr int SC_MAX_SEG_BLOCKS = 1024;
constexpr int SC_MSG_WORDS = 2 * SC_MAX_DEGREE;  // one instance's round sums, as Fp2 words
// The last rounds run in one block from the first whose segments hold this many pairs in all,
// when every job has a warp of that block for its transcript (fewer when the rounds before them
// run in the same launch as well).
constexpr uint64_t SC_TAIL_PAIRS = 4096, SC_TAIL_PAIRS_PERSIST = 512;
// With cooperative launches, the rounds from the first whose segments hold at most this many pairs
// in all run in one launch of sc_persist, on one block per SC_PERSIST_BLOCK_PAIRS pairs of its largest
// round: blocks wait for each other at every round's transcript, and the fewer they are, the more of
// the GPU stays free for other streams' work (the proof server's requests).
constexpr uint64_t SC_PERSIST_PAIRS = 1ull << 16, SC_PERSIST_BLOCK_PAIRS = 1024;
constexpr uint64_t SC_PERSIST_MIN_BLOCKS = 16, SC_PERSIST_MIN_BLOCK_PAIRS = 256;

// One instance's share of one launch.
struct Seg {
    const uint64_t* src[SC_MAX_TABLES];  // current tables (or the tables to bind first)
    uint64_t* dst[SC_MAX_TABLES];        // bound tables (when bind)
    const uint64_t* r;                   // the challenge to bind, in device memory
    uint64_t* out;                       // reduced sums, Fp2 words
    uint64_t n;                          // pairs of the (bound) table; entries for a product sum
    uint32_t base_mask;                  // bit k: table k's source holds prime-field words
    int nt, degree, bind, kind;          // kind 0: round sums, 1: Σ_x Π_k T_k[x]
    int block0, nblocks, part0;          // the segment's blocks in the launch, its first partials row
    int inst, job;                       // the instance and its job
};
static_assert(sizeof(Seg) % 8 == 0, "Seg copies as words");
// sc_persist patches words of a Seg as it copies them into shared memory
static_assert(offsetof(Seg, r) % 8 == 0 && offsetof(Seg, nblocks) % 8 == 0 && offsetof(Seg, job) % 8 == 4,
              "Seg word layout");

struct BindLast {
    const uint64_t* src;
    uint64_t* dst;
    const uint64_t* r;
    int base, pad_;
};

struct EvalRef {
    const uint64_t* ptr;
    int base, pad_;
};

// How a round reads its tables: MEM_LAUNCH in a launch of its own (streamed past the caches), MEM_L2
// where other blocks of the same launch may have written them (the persistent rounds: through L2
// only). The challenge is read with plain loads in both modes: a launched round reads it from
// device memory that an earlier launch wrote, the persistent rounds from the block's shared memory.
enum { MEM_LAUNCH = 0, MEM_L2 = 1 };

template <int MEM = MEM_LAUNCH>
__device__ __forceinline__ fp2 load_entry(const uint64_t* t, bool base, uint64_t i) {
    if (base) return e_lift(MEM == MEM_L2 ? __ldcg(t + i) : t[i]);
    const ulonglong2 v = MEM == MEM_L2 ? __ldcg(reinterpret_cast<const ulonglong2*>(t) + i)
                                       : reinterpret_cast<const ulonglong2*>(t)[i];  // (c0, c1) words
    return {v.x, v.y};
}

// The challenge to bind, written by the previous round's transcript.
__device__ __forceinline__ fp2 load_r(const uint64_t* r) { return fp2{r[0], r[1]}; }

// a + r·(b − a) on lazy words (bound tables hold lazy words; the last bind canonicalises); r7 =
// 7·r.c1.
__device__ __forceinline__ fp2 bind_pair(fp2 a, fp2 b, fp2 r, uint64_t r7, bool base) {
    if (base) {  // a, b in the prime field: two base products
        const uint64_t d = lz::sub(b.c0, a.c0);
        return {lz::add(a.c0, lz::mul(r.c0, d)), lz::mul(r.c1, d)};
    }
    return l2_fma(a, r, r7, l2_sub(b, a));
}

// Sums NW words across the block (warp shuffles, then one word per warp in shared memory);
// thread 0 gets the totals.
template <int NW>
__device__ __forceinline__ void block_sum(uint64_t (&v)[NW]) {
    __shared__ uint64_t red[SC_THREADS / 32][NW];
#pragma unroll
    for (int w = 0; w < NW; w++)
        for (int o = 16; o > 0; o >>= 1) v[w] = add(v[w], __shfl_down_sync(0xFFFFFFFFu, v[w], o));
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0)
#pragma unroll
        for (int w = 0; w < NW; w++) red[warp][w] = v[w];
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 1; k < (int)(blockDim.x >> 5); k++)
#pragma unroll
            for (int w = 0; w < NW; w++) v[w] = add(v[w], red[k][w]);
    }
    __syncthreads();
}

// A table's 16 bytes at p, read as MEM says (streamed in a launch of its own: every entry is read
// once per round).
template <int MEM>
__device__ __forceinline__ ulonglong2 ld_once(const uint64_t* t, uint64_t p) {
    ulonglong2 v;
    if constexpr (MEM == MEM_L2)
        asm volatile("ld.global.cg.v2.u64 {%0, %1}, [%2];" : "=l"(v.x), "=l"(v.y) : "l"(t + 2 * p));
    else
        asm volatile("ld.global.cs.v2.u64 {%0, %1}, [%2];" : "=l"(v.x), "=l"(v.y) : "l"(t + 2 * p));
    return v;
}

// Block lb's share of a segment of the commonest shapes — NT tables multiplied at degree DEG (three
// at degree 3: Σ f·g·h; two at degree 2: Σ f·g) — with the tables' field fixed at compile time:
// the first round (prime-field tables, nothing to bind) sums in the prime field; the later rounds
// bind r into their source (prime-field or Fp2 entries), store the bound pair and sum in Fp2. All
// of a thread's loads for U pairs are issued before any is used, so that each thread keeps
// U·NT·(1, 2 or 4) 16-byte loads in flight.
template <int D, int NT, int DEG, bool BIND, bool SRC_BASE, int U, int MEM>
__device__ __forceinline__ void seg_sums_fixed(const Seg& g, int lb, uint64_t (&words)[2 * D]) {
    static_assert(DEG <= D && NT <= DEG && (BIND || SRC_BASE), "shape");
    const uint64_t stride = (uint64_t)g.nblocks * blockDim.x, n = g.n;
    const uint64_t start = (uint64_t)lb * blockDim.x + threadIdx.x;
    if constexpr (!BIND) {
        uint64_t acc[DEG];
#pragma unroll
        for (int d = 0; d < DEG; d++) acc[d] = 0;
        for (uint64_t p0 = start; p0 < n; p0 += U * stride) {
            ulonglong2 x[U][NT];
#pragma unroll
            for (int q = 0; q < U; q++) {
                const uint64_t p = p0 + q * stride;
#pragma unroll
                for (int k = 0; k < NT; k++) x[q][k] = p < n ? ld_once<MEM>(g.src[k], p) : make_ulonglong2(0, 0);
            }
#pragma unroll
            for (int q = 0; q < U; q++) {
                uint64_t prod[DEG];
#pragma unroll
                for (int k = 0; k < NT; k++) {
                    const uint64_t u = x[q][k].x, v = x[q][k].y, diff = lz::sub(v, u);
                    uint64_t t = v;  // node 1, then 2, 3, …
                    prod[0] = k ? lz::mul(prod[0], u) : u;
#pragma unroll
                    for (int d = 1; d < DEG; d++) {
                        t = lz::add(t, diff);
                        prod[d] = k ? lz::mul(prod[d], t) : t;
                    }
                }
#pragma unroll
                for (int d = 0; d < DEG; d++) acc[d] = lz::add(acc[d], prod[d]);
            }
        }
#pragma unroll
        for (int d = 0; d < DEG; d++) words[2 * d] = lz::canon(acc[d]);
    } else {
        const fp2 r = load_r(g.r);
        const uint64_t r7 = lz::mul7(r.c1);
        constexpr int L = SRC_BASE ? 2 : 4;  // 16-byte loads per table and pair: 4 source entries
        fp2 acc[DEG];
#pragma unroll
        for (int d = 0; d < DEG; d++) acc[d] = {0, 0};
        for (uint64_t p0 = start; p0 < n; p0 += U * stride) {
            ulonglong2 x[U][NT][L];
#pragma unroll
            for (int q = 0; q < U; q++) {
                const uint64_t p = p0 + q * stride;
#pragma unroll
                for (int k = 0; k < NT; k++)
#pragma unroll
                    for (int l = 0; l < L; l++) x[q][k][l] = p < n ? ld_once<MEM>(g.src[k], L * p + l) : make_ulonglong2(0, 0);
            }
#pragma unroll
            for (int q = 0; q < U; q++) {
                const uint64_t p = p0 + q * stride;
                fp2 prod[DEG];
#pragma unroll
                for (int k = 0; k < NT; k++) {
                    fp2 u, v;
                    if constexpr (SRC_BASE) {  // entries 4p, 4p + 1 | 4p + 2, 4p + 3 as words
                        u = bind_pair(e_lift(x[q][k][0].x), e_lift(x[q][k][0].y), r, r7, true);
                        v = bind_pair(e_lift(x[q][k][1].x), e_lift(x[q][k][1].y), r, r7, true);
                    } else {
                        u = bind_pair({x[q][k][0].x, x[q][k][0].y}, {x[q][k][1].x, x[q][k][1].y}, r, r7, false);
                        v = bind_pair({x[q][k][2].x, x[q][k][2].y}, {x[q][k][3].x, x[q][k][3].y}, r, r7, false);
                    }
                    if (p < n) {
                        ulonglong2* out = reinterpret_cast<ulonglong2*>(g.dst[k]);
                        out[2 * p] = make_ulonglong2(u.c0, u.c1);
                        out[2 * p + 1] = make_ulonglong2(v.c0, v.c1);
                    }
                    const fp2 diff = l2_sub(v, u);
                    fp2 t = v;
                    prod[0] = k ? l2_muls(prod[0], u) : u;
#pragma unroll
                    for (int d = 1; d < DEG; d++) {
                        t = l2_add(t, diff);
                        prod[d] = k ? l2_muls(prod[d], t) : t;
                    }
                }
#pragma unroll
                for (int d = 0; d < DEG; d++) acc[d] = l2_add(acc[d], prod[d]);
            }
        }
#pragma unroll
        for (int d = 0; d < DEG; d++) {
            const fp2 c = l2_canon(acc[d]);
            words[2 * d] = c.c0;
            words[2 * d + 1] = c.c1;
        }
    }
}

// The bind rounds of seg_sums_fixed's shapes when a segment has at most two pairs per group of
// four threads: four lanes take a pair; lane q < NT binds table q's pair and forms its values at the
// NT nodes, then lane d < NT multiplies the tables' values at node d — passed round the group by
// shuffles, at step s from the lane of table (d + s) mod NT — and keeps node d's sum. A pair's
// arithmetic is spread over NT lanes instead of one: the persistent launch's small rounds, whose
// threads hold a pair or none, are bound by that arithmetic's latency.
template <int D, int NT, bool SRC_BASE, int MEM>
__device__ __forceinline__ void seg_sums_split(const Seg& g, int lb, uint64_t (&words)[2 * D]) {
    static_assert(NT <= D && NT >= 2 && NT <= 3, "shape");
    constexpr int L = SRC_BASE ? 2 : 4;  // 16-byte loads of a table's pair: its four source entries
    const int lane = threadIdx.x & 31, q = lane & 3;
    const bool act = q < NT;
    const uint64_t n = g.n, groups = (uint64_t)g.nblocks * (blockDim.x / 4);
    const fp2 r = load_r(g.r);
    const uint64_t r7 = lz::mul7(r.c1);
    const uint64_t* src = g.src[act ? q : 0];
    ulonglong2* out = reinterpret_cast<ulonglong2*>(g.dst[act ? q : 0]);
    fp2 acc = {0, 0};
    // warp-uniform steps: every lane of the warp takes part in every shuffle
    for (uint64_t p0 = (uint64_t)lb * (blockDim.x / 4) + (threadIdx.x >> 5) * 8; p0 < n; p0 += groups) {
        const uint64_t p = p0 + (lane >> 2);
        const bool live = act && p < n;
        ulonglong2 x[L];
#pragma unroll
        for (int l = 0; l < L; l++) x[l] = live ? ld_once<MEM>(src, L * p + l) : make_ulonglong2(0, 0);
        fp2 u, v;
        if constexpr (SRC_BASE) {
            u = bind_pair(e_lift(x[0].x), e_lift(x[0].y), r, r7, true);
            v = bind_pair(e_lift(x[1].x), e_lift(x[1].y), r, r7, true);
        } else {
            u = bind_pair({x[0].x, x[0].y}, {x[1].x, x[1].y}, r, r7, false);
            v = bind_pair({x[2].x, x[2].y}, {x[3].x, x[3].y}, r, r7, false);
        }
        if (live) {
            out[2 * p] = make_ulonglong2(u.c0, u.c1);
            out[2 * p + 1] = make_ulonglong2(v.c0, v.c1);
        }
        fp2 val[NT];  // this lane's table at the nodes: u, then v + (v − u), …
        const fp2 diff = l2_sub(v, u);
        val[0] = u;
        fp2 t = v;
#pragma unroll
        for (int d = 1; d < NT; d++) {
            t = l2_add(t, diff);
            val[d] = t;
        }
        fp2 prod = val[0];
#pragma unroll
        for (int d = 1; d < NT; d++)
            if (q == d) prod = val[d];
#pragma unroll
        for (int st = 1; st < NT; st++) {
            // lane q serves the lane d with (d + st) mod NT = q: its value at node d
            const int need = (q + NT - st) % NT;
            fp2 sv = val[0];
#pragma unroll
            for (int d = 1; d < NT; d++)
                if (need == d) sv = val[d];
            const int from = (lane & ~3) | (act ? (q + st) % NT : q);
            const fp2 rv = {__shfl_sync(0xFFFFFFFFu, sv.c0, from), __shfl_sync(0xFFFFFFFFu, sv.c1, from)};
            prod = l2_muls(prod, rv);
        }
        if (live) acc = l2_add(acc, prod);
    }
    const fp2 c = l2_canon(acc);
#pragma unroll
    for (int d = 0; d < NT; d++)
        if (q == d) words[2 * d] = c.c0, words[2 * d + 1] = c.c1;
}

// The shapes seg_sums_fixed covers; false leaves the segment to the general loops. SPLIT: the small
// bind rounds of those shapes through seg_sums_split.
template <int D, int MEM = MEM_LAUNCH, bool SPLIT = false>
__device__ __forceinline__ bool seg_sums_fast(const Seg& g, int lb, uint64_t (&words)[2 * D]) {
    if (g.kind != 0) return false;
    const bool all_base = g.base_mask == (1u << g.nt) - 1, all_ext = g.base_mask == 0;
    if constexpr (SPLIT) {
        if (g.bind && g.nt == g.degree && g.n <= (uint64_t)g.nblocks * (blockDim.x / 2)) {
            if constexpr (D >= 3) {
                if (g.nt == 3 && all_base) return seg_sums_split<D, 3, true, MEM>(g, lb, words), true;
                if (g.nt == 3 && all_ext) return seg_sums_split<D, 3, false, MEM>(g, lb, words), true;
            }
            if constexpr (D >= 2) {
                if (g.nt == 2 && all_base) return seg_sums_split<D, 2, true, MEM>(g, lb, words), true;
                if (g.nt == 2 && all_ext) return seg_sums_split<D, 2, false, MEM>(g, lb, words), true;
            }
        }
    }
    if constexpr (D >= 3) {
        if (g.nt == 3 && g.degree == 3) {
            if (!g.bind && all_base) return seg_sums_fixed<D, 3, 3, false, true, 4, MEM>(g, lb, words), true;
            if (g.bind && all_base) return seg_sums_fixed<D, 3, 3, true, true, 2, MEM>(g, lb, words), true;
            if (g.bind && all_ext) return seg_sums_fixed<D, 3, 3, true, false, 1, MEM>(g, lb, words), true;
        }
    }
    if constexpr (D >= 2) {
        if (g.nt == 2 && g.degree == 2) {
            if (!g.bind && all_base) return seg_sums_fixed<D, 2, 2, false, true, 4, MEM>(g, lb, words), true;
            if (g.bind && all_base) return seg_sums_fixed<D, 2, 2, true, true, 2, MEM>(g, lb, words), true;
            if (g.bind && all_ext) return seg_sums_fixed<D, 2, 2, true, false, 2, MEM>(g, lb, words), true;
        }
    }
    return false;
}

// Block lb's share of a segment's sums (a grid-stride loop over the segment's nblocks blocks),
// canonical, in this thread's words: the d node sums as Fp2 words (kind 0), or the product sum.
template <int D, int MEM = MEM_LAUNCH>
__device__ __forceinline__ void sc_seg_sums(const Seg& g, int lb, uint64_t (&words)[2 * D]) {
    const uint64_t stride = (uint64_t)g.nblocks * blockDim.x;
    const int deg = g.degree, nt = g.nt;
#pragma unroll
    for (int w = 0; w < 2 * D; w++) words[w] = 0;

    // lazy arithmetic throughout; the sums are canonicalised before they are reduced
    if (g.kind == 1) {
        fp2 acc = {0, 0};
        for (uint64_t x = (uint64_t)lb * blockDim.x + threadIdx.x; x < g.n; x += stride) {
            fp2 prod = {1, 0};
            for (int k = 0; k < nt; k++) {
                const fp2 e = load_entry<MEM>(g.src[k], (g.base_mask >> k) & 1, x);
                prod = k ? l2_muls(prod, e) : e;
            }
            acc = l2_add(acc, prod);
        }
        acc = l2_canon(acc);
        words[0] = acc.c0;
        words[1] = acc.c1;
    } else if (!g.bind && g.base_mask == (1u << nt) - 1) {
        // all tables in the prime field and nothing to bind: products and sums in the prime field
        uint64_t acc[D];
#pragma unroll
        for (int d = 0; d < D; d++) acc[d] = 0;
        for (uint64_t p = (uint64_t)lb * blockDim.x + threadIdx.x; p < g.n; p += stride) {
            uint64_t prod[D];
#pragma unroll
            for (int d = 0; d < D; d++) prod[d] = 1;
            for (int k = 0; k < nt; k++) {  // the first table's values start the products
                const ulonglong2 v = MEM == MEM_L2 ? __ldcg(reinterpret_cast<const ulonglong2*>(g.src[k]) + p)
                                                   : reinterpret_cast<const ulonglong2*>(g.src[k])[p];
                const uint64_t diff = lz::sub(v.y, v.x);
                uint64_t x = v.y;  // value at node 1
                prod[0] = k ? lz::mul(prod[0], v.x) : v.x;
#pragma unroll
                for (int d = 1; d < D; d++) {  // nodes 2..D
                    if (d < deg) {
                        x = lz::add(x, diff);
                        prod[d] = k ? lz::mul(prod[d], x) : x;
                    }
                }
            }
#pragma unroll
            for (int d = 0; d < D; d++) acc[d] = lz::add(acc[d], prod[d]);
        }
#pragma unroll
        for (int d = 0; d < D; d++) words[2 * d] = lz::canon(acc[d]);
    } else {
        fp2 acc[D];
#pragma unroll
        for (int d = 0; d < D; d++) acc[d] = {0, 0};
        const fp2 r = g.bind ? load_r(g.r) : fp2{0, 0};
        const uint64_t r7 = lz::mul7(r.c1);
        for (uint64_t p = (uint64_t)lb * blockDim.x + threadIdx.x; p < g.n; p += stride) {
            fp2 prod[D];
#pragma unroll
            for (int d = 0; d < D; d++) prod[d] = {1, 0};
            for (int k = 0; k < nt; k++) {
                const bool base = (g.base_mask >> k) & 1;
                fp2 u, v;
                if (g.bind) {
                    u = bind_pair(load_entry<MEM>(g.src[k], base, 4 * p), load_entry<MEM>(g.src[k], base, 4 * p + 1), r, r7,
                                  base);
                    v = bind_pair(load_entry<MEM>(g.src[k], base, 4 * p + 2), load_entry<MEM>(g.src[k], base, 4 * p + 3), r,
                                  r7, base);
                    ulonglong2* out = reinterpret_cast<ulonglong2*>(g.dst[k]);
                    out[2 * p] = make_ulonglong2(u.c0, u.c1);
                    out[2 * p + 1] = make_ulonglong2(v.c0, v.c1);
                } else {
                    u = load_entry<MEM>(g.src[k], base, 2 * p);
                    v = load_entry<MEM>(g.src[k], base, 2 * p + 1);
                }
                const fp2 diff = l2_sub(v, u);
                fp2 x = v;
                prod[0] = k ? l2_muls(prod[0], u) : u;  // the first table's values start the products
#pragma unroll
                for (int d = 1; d < D; d++) {
                    if (d < deg) {
                        x = l2_add(x, diff);
                        prod[d] = k ? l2_muls(prod[d], x) : x;
                    }
                }
            }
#pragma unroll
            for (int d = 0; d < D; d++) acc[d] = l2_add(acc[d], prod[d]);
        }
#pragma unroll
        for (int d = 0; d < D; d++) {
            const fp2 c = l2_canon(acc[d]);
            words[2 * d] = c.c0;
            words[2 * d + 1] = c.c1;
        }
    }
}

// One launch of round sums (and product sums) over all segments: a block finds its segment, runs
// a grid-stride loop over the segment's pairs, and the segment's last block to finish reduces the
// segment's partial rows into seg.out. SHAPE 0 takes any segment; SHAPE 1–6 (sc_shape) only
// segments of that one shape, through its fixed-shape sums, so that the launch carries the
// registers of that form alone.
template <int D, int SHAPE>
__global__ void __launch_bounds__(SC_THREADS) sc_rounds(const Seg* segs, int nseg, uint64_t* partials,
                                                        unsigned* counters) {
    __shared__ Seg g;
    __shared__ int si;
    if (threadIdx.x == 0) {
        int lo = 0, hi = nseg - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) / 2;
            if (segs[mid].block0 <= (int)blockIdx.x)
                lo = mid;
            else
                hi = mid - 1;
        }
        si = lo;
    }
    __syncthreads();
    {
        const uint64_t* from = reinterpret_cast<const uint64_t*>(segs + si);
        uint64_t* to = reinterpret_cast<uint64_t*>(&g);
        for (int w = threadIdx.x; w < (int)(sizeof(Seg) / 8); w += blockDim.x) to[w] = from[w];
    }
    __syncthreads();
    const int lb = blockIdx.x - g.block0;
    const int deg = g.degree;
    uint64_t words[2 * D];
#pragma unroll
    for (int w = 0; w < 2 * D; w++) words[w] = 0;
    if constexpr (SHAPE == 0) sc_seg_sums<D>(g, lb, words);
    else if constexpr (SHAPE == 1) seg_sums_fixed<D, 3, 3, false, true, 4, MEM_LAUNCH>(g, lb, words);
    else if constexpr (SHAPE == 2) seg_sums_fixed<D, 3, 3, true, true, 1, MEM_LAUNCH>(g, lb, words);
    else if constexpr (SHAPE == 3) seg_sums_fixed<D, 3, 3, true, false, 1, MEM_LAUNCH>(g, lb, words);
    else if constexpr (SHAPE == 4) seg_sums_fixed<D, 2, 2, false, true, 4, MEM_LAUNCH>(g, lb, words);
    else if constexpr (SHAPE == 5) seg_sums_fixed<D, 2, 2, true, true, 2, MEM_LAUNCH>(g, lb, words);
    else seg_sums_fixed<D, 2, 2, true, false, 1, MEM_LAUNCH>(g, lb, words);
    block_sum<2 * D>(words);

    // the segment's last block reduces its partial rows
    __shared__ bool last;
    if (threadIdx.x == 0) {
#pragma unroll
        for (int w = 0; w < 2 * D; w++) partials[(size_t)(g.part0 + lb) * 2 * D + w] = words[w];
        __threadfence();
        last = atomicAdd(&counters[si], 1u) == (unsigned)g.nblocks - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
#pragma unroll
    for (int w = 0; w < 2 * D; w++) words[w] = 0;
    for (int b = threadIdx.x; b < g.nblocks; b += blockDim.x)
#pragma unroll
        for (int w = 0; w < 2 * D; w++) words[w] = add(words[w], __ldcg(&partials[(size_t)(g.part0 + b) * 2 * D + w]));
    block_sum<2 * D>(words);
    if (threadIdx.x == 0) {
        const int nout = g.kind == 1 ? 2 : 2 * deg;
        for (int w = 0; w < nout; w++) g.out[w] = words[w];
        counters[si] = 0;
    }
}

// Binds the last round (tables of two entries into one), one thread per table.
__global__ void sc_bind_last(const BindLast* b, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const BindLast t = b[i];
    const fp2 r = {t.r[0], t.r[1]};
    const fp2 u = l2_canon(bind_pair(load_entry(t.src, t.base, 0), load_entry(t.src, t.base, 1), r, lz::mul7(r.c1), t.base));
    reinterpret_cast<ulonglong2*>(t.dst)[0] = make_ulonglong2(u.c0, u.c1);
}

// Each table's single entry after the last bind (public factors left out), as Fp2 words.
__global__ void sc_gather_evals(const EvalRef* refs, int n, uint64_t* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const EvalRef e = refs[i];
    out[2 * i] = e.ptr[0];
    out[2 * i + 1] = e.base ? 0 : e.ptr[1];
}

// ---- the transcripts on the device (one warp per job) ------------------------------------------


// A job's round message lives in registers: D (the batch's largest degree) values, of which the
// job's first `degree` are its own; the loops over them unroll to fixed indices.

// The message from each lane's node (lane x holds node x, lazy; the rest zero) into every lane.
template <int D>
__device__ __forceinline__ void persist_msg_gather(fp2 mine, fp2 (&msg)[D]) {
    mine = l2_canon(mine);
#pragma unroll
    for (int x = 0; x < D; x++)
        msg[x] = {__shfl_sync(0xFFFFFFFFu, mine.c0, x), __shfl_sync(0xFFFFFFFFu, mine.c1, x)};
}


// The padded instances' part of job jb's round-j message, added to msg: w_i·2^{pad_i − j − 1}·S_i
// at every node of each instance still in its padding rounds.
template <int D>
__device__ __forceinline__ void sc_fs_padded(const FsJob& jb, int j, const uint64_t* w, const int* pad,
                                             const uint64_t* S, fp2 (&msg)[D]) {
    if (j >= jb.pad_max) return;  // every instance of the job is past its padding rounds
    for (int i = jb.inst0; i < jb.inst0 + jb.ninst; i++) {
        if (j >= pad[i]) continue;
        const fp2 wi = {w[2 * i], w[2 * i + 1]};
        const fp2 v = e_mul(wi, e_scale(fp2{__ldcg(S + 2 * i), __ldcg(S + 2 * i + 1)}, (1ull << (pad[i] - j - 1)) % P));
#pragma unroll
        for (int x = 0; x < D; x++)
            if (x < jb.degree) msg[x] = e_add(msg[x], v);
    }
}

// Round j's transcript step of job t, its message formed (the same in every lane): the message into
// rounds_out, absorbed as TCE Vec<Fp2> under <prefix>/round/j; then r_j = challenge_fp2 under
// <prefix>/r/j. state and counter (the same in every lane) are read and updated here; lane 0 writes
// them, r_j and the challenge back to the job's FsState and to chal_out (unless !write: a copy of
// the step that another block writes), and r_j to r_local when given. With sq, another warp has
// built the absorb input's head in buf and the first squeeze's input in sq (fs_round_warp); the
// two warps meet at named barrier 1 before this one adds the message.
template <int D>
__device__ __forceinline__ void sc_fs_step(FsState* states, const FsJob& jb, int t, int j, const FsKeys& keys,
                                           const fp2 (&msg)[D], uint32_t (&state)[8], uint64_t& counter,
                                           uint64_t* rounds_out, uint64_t* chal_out, uint32_t* buf, bool write = true,
                                           uint64_t* r_local = nullptr, uint32_t* sq = nullptr) {
    const int lane = threadIdx.x & 31;
    const int degree = jb.degree;
    FsState* st = states + t;
    if (lane == 0 && write) {
        uint64_t* rj = rounds_out + jb.rounds_off + (size_t)j * 2 * degree;
#pragma unroll
        for (int x = 0; x < D; x++)
            if (x < degree) rj[2 * x] = msg[x].c0, rj[2 * x + 1] = msg[x].c1;
    }
    // the message as TCE Vec<Fp2>: its length, then the values
    uint64_t pay[1 + 2 * D];
    pay[0] = (uint64_t)degree;
#pragma unroll
    for (int x = 0; x < D; x++) pay[1 + 2 * x] = msg[x].c0, pay[2 + 2 * x] = msg[x].c1;
    uint32_t len, sq_len = 0;
    if (sq) {
        const int nd = fs_digits(j);
        sq_len = 40 + jb.label_len + fs_len("/r/") + nd + 8;
        fs_pair_sync();
        len = fs_pay_warp<1 + 2 * D>(pay, 1 + 2 * degree, 40 + jb.label_len + fs_len("/round/") + nd, buf);
    } else {
        len = fs_msg_warp<1 + 2 * D>(state, jb, fs_pack("/round/"), fs_len("/round/"), j, pay, 1 + 2 * degree, buf);
    }
    uint64_t c0, c1;
    const bool ok = fs_round_warp(keys, jb, j, buf, len, state, &counter, &c0, &c1, sq, sq_len);
    if (lane != 0) return;
    if (r_local) r_local[0] = c0, r_local[1] = c1;
    if (!write) return;
    if (!ok) {
        st->err = 1;
        return;
    }
#pragma unroll
    for (int i = 0; i < 8; i++) reinterpret_cast<uint32_t*>(st->state)[i] = state[i];
    st->counter = counter;
    st->r[0] = c0;
    st->r[1] = c1;
    chal_out[jb.chal_off + 2 * j] = c0;
    chal_out[jb.chal_off + 2 * j + 1] = c1;
}

// Round j's message of each job: Σ over its instances of w_i·(own sums, or 2^{pad_i − j − 1}·S_i
// while padded), absorbed as TCE Vec<Fp2> under <prefix>/round/j; then r_j = challenge_fp2 under
// <prefix>/r/j. One warp runs job t's round (buf: FS_BUF_WORDS of the warp's shared memory), the
// state read from the job's FsState (through L2: the persistent rounds move a job between blocks).
template <int D>
__device__ void sc_fs_job(FsState* states, const FsJob* jobs, int t, int j, const FsKeys& keys, const uint64_t* w,
                          const int* pad, const uint64_t* S, const uint64_t* msgbuf, uint64_t* rounds_out,
                          uint64_t* chal_out, uint32_t* buf) {
    const FsJob& jb = jobs[t];
    if (j >= jb.n_max) return;
    const int lane = threadIdx.x & 31;
    fp2 mine = {0, 0};  // lane x: node x of the message, lazy words
    for (int i = jb.inst0; i < jb.inst0 + jb.ninst; i++) {
        if (j < pad[i] || lane >= jb.degree) continue;
        const uint64_t* m = msgbuf + (size_t)i * SC_MSG_WORDS + 2 * lane;
        mine = l2_add(mine, l2_mul(fp2{w[2 * i], w[2 * i + 1]}, fp2{__ldcg(m), __ldcg(m + 1)}));
    }
    fp2 msg[D];
    persist_msg_gather<D>(mine, msg);
    sc_fs_padded(jb, j, w, pad, S, msg);
    uint32_t state[8];
#pragma unroll
    for (int i = 0; i < 8; i++) state[i] = __ldcg(reinterpret_cast<const uint32_t*>(states[t].state) + i);
    uint64_t counter = __ldcg(&states[t].counter);
    sc_fs_step(states, jb, t, j, keys, msg, state, counter, rounds_out, chal_out, buf);
}

template <int D>
__global__ void __launch_bounds__(FS_THREADS) sc_fs_many(FsState* states, const FsJob* jobs, int njobs, int j,
                                                         FsKeys keys, const uint64_t* w, const int* pad,
                                                         const uint64_t* S, const uint64_t* msgbuf,
                                                         uint64_t* rounds_out, uint64_t* chal_out) {
    __shared__ uint32_t sbuf[FS_THREADS / 32][FS_BUF_WORDS];
    const int t = (blockIdx.x * blockDim.x + threadIdx.x) / 32;
    if (t >= njobs) return;  // whole warps leave together
    sc_fs_job<D>(states, jobs, t, j, keys, w, pad, S, msgbuf, rounds_out, chal_out, sbuf[threadIdx.x / 32]);
}

// The rounds jp … J − 1 of a batch in one launch, with no launch between rounds. The first `multi`
// of them are spread over the launch's G co-resident blocks (a cooperative launch): every block
// takes its share of every segment of the round (a grid-stride loop over the segment's pairs, one
// partial row per block and segment), and the blocks meet. With at most eight jobs ("local"), every
// block then runs every job's transcript step itself — warp b reduces the partial rows of job b's
// instances into its message and draws its challenge, the same in every block, which only block 0
// writes out — and goes on to the next round with the challenges in its shared memory: one meeting
// a round, the partial rows alternating between two halves of the buffer so that a block already
// in the next round does not overwrite rows that another still reads. With more jobs, the warp that
// owns a job (job b: warp (b / G) mod 8 of block b mod G) runs its step and the blocks meet again
// before the next round reads the challenges. The rounds after those, whose segments are one
// block's work, run in block 0 alone (the others have returned): each sums its segments with the
// whole block, then the block's warps run the transcripts. Whatever another block may have written
// — tables, partial sums, messages, transcript states — is read through L2.
struct ScPersist {
    FsKeys keys;
    FsState* states;
    const FsJob* jobs;
    const uint64_t* w;
    const int* pad;
    const uint64_t* S;
    uint64_t* msgbuf;
    uint64_t* rounds_out;
    uint64_t* chal_out;
    const Seg* segs;     // the rounds' segments in round order
    const int* first;    // round jp + t's segments are segs[first[t] .. first[t + 1])
    uint64_t* partials;  // G rows per segment of a multi-block round
    unsigned* bar;       // the blocks' meeting point: arrivals, generation, gave up (each on its own 128-byte line)
    size_t part_words;   // the second half of partials (local): rounds alternate between the halves
    int njobs, jp, rounds, multi;
    int la_from;         // rounds la_from … rounds − 1 take their sums from the look-ahead (−1: none)
    int pad_;
    uint64_t* const* la_scratch;  // 2·D pointers to tables of 8 Fp2 entries, for the look-ahead's warm-up
};
static_assert(sizeof(ScPersist) % 8 == 0, "ScPersist copies as words");
constexpr int SC_MAX_VARS = 40;  // an instance's variables at most (so at most 40 rounds)

// The meeting point's words: the arrivals (which the waiting blocks poll) and, on its own 128-byte
// line, the give-up flag.
constexpr int SC_BAR_COUNT = 0, SC_BAR_FAIL = 32, SC_BAR_WORDS = 64;
constexpr unsigned SC_BAR_POLLS = 1u << 24;  // about a second of polling before a meeting gives up

// All G blocks of the launch meet. The arrivals count up one word that is never reset within a
// launch (the host zeroes it before): meeting m is complete once it reaches G·m. Thread 0 of each
// block adds its arrival with an acquire-release atomic (its block's writes, ordered before it by
// the barrier, go out with it) and polls the count with acquire loads (the other blocks' writes come
// in with it); the barrier after hands both to the block's other threads. A block waits at most
// SC_BAR_POLLS polls, and stops waiting once another block has given up; then every thread of the
// block gets false (and the caller returns, so that no block waits on one that has left). The
// transcripts record the failure.
__device__ bool grid_meet(unsigned* bar, unsigned G, unsigned& gen, unsigned polls = SC_BAR_POLLS) {
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned target = G * (gen + 1);
        int good = 1;
        unsigned seen;
        asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], 1;" : "=r"(seen) : "l"(bar + SC_BAR_COUNT) : "memory");
        seen += 1;
        for (unsigned it = 1; seen < target; it++) {
            if ((it & 255) == 0 && (*(volatile unsigned*)(bar + SC_BAR_FAIL) || it >= polls)) {
                atomicExch(bar + SC_BAR_FAIL, 1u);
                good = 0;
                break;
            }
            __nanosleep(32);
            asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(seen) : "l"(bar + SC_BAR_COUNT) : "memory");
        }
        // a block that gave up before the last arrival is seen at the next meeting (its flag is
        // polled there, and it does not arrive); the rounds up to here had every block's share
        ok = good;
    }
    __syncthreads();
    gen++;
    return ok;
}

// A self-check of the meeting point (for tests): the launch's blocks meet `meetings` times, except
// block `absent` (−1: none), which leaves before the first meeting, so the others must give up
// after `polls` polls. out[0] counts the blocks that met every time, out[1] is the give-up flag.
__global__ void grid_meet_check(unsigned* bar, int meetings, int absent, unsigned polls, unsigned* out) {
    if ((int)blockIdx.x == absent) return;
    unsigned gen = 0;
    bool all = true;
    for (int m = 0; m < meetings && all; m++) all = grid_meet(bar, gridDim.x, gen, polls);
    if (threadIdx.x == 0) {
        if (all) atomicAdd(out, 1u);
        if (*(volatile unsigned*)(bar + SC_BAR_FAIL)) out[1] = 1;
    }
}

// Segments of a one-block round whose sums the block keeps in shared memory for the transcripts
// (the rest go through their instances' message words in device memory).
constexpr int SC_SMSG_SEGS = 32;

// The transcript state of the job a warp owns, kept in shared memory between its rounds: the 8
// state words, then the counter as two words.
__device__ __forceinline__ void fst_load(const uint32_t* f, uint32_t (&state)[8], uint64_t& counter) {
#pragma unroll
    for (int i = 0; i < 8; i++) state[i] = f[i];
    counter = (uint64_t)f[8] | ((uint64_t)f[9] << 32);
}
__device__ __forceinline__ void fst_store(uint32_t* f, const uint32_t (&state)[8], uint64_t counter) {
    if ((threadIdx.x & 31) == 0) {
#pragma unroll
        for (int i = 0; i < 8; i++) f[i] = state[i];
        f[8] = (uint32_t)counter;
        f[9] = (uint32_t)(counter >> 32);
    }
    __syncwarp();
}
__device__ __forceinline__ void fst_global(const FsState& st, uint32_t (&state)[8], uint64_t& counter) {
#pragma unroll
    for (int i = 0; i < 8; i++) state[i] = __ldcg(reinterpret_cast<const uint32_t*>(st.state) + i);
    counter = __ldcg(&st.counter);
}

// Segment si's Seg into shared memory, word i by the calling thread (threads with i in 0 … 21 of
// one warp or of the block; no barrier), patched on the way: nblocks replaces the segment's block
// count (the multi-block rounds take every segment over all blocks of the launch); the challenge
// pointer is redirected to shared memory — to the job's latest challenge in sr[job] when local,
// else to sr_seg, into which the thread copies the challenge from device memory (through L2:
// another block wrote it).
__device__ __forceinline__ void persist_seg_load(const Seg* segs, int si, Seg& g, int nblocks, bool local,
                                                 uint64_t (*sr)[2], uint64_t* sr_seg, int i) {
    constexpr int W = sizeof(Seg) / 8, WR = offsetof(Seg, r) / 8, WNB = offsetof(Seg, nblocks) / 8,
                  WJOB = offsetof(Seg, job) / 8;
    static_assert(W <= 32, "a warp copies a Seg");
    const uint64_t* src = reinterpret_cast<const uint64_t*>(segs + si);
    if (i < W) {
        uint64_t v = src[i];
        if (i == WR) {
            if (local) {
                v = reinterpret_cast<uint64_t>(&sr[(int)(src[WJOB] >> 32)][0]);
            } else {
                const uint64_t* rp = reinterpret_cast<const uint64_t*>(v);
                sr_seg[0] = __ldcg(rp);
                sr_seg[1] = __ldcg(rp + 1);
                v = reinterpret_cast<uint64_t>(sr_seg);
            }
        }
        if (i == WNB) v = (v & 0xFFFFFFFF00000000ull) | (uint32_t)nblocks;
        reinterpret_cast<uint64_t*>(&g)[i] = v;
    }
}

// The instance of segment si of a round whose first segment is s0 (recorded in sinst while the
// block summed the round's segments).
__device__ __forceinline__ int persist_inst(const ScPersist* A, const int* sinst, int si, int s0) {
    return si - s0 < SC_SMSG_SEGS ? sinst[si - s0] : __ldg(&A->segs[si].inst);
}

// Warp-wide: round j's message of job jb from the G partial rows of each of its segments of the
// round (part: the round's rows, through L2), the same in every lane.
// Instance inst's weight: from the job's first SC_SW weights in shared memory (sw, when given), else
// from device memory.
constexpr int SC_SW = 8;
__device__ __forceinline__ fp2 persist_weight(const ScPersist* A, const FsJob& jb, const uint64_t (*sw)[2], int inst) {
    const int k = inst - jb.inst0;
    if (sw && k < SC_SW) return fp2{sw[k][0], sw[k][1]};
    return fp2{A->w[2 * inst], A->w[2 * inst + 1]};
}

template <int D>
__device__ __forceinline__ void persist_msg_rows(const ScPersist* A, const FsJob& jb, const uint64_t (*sw)[2],
                                                 const uint64_t* part, const int* sinst, int s0, int s1, unsigned G,
                                                 fp2 (&msg)[D]) {
    const int lane = threadIdx.x & 31;
    fp2 mine = {0, 0};
    for (int si = s0; si < s1; si++) {
        const int inst = persist_inst(A, sinst, si, s0);
        if (inst < jb.inst0 || inst >= jb.inst0 + jb.ninst) continue;
        uint64_t acc[2 * D];
#pragma unroll
        for (int w = 0; w < 2 * D; w++) acc[w] = 0;
        const uint64_t* rows = part + (size_t)(si - s0) * G * 2 * D;
        for (int lb0 = lane; lb0 < (int)G; lb0 += 4 * 32) {  // four rows' loads in flight per lane
            uint64_t v[4][2 * D];
#pragma unroll
            for (int q = 0; q < 4; q++)
#pragma unroll
                for (int w = 0; w < 2 * D; w++) v[q][w] = lb0 + 32 * q < (int)G ? __ldcg(&rows[(size_t)(lb0 + 32 * q) * 2 * D + w]) : 0;
#pragma unroll
            for (int q = 0; q < 4; q++)
#pragma unroll
                for (int w = 0; w < 2 * D; w++) acc[w] = add(acc[w], v[q][w]);
        }
#pragma unroll
        for (int w = 0; w < 2 * D; w++)
            for (int o = 16; o > 0; o >>= 1) acc[w] = add(acc[w], __shfl_xor_sync(0xFFFFFFFFu, acc[w], o));
        if (lane < jb.degree) {  // lane x: node x
            fp2 v = {acc[0], acc[1]};
#pragma unroll
            for (int x = 1; x < D; x++)
                if (lane == x) v = {acc[2 * x], acc[2 * x + 1]};
            mine = l2_add(mine, l2_mul(persist_weight(A, jb, sw, inst), v));
        }
    }
    persist_msg_gather<D>(mine, msg);
}

// Warp-wide: round j's message of job jb from the sums of its segments that this block kept (smsg,
// or the instance's message words in device memory past SC_SMSG_SEGS segments), the same in every
// lane.
template <int D>
__device__ __forceinline__ void persist_msg_block(const ScPersist* A, const FsJob& jb, const uint64_t (*sw)[2],
                                                  const uint64_t (*smsg)[2 * D], const int* sinst, int s0, int s1,
                                                  fp2 (&msg)[D]) {
    const int lane = threadIdx.x & 31;
    fp2 mine = {0, 0};  // lane x: node x
    for (int si = s0; si < s1; si++) {
        const int inst = persist_inst(A, sinst, si, s0);
        if (inst < jb.inst0 || inst >= jb.inst0 + jb.ninst || lane >= jb.degree) continue;
        const bool kept = si - s0 < SC_SMSG_SEGS;
        const uint64_t* m = kept ? smsg[si - s0] : A->msgbuf + (size_t)inst * SC_MSG_WORDS;
        const fp2 v = kept ? fp2{m[2 * lane], m[2 * lane + 1]} : fp2{__ldcg(m + 2 * lane), __ldcg(m + 2 * lane + 1)};
        mine = l2_add(mine, l2_mul(persist_weight(A, jb, sw, inst), v));
    }
    persist_msg_gather<D>(mine, msg);
}

// Warp-wide: the rest of job b's round-j step with its state in shared memory (fstb) and its
// message formed: the padded instances' part, then the transcript step; r_j into srb.
template <int D>
__device__ __forceinline__ void persist_step(const ScPersist* A, const FsJob& jb, const FsKeys& keys, int b, int j,
                                             fp2 (&msg)[D], uint32_t* fstb, uint64_t* srb, uint32_t* buf, bool write,
                                             uint32_t* sq) {
    sc_fs_padded(jb, j, A->w, A->pad, A->S, msg);
    uint32_t state[8];
    uint64_t counter;
    fst_load(fstb, state, counter);
    sc_fs_step(A->states, jb, b, j, keys, msg, state, counter, A->rounds_out, A->chal_out, buf, write, srb, sq);
    fst_store(fstb, state, counter);
}

// ---- the look-ahead of the small one-block rounds ----------------------------------------------
//
// With one job of one instance of NT tables at degree NT (Σ f·g·h, Σ f·g), a one-block round of at
// most SC_LA_PAIRS pairs takes its sums from the round before it: while warp 0 draws r_t, warps
// 1 … 7 write round t+1's sums as polynomials in r_t. Pair p of round t+1 is T_{t+1}[2p] =
// a + r_t·(b − a), T_{t+1}[2p+1] = c + r_t·(d − c) with (a, b, c, d) = T_t[4p … 4p+3], so each node
// value is α + r_t·β and the product over the tables a polynomial of degree NT in r_t, whose
// coefficients the warps sum over the pairs. Once r_t is drawn, round t+1's message is those sums
// evaluated at r_t, and its transcript step starts at once; in its shadow the warps bind r_t into T_t
// (forming T_{t+1}, which the later rounds and the final evaluations read) and write round t+2's
// polynomials. The round's own sums, about a third of a one-block round, leave the critical path.
constexpr uint64_t SC_LA_PAIRS = 32;
__device__ int g_la_sink;  // written only to keep the look-ahead's warm-up call
constexpr int SC_LA_GROUPS = (SC_THREADS / 32 - 1) * 8;  // lane groups of four in warps 1 … 7

// Warps 1 … 7 of the block (named barrier 2): with bind, T_t = T_{t−1} bound by rprev (src → dst,
// n_t pairs of round t); with cubic, round t+1's polynomials from T_t (dst) summed into cub[x] (node
// x, NT + 1 Fp2 coefficients in lazy words, lowest first). red: the warps' rows.
template <int NT>
__device__ __noinline__ void persist_lookahead(const uint64_t* const* src, uint64_t* const* dst, uint64_t n_t, fp2 rprev,
                                               bool bind, bool cubic, uint64_t (*red)[NT][2 * (NT + 1)],
                                               uint64_t (*cub)[2 * (NT + 1)]) {
    constexpr int C = NT + 1;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, q = lane & 3;
    const uint64_t r7 = lz::mul7(rprev.c1);
    if (!cubic) {  // the last round: only T_t, 2·n_t entries a table
        for (uint64_t e = threadIdx.x - 32; e < (uint64_t)NT * 2 * n_t; e += SC_THREADS - 32) {
            const int k = (int)(e / (2 * n_t));
            const uint64_t i = e % (2 * n_t);
            const ulonglong2* s2 = reinterpret_cast<const ulonglong2*>(src[k]);
            const ulonglong2 x0 = __ldcg(s2 + 2 * i), x1 = __ldcg(s2 + 2 * i + 1);
            const fp2 v = bind_pair({x0.x, x0.y}, {x1.x, x1.y}, rprev, r7, false);
            reinterpret_cast<ulonglong2*>(dst[k])[i] = make_ulonglong2(v.c0, v.c1);
        }
        asm volatile("bar.sync 2, %0;" ::"r"(SC_THREADS - 32) : "memory");
        return;
    }
    const bool act = q < NT;
    const uint64_t n_next = n_t / 2;
    fp2 acc[C];
#pragma unroll
    for (int i = 0; i < C; i++) acc[i] = {0, 0};
    const int group = (warp - 1) * 8 + (lane >> 2);
    for (uint64_t p0 = 0; p0 < n_next; p0 += SC_LA_GROUPS) {  // the same steps in every lane
        const uint64_t p = p0 + group;
        const bool live = act && p < n_next;
        fp2 e[4];
        if (live) {
            if (bind) {  // T_t[4p + i] from T_{t−1}[8p + 2i], [8p + 2i + 1]
                const ulonglong2* s2 = reinterpret_cast<const ulonglong2*>(src[q]) + 8 * p;
                ulonglong2 x[8];
#pragma unroll
                for (int i = 0; i < 8; i++) x[i] = __ldcg(s2 + i);
                ulonglong2* d2 = reinterpret_cast<ulonglong2*>(dst[q]) + 4 * p;
#pragma unroll
                for (int i = 0; i < 4; i++) {
                    e[i] = bind_pair({x[2 * i].x, x[2 * i].y}, {x[2 * i + 1].x, x[2 * i + 1].y}, rprev, r7, false);
                    d2[i] = make_ulonglong2(e[i].c0, e[i].c1);
                }
            } else {
                const ulonglong2* d2 = reinterpret_cast<const ulonglong2*>(dst[q]) + 4 * p;
#pragma unroll
                for (int i = 0; i < 4; i++) {
                    const ulonglong2 v = __ldcg(d2 + i);
                    e[i] = {v.x, v.y};
                }
            }
        } else {
#pragma unroll
            for (int i = 0; i < 4; i++) e[i] = {0, 0};
        }
        // this table's nodes 0, 2, 3 as α + r·β: u = e0 + r(e1 − e0), v = e2 + r(e3 − e2)
        const fp2 au = e[0], bu = l2_sub(e[1], e[0]), av = e[2], bv = l2_sub(e[3], e[2]);
        fp2 al[NT], be[NT];
        al[0] = au, be[0] = bu;
        const fp2 da = l2_sub(av, au), db = l2_sub(bv, bu);  // v − u
        fp2 ta = av, tb = bv;
#pragma unroll
        for (int x = 1; x < NT; x++) {
            ta = l2_add(ta, da), tb = l2_add(tb, db);
            al[x] = ta, be[x] = tb;
        }
        // lane x gathers node x of every table (at step st from the lane of table (x + st) mod NT)
        fp2 ga[NT], gb[NT];
        ga[0] = al[0], gb[0] = be[0];
#pragma unroll
        for (int x = 1; x < NT; x++)
            if (q == x) ga[0] = al[x], gb[0] = be[x];
#pragma unroll
        for (int st = 1; st < NT; st++) {
            const int need = (q + NT - st) % NT;
            fp2 sa = al[0], sb = be[0];
#pragma unroll
            for (int x = 1; x < NT; x++)
                if (need == x) sa = al[x], sb = be[x];
            const int from = (lane & ~3) | (act ? (q + st) % NT : q);
            ga[st] = {__shfl_sync(0xFFFFFFFFu, sa.c0, from), __shfl_sync(0xFFFFFFFFu, sa.c1, from)};
            gb[st] = {__shfl_sync(0xFFFFFFFFu, sb.c0, from), __shfl_sync(0xFFFFFFFFu, sb.c1, from)};
        }
        if (live) {  // Π_k (ga_k + r·gb_k): coefficients of r^0 … r^NT
            const fp2 pa = l2_mul(ga[0], ga[1]), pb = l2_mul(gb[0], gb[1]);
            const fp2 pm = l2_sub(l2_sub(l2_mul(l2_add(ga[0], gb[0]), l2_add(ga[1], gb[1])), pa), pb);
            if constexpr (NT == 2) {
                acc[0] = l2_add(acc[0], pa), acc[1] = l2_add(acc[1], pm), acc[2] = l2_add(acc[2], pb);
            } else {
                acc[0] = l2_add(acc[0], l2_mul(pa, ga[2]));
                acc[1] = l2_add(acc[1], l2_add(l2_mul(pa, gb[2]), l2_mul(pm, ga[2])));
                acc[2] = l2_add(acc[2], l2_add(l2_mul(pm, gb[2]), l2_mul(pb, ga[2])));
                acc[3] = l2_add(acc[3], l2_mul(pb, gb[2]));
            }
        }
    }
    // the lanes of one node across the warp's eight groups, then across the warps
#pragma unroll
    for (int i = 0; i < C; i++)
        for (int o = 4; o < 32; o <<= 1) {
            acc[i].c0 = lz::add(acc[i].c0, __shfl_xor_sync(0xFFFFFFFFu, acc[i].c0, o));
            acc[i].c1 = lz::add(acc[i].c1, __shfl_xor_sync(0xFFFFFFFFu, acc[i].c1, o));
        }
    if (lane < NT)
#pragma unroll
        for (int i = 0; i < C; i++) red[warp - 1][lane][2 * i] = acc[i].c0, red[warp - 1][lane][2 * i + 1] = acc[i].c1;
    asm volatile("bar.sync 2, %0;" ::"r"(SC_THREADS - 32) : "memory");
    if (warp == 1 && lane < NT)
#pragma unroll
        for (int i = 0; i < 2 * C; i++) {
            uint64_t v = red[0][lane][i];
            for (int w = 1; w < SC_THREADS / 32 - 1; w++) v = lz::add(v, red[w][lane][i]);
            cub[lane][i] = v;
        }
}

// Lane x (< D) of a warp: node x of the message from the look-ahead's polynomials (cub) at r, the
// round before's challenge, times the instance's weight w (lazy words); zero in the other lanes.
// One copy of the code for every call, so that a call in an earlier round has fetched it.
template <int D>
__device__ __noinline__ fp2 persist_eval_lookahead(const uint64_t (*cub)[2 * (D + 1)], fp2 r, fp2 w) {
    const int lane = threadIdx.x & 31;
    if (lane >= D) return fp2{0, 0};
    fp2 v = {cub[lane][2 * D], cub[lane][2 * D + 1]};  // by Horner from the top coefficient
#pragma unroll
    for (int i = D - 1; i >= 0; i--) v = l2_add(l2_mul(v, r), fp2{cub[lane][2 * i], cub[lane][2 * i + 1]});
    return w.c0 == 1 && w.c1 == 0 ? v : l2_mul(w, v);
}

// Every block sets the given jobs' error flag (each job by one block) before the launch returns.
__device__ __forceinline__ void persist_gave_up(const ScPersist* A) {
    if (threadIdx.x == 0)
        for (int b = blockIdx.x; b < A->njobs; b += gridDim.x) atomicExch(&A->states[b].err, 2u);
}

template <int D>
__global__ void __launch_bounds__(SC_THREADS, 2) sc_persist(const ScPersist* __restrict__ Ag) {
    constexpr int NW = SC_THREADS / 32;
    // the launch's descriptor and round table in shared memory: they are read at every step, and
    // after each meeting's fence a load from device memory would miss the L1
    __shared__ ScPersist sA;
    __shared__ int sfirst[SC_MAX_VARS + 1];
    for (int i = threadIdx.x; i < (int)(sizeof(ScPersist) / 8); i += SC_THREADS)
        reinterpret_cast<uint64_t*>(&sA)[i] = reinterpret_cast<const uint64_t*>(Ag)[i];
    for (int i = threadIdx.x; i <= Ag->rounds; i += SC_THREADS) sfirst[i] = Ag->first[i];
    const ScPersist* A = &sA;
    __shared__ Seg g;
    __shared__ uint32_t sbuf[NW][FS_BUF_WORDS];
    __shared__ uint32_t fst[NW][10];
    __shared__ uint64_t smsg[SC_SMSG_SEGS][2 * D];
    __shared__ int sinst[SC_SMSG_SEGS];
    __shared__ FsJob sjob[NW];
    __shared__ uint64_t sw[NW][SC_SW][2];  // each job's first instances' weights (local)
    __shared__ uint64_t sr[NW][2];  // each job's latest challenge (local)
    // the look-ahead (one job): round t's challenge by round parity, the polynomials of the round
    // they are for by its parity, and the warps' rows
    __shared__ uint64_t srl[2][2];
    constexpr int LNT = D == 2 || D == 3 ? D : 2;
    __shared__ uint64_t cub[2][LNT][2 * (LNT + 1)];
    __shared__ uint64_t red[NW - 1][LNT][2 * (LNT + 1)];
    __shared__ uint64_t sr_seg[2];  // the current segment's challenge (not local)
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const unsigned G = gridDim.x;
    const int njobs = Ag->njobs;
    const bool local = njobs <= NW;
    if (local) {  // the jobs, their transcripts, weights and latest challenges, in every block
        for (int i = threadIdx.x; i < njobs * (int)(sizeof(FsJob) / 8); i += SC_THREADS)
            reinterpret_cast<uint64_t*>(sjob)[i] = reinterpret_cast<const uint64_t*>(Ag->jobs)[i];
        if (warp < njobs) {
            const FsState& st = Ag->states[warp];
            if (lane < 10)
                fst[warp][lane] = lane < 8 ? reinterpret_cast<const uint32_t*>(st.state)[lane]
                                           : (uint32_t)(st.counter >> (32 * (lane - 8)));
            if (lane < 2) sr[warp][lane] = st.r[lane];
            const FsJob& jb = Ag->jobs[warp];
            if (lane < SC_SW && lane < jb.ninst) {
                sw[warp][lane][0] = Ag->w[2 * (jb.inst0 + lane)];
                sw[warp][lane][1] = Ag->w[2 * (jb.inst0 + lane) + 1];
            }
        }
    }
    __syncthreads();
    unsigned gen = 0;
    // the block's last warp has no job (local, fewer than eight jobs): while the others run the
    // transcripts it copies the next round's first Seg into g, which the round's sums no longer read;
    // with one job it first builds that job's transcript inputs but the message (build)
    const bool prefetch = local && njobs < NW, build = local && njobs == 1;
    bool have_seg = false;  // g already holds the round's first Seg
    // One loop over all rounds, so that the sums and the transcript step are each one copy of code
    // (a copy first run in a later round would start there with its instructions out of cache).
    for (int t = 0; t < A->rounds; t++) {
        const bool multi = t < A->multi;
        if (!multi && blockIdx.x != 0) return;  // one block's work from here: at most eight jobs (local)
        const int s0 = sfirst[t], s1 = sfirst[t + 1];
        uint64_t* part = A->partials + (local && (t & 1) ? A->part_words : 0);
        // this round's sums came from the look-ahead (g holds its Seg, fetched in the round before)
        const bool ahead = A->la_from >= 0 && t >= A->la_from;
        for (int si = s0; si < s1 && !ahead; si++) {
            // a multi-block round takes every segment over all blocks of the launch
            if (si > s0 || !have_seg) persist_seg_load(A->segs, si, g, multi ? (int)G : 1, local, sr, sr_seg, threadIdx.x);
            __syncthreads();
            uint64_t words[2 * D];
#pragma unroll
            for (int w = 0; w < 2 * D; w++) words[w] = 0;
            const int lb = multi ? (int)blockIdx.x : 0;
            if (!seg_sums_fast<D, MEM_L2, true>(g, lb, words)) sc_seg_sums<D, MEM_L2>(g, lb, words);
            block_sum<2 * D>(words);  // ends with a barrier
            if (threadIdx.x == 0) {
                if (si - s0 < SC_SMSG_SEGS) sinst[si - s0] = g.inst;
                if (multi) {
#pragma unroll
                    for (int w = 0; w < 2 * D; w++) part[((size_t)(si - s0) * G + blockIdx.x) * 2 * D + w] = words[w];
                } else if (si - s0 < SC_SMSG_SEGS) {
#pragma unroll
                    for (int w = 0; w < 2 * D; w++) smsg[si - s0][w] = words[w];
                } else {
                    for (int w = 0; w < 2 * g.degree; w++) g.out[w] = words[w];
                }
            }
            __syncthreads();  // g is rewritten for the next segment
        }
        if (multi && !grid_meet(A->bar, G, gen)) return persist_gave_up(A);
        const int j = A->jp + t;
        if (local) {
            // warps 1 … 7 work in this round's transcript step's shadow: round t+1's polynomials
            // (binding r_{t−1} into this round's tables first when its sums came from the look-ahead),
            // or after the last round its bound tables alone
            const bool work_ahead =
                A->la_from >= 0 && !multi && (t + 1 < A->rounds ? t + 1 >= A->la_from : ahead);
            if (warp < njobs && j < sjob[warp].n_max) {
                const FsJob& jb = sjob[warp];
                fp2 msg[D];
                if constexpr (D == 2 || D == 3) {
                    if (ahead)
                        persist_msg_gather<D>(persist_eval_lookahead<D>(cub[t & 1], fp2{sr[0][0], sr[0][1]},
                                                                        persist_weight(A, jb, sw[warp], jb.inst0)),
                                              msg);
                }
                if (!ahead) {
                    if (multi)
                        persist_msg_rows<D>(A, jb, sw[warp], part, sinst, s0, s1, G, msg);
                    else
                        persist_msg_block<D>(A, jb, sw[warp], smsg, sinst, s0, s1, msg);
                }
                persist_step(A, jb, A->keys, warp, j, msg, fst[warp], sr[warp], sbuf[warp], blockIdx.x == 0,
                             build ? sbuf[NW - 1] : nullptr);
                if (lane == 0) srl[t & 1][0] = sr[warp][0], srl[t & 1][1] = sr[warp][1];
            } else if (prefetch && warp == NW - 1) {
                if (build && j < sjob[0].n_max) {  // job 0's absorb head and first squeeze input
                    uint32_t state[8];
                    uint64_t counter;
                    fst_load(fst[0], state, counter);
                    fs_head_warp(state, sjob[0], fs_pack("/round/"), fs_len("/round/"), j, sbuf[0]);
                    const uint64_t pay[1] = {counter};
                    fs_msg_warp<1>(state, sjob[0], fs_pack("/r/"), fs_len("/r/"), j, pay, 1, sbuf[NW - 1]);
                    fs_pair_sync();
                }
                if constexpr (D == 2 || D == 3) {
                    if (work_ahead)
                        persist_lookahead<D>(g.src, g.dst, g.n, fp2{srl[(t + 1) & 1][0], srl[(t + 1) & 1][1]}, ahead,
                                             t + 1 < A->rounds, red, cub[(t + 1) & 1]);
                }
                if (t + 1 < A->rounds) {
                    const bool multi_next = t + 1 < A->multi;
                    persist_seg_load(A->segs, sfirst[t + 1], g, multi_next ? (int)G : 1, true, sr, sr_seg, lane);
                }
            } else if (work_ahead && warp >= 1) {
                if constexpr (D == 2 || D == 3)
                    persist_lookahead<D>(g.src, g.dst, g.n, fp2{srl[(t + 1) & 1][0], srl[(t + 1) & 1][1]}, ahead,
                                         t + 1 < A->rounds, red, cub[(t + 1) & 1]);
            }
            if constexpr (D == 2 || D == 3) {
                // round 0 (or the first round, when it is one block's): warps 1 … 7 of block 0 run the
                // look-ahead's code once on a scratch table, in the transcript step's shadow, so that
                // its first real use does not fetch its instructions from device memory
                if (A->la_from >= 2 && t == 0 && blockIdx.x == 0 && warp >= 1) {
                    const uint64_t* const* src = A->la_scratch;
                    persist_lookahead<D>(src, A->la_scratch + D, 2, fp2{1, 0}, true, true, red, cub[1]);
                    persist_lookahead<D>(src, A->la_scratch + D, 2, fp2{1, 0}, false, true, red, cub[1]);
                    const fp2 v = persist_eval_lookahead<D>(cub[1], fp2{1, 0}, fp2{2, 0});
                    if (lane == 0 && v.c0 == 1 && v.c1 == 1) g_la_sink = 1;  // keeps the call
                }
            }
            __syncthreads();  // the challenges in sr (and the next Seg in g) for the next round
            have_seg = prefetch && t + 1 < A->rounds;
            continue;
        }
        // each warp owns at most one job when there are few: its state then stays in shared memory
        const bool keep = njobs <= (int)G * NW;
        for (int b = blockIdx.x + G * warp; b < njobs; b += G * NW) {
            const FsJob& jb = A->jobs[b];
            if (j >= jb.n_max) continue;
            fp2 msg[D];
            persist_msg_rows<D>(A, jb, nullptr, part, sinst, s0, s1, G, msg);
            sc_fs_padded(jb, j, A->w, A->pad, A->S, msg);
            uint32_t state[8];
            uint64_t counter;
            if (keep && t > 0)
                fst_load(fst[warp], state, counter);
            else
                fst_global(A->states[b], state, counter);
            sc_fs_step(A->states, jb, b, j, A->keys, msg, state, counter, A->rounds_out, A->chal_out, sbuf[warp]);
            if (keep) fst_store(fst[warp], state, counter);
        }
        if (!grid_meet(A->bar, G, gen)) return persist_gave_up(A);
    }
}

// ---- host driver -----------------------------------------------------------------------------


// The fixed shape of a segment for sc_rounds' SHAPE (0: none): 1–3 three tables at degree 3 (the
// first round over prime-field tables; a bind of prime-field entries; a bind of Fp2 entries), 4–6
// two tables at degree 2, likewise.
static int sc_shape(const Seg& g) {
    if (g.kind != 0) return 0;
    const bool all_base = g.base_mask == (1u << g.nt) - 1, all_ext = g.base_mask == 0;
    const int first = (g.nt == 3 && g.degree == 3) ? 1 : (g.nt == 2 && g.degree == 2) ? 4 : 0;
    if (!first) return 0;
    if (!g.bind) return all_base ? first : 0;
    return all_base ? first + 1 : all_ext ? first + 2 : 0;
}

template <typename F>
static void with_degree(int degree, F&& f) {
    switch (degree) {
        case 1: f(std::integral_constant<int, 1>{}); break;
        case 2: f(std::integral_constant<int, 2>{}); break;
        case 3: f(std::integral_constant<int, 3>{}); break;
        case 4: f(std::integral_constant<int, 4>{}); break;
        case 5: f(std::integral_constant<int, 5>{}); break;
        case 6: f(std::integral_constant<int, 6>{}); break;
        default: f(std::integral_constant<int, 7>{}); break;
    }
}

struct TableState {
    const uint64_t* src = nullptr;  // original entries (device, once uploaded)
    const uint64_t* host = nullptr; // original entries in host memory (when not on the device)
    bool base = false, is_public = false;
    size_t up_off = 0, buf_off[2] = {0, 0};
};

struct InstState {
    int job = 0, vars = 0, pad = 0;
    std::vector<TableState> tables;
};

// check_batch (prover.rs:1196-1218), in its order: degree, instances, then each instance.
static int check_job(const tg_sumcheck_job& jb, int index) {
    if (!jb.transcript || !jb.prefix) return fail(TG_ERR_INVALID, "job %d: null transcript or prefix", index);
    if (jb.degree < 1 || jb.degree > SC_MAX_DEGREE) return fail(TG_ERR_INVALID, "degree %d outside 1..=7", jb.degree);
    if (jb.ninstances < 1 || !jb.instances) return fail(TG_ERR_INVALID, "a batch needs at least one instance");
    for (int i = 0; i < jb.ninstances; i++) {
        const tg_instance& in = jb.instances[i];
        if (in.ntables < 1 || !in.tables) return fail(TG_ERR_INVALID, "instance %d has no table", i);
        if (in.ntables > jb.degree)
            return fail(TG_ERR_INVALID, "instance %d: a product of %d tables exceeds degree %d", i, in.ntables, jb.degree);
        if (in.vars < 0 || in.vars > SC_MAX_VARS) return fail(TG_ERR_INVALID, "instance %d: %d variables", i, in.vars);
        for (int k = 0; k < in.ntables; k++)
            if (!in.tables[k].values) return fail(TG_ERR_INVALID, "instance %d table %d: null values", i, k);
    }
    if (strlen(jb.prefix) > 160) return fail(TG_ERR_INVALID, "prefix longer than 160 characters");
    return TG_OK;
}

struct Plan {
    std::vector<std::pair<int, int>> who;  // (instance, own round, or −1 for a product sum)
    int blocks = 0;
};

// Whether the device takes cooperative launches (the persistent rounds' blocks must be co-resident).
static bool cooperative(Device* d) {
    if (d->coop < 0) {
        int v = 0;
        d->coop = cudaDeviceGetAttribute(&v, cudaDevAttrCooperativeLaunch, d->ordinal) == cudaSuccess && v ? 1 : 0;
    }
    return d->coop == 1;
}

// Blocks of sc_persist<D> that fit on one SM at once.
template <int D>
static int persist_blocks_per_sm() {
    static int nb = -1;
    if (nb < 0) {
        int v = 0;
        nb = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, sc_persist<D>, SC_THREADS, 0) == cudaSuccess ? v : 0;
    }
    return nb;
}

// One prove_many call in flight: planned on the host (γ drawn), then enqueued on a stream over
// a device arena, then finished on the host once the stream has run.
struct ScRun {
    ScOptions opts;
    tg_sumcheck_job* jobs = nullptr;
    int njobs = 0, tables_on_device = 0;
    std::vector<tg_transcript> saved;
    std::vector<InstState> inst;
    std::vector<int> n_max, inst0;
    std::vector<fp2> weights;
    int D = 1, J = 0, nevals = 0;
    size_t rounds_words = 0, chal_words = 0;
    std::vector<uint64_t> rounds_off, chal_off, evals_off;
    std::vector<Plan> plans;
    size_t max_segs = 1, max_blocks = 1, total_segs = 0, nbind = 0;
    int seg_cap = 1;
    int j0 = 0;  // rounds j0 … J − 1 are one block's work
    int jp = 0;  // rounds jp … J − 1 run in sc_persist (jp <= j0)
    ScPersist persist_h;
    std::vector<int> persist_first;
    int persist_grid = 1;  // sc_persist's blocks
    size_t persist_rows = 0;  // partial rows of sc_persist's largest multi-block round (two sets of them)
    // arena layout (offsets from the arena's base)
    size_t off_fs = 0, off_jobs = 0, off_w = 0, off_pad = 0, off_S = 0, off_msg = 0, off_rounds = 0, off_chal = 0,
           off_partials = 0, off_counters = 0, off_segs = 0, off_bind = 0, off_erefs = 0, off_evals = 0, off_persist = 0,
           off_first = 0, off_bar = 0, off_la = 0;
    std::vector<uint64_t*> la_ptrs;
    size_t arena_bytes = 0;
    // host-side staging that the enqueued copies read (kept until finish)
    std::vector<FsState> fs0;
    std::vector<FsJob> hj;
    std::vector<uint64_t> wv;
    std::vector<int> pads;
    std::vector<Seg> all_segs;
    std::vector<size_t> plan_seg0;
    std::vector<BindLast> binds;
    std::vector<EvalRef> erefs;
    // the host block the results come back into: FsState[njobs], rounds, challenges, evaluations
    size_t host_bytes = 0;
    const uint8_t* host_out = nullptr;
};

int sc_restore(ScRun* r, int rc) {
    for (int b = 0; b < r->njobs; b++) *r->jobs[b].transcript = r->saved[b];
    return rc;
}

ScRun* sc_prepare(Device* d, tg_sumcheck_job* jobs, int njobs, int tables_on_device, int* status,
                  const ScOptions& opts) {
    *status = TG_OK;
    if (njobs < 1 || !jobs) {
        *status = fail(TG_ERR_INVALID, "no sumcheck jobs");
        return nullptr;
    }
    for (int b = 0; b < njobs; b++) {
        *status = check_job(jobs[b], b);
        if (*status) return nullptr;
    }
    if (opts.weights && njobs != 1) {
        *status = fail(TG_ERR_INVALID, "caller weights are for one job");
        return nullptr;
    }
    ScRun* r = new ScRun();
    r->opts = opts;
    r->jobs = jobs;
    r->njobs = njobs;
    r->tables_on_device = tables_on_device;
    r->saved.resize(njobs);
    for (int b = 0; b < njobs; b++) r->saved[b] = *jobs[b].transcript;
    r->n_max.assign(njobs, 0);
    r->inst0.assign(njobs, 0);
    r->rounds_off.resize(njobs);
    r->chal_off.resize(njobs);
    r->evals_off.resize(njobs);

    // per job: γ (host transcript), weights; per instance: padding
    for (int b = 0; b < njobs; b++) {
        tg_sumcheck_job& jb = jobs[b];
        uint64_t g[2] = {jb.gamma[0], jb.gamma[1]};
        if (!opts.weights) {
            int rc = tg_transcript_challenge_fp2(jb.transcript, (std::string(jb.prefix) + "/gamma").c_str(), g);
            if (rc) {
                *status = sc_restore(r, rc);
                delete r;
                return nullptr;
            }
            jb.gamma[0] = g[0];
            jb.gamma[1] = g[1];
        } else if ((int)opts.weights->size() != jb.ninstances) {
            *status = sc_restore(r, fail(TG_ERR_INVALID, "one weight per instance"));
            delete r;
            return nullptr;
        }
        const fp2 gam = {g[0], g[1]};
        r->D = std::max(r->D, jb.degree);
        r->inst0[b] = (int)r->inst.size();
        for (int i = 0; i < jb.ninstances; i++) r->n_max[b] = std::max(r->n_max[b], jb.instances[i].vars);
        r->J = std::max(r->J, r->n_max[b]);
        fp2 acc = {1, 0};
        r->evals_off[b] = (uint64_t)r->nevals * 2;
        for (int i = 0; i < jb.ninstances; i++) {
            const tg_instance& src = jb.instances[i];
            InstState is;
            is.job = b;
            is.vars = src.vars;
            is.pad = r->n_max[b] - src.vars;
            for (int k = 0; k < src.ntables; k++) {
                TableState ts;
                if (tables_on_device)
                    ts.src = src.tables[k].values;
                else
                    ts.host = src.tables[k].values;
                ts.base = !src.tables[k].is_ext;
                ts.is_public = src.tables[k].is_public != 0;
                if (!ts.is_public) r->nevals++;
                is.tables.push_back(ts);
            }
            r->inst.push_back(std::move(is));
            r->weights.push_back(opts.weights ? (*opts.weights)[i] : acc);
            acc = e_mul(acc, gam);
        }
        r->rounds_off[b] = r->rounds_words;
        r->chal_off[b] = r->chal_words;
        r->rounds_words += (size_t)r->n_max[b] * 2 * jb.degree;
        r->chal_words += (size_t)r->n_max[b] * 2;
    }
    const int ninst = (int)r->inst.size();

    // the launches' segments, all planned before anything runs
    r->seg_cap = std::min(SC_MAX_SEG_BLOCKS, 4 * d->sm_count);
    const int seg_cap = r->seg_cap;
    auto blocks_for = [&](uint64_t n) {
        return (int)std::max<uint64_t>(1, std::min<uint64_t>((n + SC_THREADS - 1) / SC_THREADS, seg_cap));
    };
    r->plans.resize(1 + r->J);  // [0]: product sums, [1 + j]: round j
    for (int i = 0; i < ninst; i++)
        if (r->inst[i].pad > 0) r->plans[0].who.push_back({i, -1});
    for (int j = 0; j < r->J; j++)
        for (int i = 0; i < ninst; i++) {
            const int own = j - r->inst[i].pad;
            if (own >= 0 && own < r->inst[i].vars) r->plans[1 + j].who.push_back({i, own});
        }
    for (auto& p : r->plans) {
        for (auto& w : p.who) {
            const InstState& is = r->inst[w.first];
            const uint64_t n = w.second < 0 ? (1ull << is.vars) : (1ull << (is.vars - w.second - 1));
            p.blocks += blocks_for(n);
        }
        r->max_segs = std::max(r->max_segs, p.who.size());
        r->max_blocks = std::max(r->max_blocks, (size_t)p.blocks);
        r->total_segs += p.who.size();
    }
    auto plan_pairs = [&](int j) {
        uint64_t pairs = 0;
        for (auto& w : r->plans[1 + j].who) pairs += 1ull << (r->inst[w.first].vars - w.second - 1);
        return pairs;
    };
    const bool coop = cooperative(d);
    r->j0 = r->J;
    if (njobs <= SC_THREADS / 32)
        for (int j = r->J - 1; j >= 0 && plan_pairs(j) <= (coop ? SC_TAIL_PAIRS_PERSIST : SC_TAIL_PAIRS); j--) r->j0 = j;
    r->jp = r->j0;
    if (coop)
        for (int j = r->j0 - 1; j >= 0 && plan_pairs(j) <= SC_PERSIST_PAIRS; j--) r->jp = j;
    // the persistent launch's blocks, and the partial rows its multi-block rounds write
    size_t& persist_rows = r->persist_rows;
    if (r->jp < r->j0) {
        int per_sm = 0;
        with_degree(r->D, [&](auto D_) { per_sm = persist_blocks_per_sm<decltype(D_)::value>(); });
        // one block per SC_PERSIST_BLOCK_PAIRS pairs of the first round, but at least SC_PERSIST_MIN_BLOCKS
        // while each keeps SC_PERSIST_MIN_BLOCK_PAIRS (a small proof's first rounds are otherwise
        // a few blocks' long sums)
        const uint64_t p0 = plan_pairs(r->jp);
        const uint64_t want = std::max<uint64_t>(p0 / SC_PERSIST_BLOCK_PAIRS,
                                                 std::min<uint64_t>(SC_PERSIST_MIN_BLOCKS, p0 / SC_PERSIST_MIN_BLOCK_PAIRS));
        r->persist_grid = (int)std::max<uint64_t>(1, std::min<uint64_t>(want, (uint64_t)per_sm * d->sm_count));
        for (int j = r->jp; j < r->j0; j++) persist_rows = std::max(persist_rows, r->plans[1 + j].who.size() * r->persist_grid);
    }

    // the arena: tables, transcripts, plans and outputs
    Arena ar;
    for (auto& is : r->inst) {
        const size_t len = (size_t)1 << is.vars;
        for (auto& ts : is.tables) {
            ts.up_off = tables_on_device ? 0 : ar.take(len * (ts.base ? 8 : 16));
            ts.buf_off[0] = is.vars >= 1 ? ar.take(std::max<size_t>(len / 2, 1) * 16) : 0;
            ts.buf_off[1] = is.vars >= 2 ? ar.take(std::max<size_t>(len / 4, 1) * 16) : 0;
        }
    }
    r->off_fs = ar.take(sizeof(FsState) * njobs);
    r->off_jobs = ar.take(sizeof(FsJob) * njobs);
    r->off_w = ar.take(16 * ninst);
    r->off_pad = ar.take(4 * ninst);
    r->off_S = ar.take(16 * ninst);
    r->off_msg = ar.take((size_t)8 * SC_MSG_WORDS * ninst);
    r->off_rounds = ar.take(8 * std::max<size_t>(r->rounds_words, 1));
    r->off_chal = ar.take(8 * std::max<size_t>(r->chal_words, 1));
    r->off_partials = ar.take(std::max(r->max_blocks, 2 * persist_rows) * 2 * SC_MAX_DEGREE * 8);
    r->off_counters = ar.take(4 * r->max_segs);
    r->off_segs = ar.take(sizeof(Seg) * std::max<size_t>(r->total_segs, 1));
    r->off_persist = ar.take(sizeof(ScPersist));
    r->off_first = ar.take(4 * ((size_t)(r->J - r->jp) + 1));
    r->off_bar = ar.take(4 * SC_BAR_WORDS + 128);
    r->off_la = ar.take(2 * SC_MAX_TABLES * 8 + (size_t)SC_MAX_TABLES * 12 * 16);  // the look-ahead's warm-up tables
    for (auto& is : r->inst)
        if (is.vars >= 1) r->nbind += is.tables.size();
    r->off_bind = ar.take(sizeof(BindLast) * std::max<size_t>(r->nbind, 1));
    r->off_erefs = ar.take(sizeof(EvalRef) * std::max(r->nevals, 1));
    r->off_evals = ar.take(16 * std::max(r->nevals, 1));
    r->arena_bytes = ar.used;
    r->host_bytes = sizeof(FsState) * njobs + 8 * (r->rounds_words + r->chal_words) + 16 * (size_t)r->nevals;
    return r;
}

size_t sc_arena_bytes(const ScRun* r) { return r->arena_bytes; }
size_t sc_host_bytes(const ScRun* r) { return r->host_bytes; }
void sc_free(ScRun* r) { delete r; }

int sc_enqueue(Device* d, ScRun* r, cudaStream_t s, void* arena, void* host_out) {
    Arena ar;
    ar.base = (uint8_t*)arena;
    ar.used = r->arena_bytes;
    r->host_out = (const uint8_t*)host_out;
    const int njobs = r->njobs, ninst = (int)r->inst.size();
    tg_sumcheck_job* jobs = r->jobs;

    // tables: the current entries after `bound` binds are src (bound 0), else buf[(bound − 1) & 1]
    for (auto& is : r->inst)
        for (auto& ts : is.tables) {
            if (ts.host) {
                uint64_t* dst = ar.at<uint64_t>(ts.up_off);
                const size_t bytes = ((size_t)1 << is.vars) * (ts.base ? 8 : 16);
                host_prefault(ts.host, bytes);
                TG_CUDA(cudaMemcpyAsync(dst, ts.host, bytes, cudaMemcpyHostToDevice, s));
                ts.src = dst;
            }
        }
    auto cur = [&](const InstState& is, int k, int bound) -> const uint64_t* {
        return bound == 0 ? is.tables[k].src : ar.at<uint64_t>(is.tables[k].buf_off[(bound - 1) & 1]);
    };
    const int seg_cap = r->seg_cap;
    auto blocks_for = [&](uint64_t n) {
        return (int)std::max<uint64_t>(1, std::min<uint64_t>((n + SC_THREADS - 1) / SC_THREADS, seg_cap));
    };
    FsState* dfs = ar.at<FsState>(r->off_fs);
    uint64_t* dS = ar.at<uint64_t>(r->off_S);
    uint64_t* dmsg = ar.at<uint64_t>(r->off_msg);
    r->all_segs.clear();
    r->plan_seg0.clear();
    for (auto& p : r->plans) {
        r->plan_seg0.push_back(r->all_segs.size());
        int block0 = 0;
        for (auto& w : p.who) {
            const InstState& is = r->inst[w.first];
            Seg g;
            memset(&g, 0, sizeof g);
            g.nt = (int)is.tables.size();
            g.degree = jobs[is.job].degree;
            g.r = dfs[is.job].r;
            const int own = w.second;
            const int bound = own <= 0 ? 0 : own - 1;  // binds applied before this launch
            for (int k = 0; k < g.nt; k++) {
                g.src[k] = cur(is, k, bound);
                if (bound == 0 && is.tables[k].base) g.base_mask |= 1u << k;
            }
            if (own < 0) {
                g.kind = 1;
                g.n = 1ull << is.vars;
                g.out = dS + 2 * w.first;
            } else {
                g.kind = 0;
                g.n = 1ull << (is.vars - own - 1);
                g.out = dmsg + (size_t)w.first * SC_MSG_WORDS;
                if (own >= 1) {
                    g.bind = 1;
                    for (int k = 0; k < g.nt; k++) g.dst[k] = ar.at<uint64_t>(is.tables[k].buf_off[(own - 1) & 1]);
                }
            }
            const bool tail = &p - r->plans.data() >= 1 + r->j0;  // one block's work in sc_persist
            g.block0 = tail ? 0 : block0;
            g.nblocks = tail ? 1 : blocks_for(g.n);
            g.part0 = g.block0;
            g.inst = w.first;
            g.job = is.job;
            block0 += g.nblocks;
            r->all_segs.push_back(g);
        }
    }
    // the last own round's challenge, bound into one entry per table; then the final evaluations
    r->binds.clear();
    r->erefs.clear();
    for (auto& is : r->inst) {
        for (int k = 0; k < (int)is.tables.size(); k++) {
            const uint64_t* fin = is.tables[k].src;
            bool fin_base = is.tables[k].base;
            if (is.vars >= 1) {
                BindLast bl;
                memset(&bl, 0, sizeof bl);
                bl.src = cur(is, k, is.vars - 1);
                bl.base = is.vars == 1 && is.tables[k].base;
                bl.dst = ar.at<uint64_t>(is.tables[k].buf_off[(is.vars - 1) & 1]);
                bl.r = dfs[is.job].r;
                r->binds.push_back(bl);
                fin = bl.dst;
                fin_base = false;
            }
            if (!is.tables[k].is_public) {
                EvalRef e;
                memset(&e, 0, sizeof e);
                e.ptr = fin;
                e.base = fin_base;
                r->erefs.push_back(e);
            }
        }
    }

    // uploads: transcripts, jobs, weights, pads, plans
    r->fs0.assign(njobs, FsState());
    r->hj.assign(njobs, FsJob());
    FsKeys keys;
    context_key("transcript-absorb", keys.absorb);
    context_key("transcript-squeeze", keys.squeeze);
    context_key("transcript-ratchet", keys.ratchet);
    for (int b = 0; b < njobs; b++) {
        memset(&r->fs0[b], 0, sizeof(FsState));
        memcpy(r->fs0[b].state, jobs[b].transcript->state, 32);
        r->fs0[b].counter = jobs[b].transcript->counter;
        memset(&r->hj[b], 0, sizeof(FsJob));
        r->hj[b].label_len = (int)strlen(jobs[b].prefix);
        memcpy(r->hj[b].label, jobs[b].prefix, r->hj[b].label_len);
        r->hj[b].degree = jobs[b].degree;
        r->hj[b].ninst = jobs[b].ninstances;
        r->hj[b].n_max = r->n_max[b];
        r->hj[b].inst0 = r->inst0[b];
        r->hj[b].rounds_off = r->rounds_off[b];
        r->hj[b].chal_off = r->chal_off[b];
        for (int i = 0; i < jobs[b].ninstances; i++)
            r->hj[b].pad_max = std::max(r->hj[b].pad_max, r->inst[r->inst0[b] + i].pad);
    }
    r->wv.assign(2 * ninst, 0);
    r->pads.assign(ninst, 0);
    for (int i = 0; i < ninst; i++) {
        r->wv[2 * i] = r->weights[i].c0;
        r->wv[2 * i + 1] = r->weights[i].c1;
        r->pads[i] = r->inst[i].pad;
    }
    // The copies read host vectors of the run, which live until sc_free.
    TG_CUDA(cudaMemcpyAsync(dfs, r->fs0.data(), sizeof(FsState) * njobs, cudaMemcpyHostToDevice, s));
    TG_CUDA(cudaMemcpyAsync(ar.at<FsJob>(r->off_jobs), r->hj.data(), sizeof(FsJob) * njobs, cudaMemcpyHostToDevice, s));
    TG_CUDA(cudaMemcpyAsync(ar.at<uint64_t>(r->off_w), r->wv.data(), 16 * ninst, cudaMemcpyHostToDevice, s));
    TG_CUDA(cudaMemcpyAsync(ar.at<int>(r->off_pad), r->pads.data(), 4 * ninst, cudaMemcpyHostToDevice, s));
    if (!r->all_segs.empty())
        TG_CUDA(cudaMemcpyAsync(ar.at<Seg>(r->off_segs), r->all_segs.data(), sizeof(Seg) * r->all_segs.size(),
                                cudaMemcpyHostToDevice, s));
    if (!r->binds.empty())
        TG_CUDA(cudaMemcpyAsync(ar.at<BindLast>(r->off_bind), r->binds.data(), sizeof(BindLast) * r->binds.size(),
                                cudaMemcpyHostToDevice, s));
    if (!r->erefs.empty())
        TG_CUDA(cudaMemcpyAsync(ar.at<EvalRef>(r->off_erefs), r->erefs.data(), sizeof(EvalRef) * r->erefs.size(),
                                cudaMemcpyHostToDevice, s));
    TG_CUDA(cudaMemsetAsync(ar.at<unsigned>(r->off_counters), 0, 4 * r->max_segs, s));
    const int persist_grid = r->persist_grid;
    if (r->jp < r->J) {
        ScPersist& t = r->persist_h;
        memset(&t, 0, sizeof t);
        t.keys = keys;
        t.states = dfs;
        t.jobs = ar.at<FsJob>(r->off_jobs);
        t.w = ar.at<uint64_t>(r->off_w);
        t.pad = ar.at<int>(r->off_pad);
        t.S = dS;
        t.msgbuf = dmsg;
        t.rounds_out = ar.at<uint64_t>(r->off_rounds);
        t.chal_out = ar.at<uint64_t>(r->off_chal);
        t.segs = ar.at<Seg>(r->off_segs) + r->plan_seg0[1 + r->jp];
        t.first = ar.at<int>(r->off_first);
        t.partials = ar.at<uint64_t>(r->off_partials);
        t.bar = ar.at<unsigned>(r->off_bar);
        t.part_words = r->persist_rows * 2 * r->D;
        t.njobs = njobs;
        t.jp = r->jp;
        t.rounds = r->J - r->jp;
        t.multi = r->j0 - r->jp;
        // the look-ahead: one job of one instance (one segment a round) of D tables at degree D, from
        // the first one-block round of at most SC_LA_PAIRS pairs whose round before is one-block too
        // and whose tables were bound from Fp2 entries (round 2 on)
        t.la_from = -1;
        {  // the warm-up's tables (zeros): D sources of 8 Fp2 entries, then D destinations of 4
            uint8_t* base = ar.at<uint8_t>(r->off_la);
            uint64_t* data = reinterpret_cast<uint64_t*>(base + 2 * SC_MAX_TABLES * 8);
            r->la_ptrs.assign(2 * SC_MAX_TABLES, nullptr);
            for (int k = 0; k < r->D; k++) {
                r->la_ptrs[k] = data + 16 * k;
                r->la_ptrs[r->D + k] = data + 16 * SC_MAX_TABLES + 8 * k;
            }
            t.la_scratch = reinterpret_cast<uint64_t* const*>(base);
            TG_CUDA(cudaMemcpyAsync(base, r->la_ptrs.data(), 2 * SC_MAX_TABLES * 8, cudaMemcpyHostToDevice, s));
            TG_CUDA(cudaMemsetAsync(data, 0, (size_t)SC_MAX_TABLES * 12 * 16, s));
        }
        if (njobs == 1 && ninst == 1 && (r->D == 2 || r->D == 3) && jobs[0].degree == r->D &&
            (int)r->inst[0].tables.size() == r->D)
            for (int tt = t.rounds - 1; tt >= 1; tt--) {
                const int j = r->jp + tt;
                if (j < 2 || tt - 1 < t.multi || r->all_segs[r->plan_seg0[1 + j]].n > SC_LA_PAIRS) break;
                t.la_from = tt;
            }
        r->persist_first.assign(1, 0);
        for (int j = r->jp; j < r->J; j++) r->persist_first.push_back(r->persist_first.back() + (int)r->plans[1 + j].who.size());
        TG_CUDA(cudaMemcpyAsync(ar.at<ScPersist>(r->off_persist), &t, sizeof t, cudaMemcpyHostToDevice, s));
        TG_CUDA(cudaMemcpyAsync(ar.at<int>(r->off_first), r->persist_first.data(), 4 * r->persist_first.size(),
                                cudaMemcpyHostToDevice, s));
        TG_CUDA(cudaMemsetAsync(ar.at<unsigned>(r->off_bar), 0, 4 * SC_BAR_WORDS, s));
    }

    // the launches
    uint64_t* partials = ar.at<uint64_t>(r->off_partials);
    unsigned* counters = ar.at<unsigned>(r->off_counters);
    uint64_t* drounds = ar.at<uint64_t>(r->off_rounds);
    uint64_t* dchal = ar.at<uint64_t>(r->off_chal);
    auto run_plan = [&](int pi, const char* name) -> int {
        const Plan& p = r->plans[pi];
        if (p.who.empty()) return TG_OK;
        const Seg* segs = ar.at<Seg>(r->off_segs) + r->plan_seg0[pi];
        uint64_t units = 0;
        for (size_t q = 0; q < p.who.size(); q++) units += r->all_segs[r->plan_seg0[pi] + q].n;
        int shape = sc_shape(r->all_segs[r->plan_seg0[pi]]);
        for (size_t q = 1; q < p.who.size() && shape; q++)
            if (sc_shape(r->all_segs[r->plan_seg0[pi] + q]) != shape) shape = 0;
        Launch L(d, s, name, 1, units);
        const dim3 grid(p.blocks), block(SC_THREADS);
        const int nseg = (int)p.who.size();
        if (r->D == 3 && shape >= 1 && shape <= 3) {
            if (shape == 1) sc_rounds<3, 1><<<grid, block, 0, s>>>(segs, nseg, partials, counters);
            else if (shape == 2) sc_rounds<3, 2><<<grid, block, 0, s>>>(segs, nseg, partials, counters);
            else sc_rounds<3, 3><<<grid, block, 0, s>>>(segs, nseg, partials, counters);
        } else if (r->D == 2 && shape >= 4) {
            if (shape == 4) sc_rounds<2, 4><<<grid, block, 0, s>>>(segs, nseg, partials, counters);
            else if (shape == 5) sc_rounds<2, 5><<<grid, block, 0, s>>>(segs, nseg, partials, counters);
            else sc_rounds<2, 6><<<grid, block, 0, s>>>(segs, nseg, partials, counters);
        } else {
            with_degree(r->D, [&](auto D_) {
                constexpr int DD = decltype(D_)::value;
                sc_rounds<DD, 0><<<grid, block, 0, s>>>(segs, nseg, partials, counters);
            });
        }
        TG_CUDA(cudaGetLastError());
        return TG_OK;
    };
    int rc = run_plan(0, "sumcheck_product_sum");
    if (rc) return rc;
    for (int j = 0; j < r->jp; j++) {
        rc = run_plan(1 + j, "sumcheck_round");
        if (rc) return rc;
        {
            Launch L(d, s, "sumcheck_transcript", 1, njobs);
            with_degree(r->D, [&](auto D_) {
                constexpr int DD = decltype(D_)::value;
                sc_fs_many<DD><<<(njobs * 32 + FS_THREADS - 1) / FS_THREADS, FS_THREADS, 0, s>>>(
                    dfs, ar.at<FsJob>(r->off_jobs), njobs, j, keys, ar.at<uint64_t>(r->off_w), ar.at<int>(r->off_pad), dS,
                    dmsg, drounds, dchal);
            });
        }
        TG_CUDA(cudaGetLastError());
    }
    if (r->jp < r->J) {
        uint64_t units = 0;
        for (int j = r->jp; j < r->J; j++)
            for (size_t q = 0; q < r->plans[1 + j].who.size(); q++) units += r->all_segs[r->plan_seg0[1 + j] + q].n;
        Launch L(d, s, "sumcheck_persist", 1, units);
        const ScPersist* arg = ar.at<ScPersist>(r->off_persist);
        cudaError_t e = cudaSuccess;
        with_degree(r->D, [&](auto D_) {
            constexpr int DD = decltype(D_)::value;
            if (persist_grid > 1) {  // the blocks meet between rounds: all of them must be resident at once
                void* args[] = {(void*)&arg};
                e = cudaLaunchCooperativeKernel((const void*)sc_persist<DD>, dim3(persist_grid), dim3(SC_THREADS), args, 0,
                                                s);
            } else {
                sc_persist<DD><<<1, SC_THREADS, 0, s>>>(arg);
            }
        });
        if (e != cudaSuccess) return cuda_fail(e, "cudaLaunchCooperativeKernel(sc_persist)");
        TG_CUDA(cudaGetLastError());
    }
    if (!r->binds.empty()) {
        Launch L(d, s, "sumcheck_bind_last", 1, r->binds.size());
        sc_bind_last<<<(unsigned)((r->binds.size() + 127) / 128), 128, 0, s>>>(ar.at<BindLast>(r->off_bind),
                                                                               (int)r->binds.size());
        TG_CUDA(cudaGetLastError());
    }
    uint64_t* devals = ar.at<uint64_t>(r->off_evals);
    if (r->nevals) {
        Launch L(d, s, "sumcheck_evals", 1, r->nevals);
        sc_gather_evals<<<(r->nevals + 127) / 128, 128, 0, s>>>(ar.at<EvalRef>(r->off_erefs), r->nevals, devals);
        TG_CUDA(cudaGetLastError());
    }

    // one trip back: transcripts, rounds, challenges, evaluations
    uint8_t* h = (uint8_t*)host_out;
    TG_CUDA(cudaMemcpyAsync(h, dfs, sizeof(FsState) * njobs, cudaMemcpyDeviceToHost, s));
    h += sizeof(FsState) * njobs;
    if (r->rounds_words) TG_CUDA(cudaMemcpyAsync(h, drounds, r->rounds_words * 8, cudaMemcpyDeviceToHost, s));
    h += r->rounds_words * 8;
    if (r->chal_words) TG_CUDA(cudaMemcpyAsync(h, dchal, r->chal_words * 8, cudaMemcpyDeviceToHost, s));
    h += r->chal_words * 8;
    if (r->nevals) TG_CUDA(cudaMemcpyAsync(h, devals, (size_t)r->nevals * 16, cudaMemcpyDeviceToHost, s));
    return TG_OK;
}

// After the stream has run: errors, transcripts, outputs, and the evaluations absorbed.
int sc_finish(ScRun* r) {
    const int njobs = r->njobs;
    const FsState* fs1 = reinterpret_cast<const FsState*>(r->host_out);
    const uint8_t* h = r->host_out + sizeof(FsState) * njobs;
    const uint64_t* hr = reinterpret_cast<const uint64_t*>(h);
    const uint64_t* hc = hr + r->rounds_words;
    const uint64_t* he = hc + r->chal_words;
    for (int b = 0; b < njobs; b++) {
        if (fs1[b].err == 2)
            return sc_restore(r, fail(TG_ERR_STATE, "job %d: the persistent rounds' blocks gave up waiting for each other", b));
        if (fs1[b].err)
            return sc_restore(r, fail(TG_ERR_STATE, "job %d: a transcript challenge found no canonical Fp2 in %d squeezes",
                                      b, FS_MAX_TRIES));
    }
    for (int b = 0; b < njobs; b++) {
        tg_sumcheck_job& jb = r->jobs[b];
        memcpy(jb.transcript->state, fs1[b].state, 32);
        jb.transcript->counter = fs1[b].counter;
        const size_t nr = (size_t)r->n_max[b] * 2 * jb.degree;
        if (jb.rounds && nr) memcpy(jb.rounds, hr + r->rounds_off[b], nr * 8);
        if (jb.challenges && r->n_max[b]) memcpy(jb.challenges, hc + r->chal_off[b], (size_t)r->n_max[b] * 16);
        const size_t ne = (b + 1 < njobs ? r->evals_off[b + 1] : (uint64_t)2 * r->nevals) - r->evals_off[b];
        jb.n_evals = ne / 2;
        if (jb.final_evals && ne) memcpy(jb.final_evals, he + r->evals_off[b], ne * 8);
        if (!r->opts.absorb_evals) continue;
        const int rc = tg_transcript_absorb_fp2s(jb.transcript, (std::string(jb.prefix) + "/evals").c_str(),
                                                 he + r->evals_off[b], ne / 2);
        if (rc) return rc;
    }
    return TG_OK;
}

int prove_many_opts(Device* d, tg_sumcheck_job* jobs, int njobs, int tables_on_device, const ScOptions& opts) {
    int rc;
    ScRun* r = sc_prepare(d, jobs, njobs, tables_on_device, &rc, opts);
    if (!r) return rc;
    std::vector<uint8_t> host(r->host_bytes);
    {
        std::lock_guard<std::mutex> lock(d->mu);
        rc = d->scratch_sc.ensure(r->arena_bytes);
        if (!rc) rc = readback_ensure(d, r->host_bytes);
        // the outputs come back through the device's pinned readback (one wait, not a synchronous
        // copy each), then move to the run's own buffer before the lock is released
        if (!rc) rc = sc_enqueue(d, r, d->stream, d->scratch_sc.ptr, d->readback);
        if (!rc) {
            const cudaError_t e = cudaStreamSynchronize(d->stream);
            if (e != cudaSuccess) rc = cuda_fail(e, "cudaStreamSynchronize");
        }
        if (!rc) {
            memcpy(host.data(), d->readback, r->host_bytes);
            r->host_out = host.data();
        }
    }
    if (!rc) rc = sc_finish(r);
    else sc_restore(r, rc);
    sc_free(r);
    return rc;
}

static int prove_many(Device* d, tg_sumcheck_job* jobs, int njobs, int tables_on_device) {
    return prove_many_opts(d, jobs, njobs, tables_on_device, ScOptions());
}

}  // namespace tg

using namespace tg;

extern "C" int tg_prove_many(tg_device* dev, tg_sumcheck_job* jobs, int njobs, int tables_on_device) {
    Device* d = reinterpret_cast<Device*>(dev);
    if (!d) return fail(TG_ERR_INVALID, "tg_prove_many: null device");
    return prove_many(d, jobs, njobs, tables_on_device);
}

extern "C" int tg_prove_batch(tg_device* dev, tg_transcript* t, const char* prefix, int degree, const tg_instance* inst,
                              int ninst, int tables_on_device, uint64_t gamma[2], uint64_t* rounds, uint64_t* challenges,
                              uint64_t* final_evals, size_t* n_evals) {
    Device* d = reinterpret_cast<Device*>(dev);
    if (!d || !t || !prefix || !gamma || !n_evals) return fail(TG_ERR_INVALID, "tg_prove_batch: null argument");
    tg_sumcheck_job jb;
    memset(&jb, 0, sizeof jb);
    jb.transcript = t;
    jb.prefix = prefix;
    jb.degree = degree;
    jb.instances = inst;
    jb.ninstances = ninst;
    jb.rounds = rounds;
    jb.challenges = challenges;
    jb.final_evals = final_evals;
    const int rc = prove_many(d, &jb, 1, tables_on_device);
    if (rc) return rc;
    gamma[0] = jb.gamma[0];
    gamma[1] = jb.gamma[1];
    *n_evals = jb.n_evals;
    return TG_OK;
}

extern "C" int tg_check_grid_meet(tg_device* dev, int blocks, int meetings, int absent, uint32_t polls, int* met,
                                  int* gave_up) {
    Device* d = reinterpret_cast<Device*>(dev);
    if (!d || !met || !gave_up) return fail(TG_ERR_INVALID, "tg_check_grid_meet: null argument");
    if (blocks < 1 || blocks > d->sm_count || meetings < 0 || absent >= blocks || polls < 256)
        return fail(TG_ERR_INVALID, "tg_check_grid_meet: %d blocks, %d meetings, absent %d, %u polls", blocks, meetings,
                    absent, polls);
    if (!cooperative(d)) return fail(TG_ERR_STATE, "the device takes no cooperative launches");
    std::lock_guard<std::mutex> lock(d->mu);
    DevBuf b;
    int rc = b.ensure(4 * SC_BAR_WORDS + 8);
    if (rc) return rc;
    cudaStream_t s = d->stream;
    unsigned* bar = (unsigned*)b.ptr;
    unsigned* out = bar + SC_BAR_WORDS;
    TG_CUDA(cudaMemsetAsync(b.ptr, 0, 4 * SC_BAR_WORDS + 8, s));
    void* args[] = {(void*)&bar, (void*)&meetings, (void*)&absent, (void*)&polls, (void*)&out};
    TG_CUDA(cudaLaunchCooperativeKernel((const void*)grid_meet_check, dim3(blocks), dim3(SC_THREADS), args, 0, s));
    unsigned h[2] = {0, 0};
    TG_CUDA(cudaMemcpyAsync(h, out, 8, cudaMemcpyDeviceToHost, s));
    TG_CUDA(cudaStreamSynchronize(s));
    *met = (int)h[0];
    *gave_up = (int)h[1];
    return TG_OK;
}
