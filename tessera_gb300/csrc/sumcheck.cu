// SPDX-License-Identifier: Apache-2.0 OR MIT
//
// Batched sumcheck of products of multilinear tables on the device: the reference's prove_batch
// (crates/tessera-sumcheck/src/prover.rs:1122-1421) with its round sums and binds
// (crates/tessera-sumcheck/src/kernel.rs:90-101, 292-355, 591-633). Conventions (RFC-0010 as the
// reference applies them): x_1 is the index's least significant bit; round j binds x_j; the
// message is p(0), p(2), …, p(d); instance i weighs γ^i; an instance on fewer variables than the
// batch is front-padded and contributes 2^{n_max − n_i − j − 1}·S_i to each of its padding rounds.
//
// The rounds run without returning to the host. Each own round of an instance is one kernel: it
// binds the previous challenge into the tables (t'[i] = t[2i] + r·(t[2i+1] − t[2i])) and, in the
// same pass over the pairs of the new table, accumulates the d node sums; the last block to
// finish reduces the blocks' partial sums. A one-thread kernel then forms the round message
// (weights, padding terms), absorbs it into the Fiat–Shamir transcript and squeezes the next
// challenge with BLAKE3 on the device (crates/tessera-hash/src/transcript.rs:168-219), so the
// next round's kernel reads its challenge from device memory. γ is drawn on the host before the
// rounds and the final evaluations are absorbed on the host after them; the transcript state
// travels to the device and back once per batch.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <memory>
#include <string>
#include <vector>

#include "b3.cuh"
#include "gl.cuh"
#include "internal.h"

namespace tg {

constexpr int SC_MAX_TABLES = 7;
constexpr int SC_THREADS = 256;
constexpr int SC_MAX_BLOCKS = 1024;
constexpr int FS_MAX_TRIES = 64;  // squeezes per challenge before giving up (each retries with p < 2^-31)

// The transcript while it lives on the device.
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

struct FsLabel {
    char text[192];
    int len;
};

struct ScArgs {
    const uint64_t* src[SC_MAX_TABLES];  // current tables (or the tables to bind first)
    uint64_t* dst[SC_MAX_TABLES];        // bound tables (when bind)
    uint32_t base_mask;                  // bit k: table k's source holds prime-field words
    int nt;
    int degree;
    int bind;             // bind src by *r into dst first
    const uint64_t* r;    // the challenge, in device memory
    uint64_t npairs;      // pairs of the (bound) table
    uint64_t* partials;   // gridDim.x rows of words
    unsigned* counter;    // blocks finished; the last resets it
    uint64_t* out;        // the reduced sums as 2·degree Fp2 words
};

__device__ __forceinline__ fp2 load_entry(const uint64_t* t, bool base, uint64_t i) {
    if (base) return e_lift(t[i]);
    const ulonglong2 v = reinterpret_cast<const ulonglong2*>(t)[i];  // (c0, c1) words
    return {v.x, v.y};
}

__device__ __forceinline__ fp2 bind_pair(fp2 a, fp2 b, fp2 r, bool base) {
    if (base) {  // a, b in the prime field: two base products
        const uint64_t d = sub(b.c0, a.c0);
        return {add(a.c0, mul(r.c0, d)), mul(r.c1, d)};
    }
    return e_add(a, e_mul(r, e_sub(b, a)));
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

// Writes this block's NW words, and lets the last block to finish reduce all rows into a.out
// (as Fp2 words; prime-field sums are lifted when LIFT).
template <int NW, bool LIFT>
__device__ __forceinline__ void finish_partials(const ScArgs& a, uint64_t (&v)[NW]) {
    __shared__ bool last;
    if (threadIdx.x == 0) {
#pragma unroll
        for (int w = 0; w < NW; w++) a.partials[(size_t)blockIdx.x * NW + w] = v[w];
        __threadfence();
        last = atomicAdd(a.counter, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    uint64_t t[NW];
#pragma unroll
    for (int w = 0; w < NW; w++) t[w] = 0;
    for (unsigned b = threadIdx.x; b < gridDim.x; b += blockDim.x)
#pragma unroll
        for (int w = 0; w < NW; w++) t[w] = add(t[w], __ldcg(&a.partials[(size_t)b * NW + w]));
    block_sum<NW>(t);
    if (threadIdx.x == 0) {
        if (LIFT) {
            for (int w = 0; w < NW; w++) {
                a.out[2 * w] = t[w];
                a.out[2 * w + 1] = 0;
            }
        } else {
            for (int w = 0; w < NW; w++) a.out[w] = t[w];
        }
        *a.counter = 0;
    }
}

// All tables in the prime field and nothing to bind: products and sums in the prime field.
template <int D>
__global__ void __launch_bounds__(SC_THREADS) sc_round_base(ScArgs a) {
    uint64_t acc[D];
#pragma unroll
    for (int d = 0; d < D; d++) acc[d] = 0;
    for (uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; p < a.npairs; p += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t prod[D];
#pragma unroll
        for (int d = 0; d < D; d++) prod[d] = 1;
        for (int k = 0; k < a.nt; k++) {
            const ulonglong2 v = reinterpret_cast<const ulonglong2*>(a.src[k])[p];
            const uint64_t diff = sub(v.y, v.x);
            uint64_t x = v.y;  // value at node 1
            prod[0] = mul(prod[0], v.x);
#pragma unroll
            for (int d = 1; d < D; d++) {  // nodes 2..D
                x = add(x, diff);
                prod[d] = mul(prod[d], x);
            }
        }
#pragma unroll
        for (int d = 0; d < D; d++) acc[d] = add(acc[d], prod[d]);
    }
    block_sum<D>(acc);
    finish_partials<D, true>(a, acc);
}

// General round: Fp2 values (tables may mix prime-field and extension sources), binding first
// when a.bind.
template <int D>
__global__ void __launch_bounds__(SC_THREADS) sc_round_ext(ScArgs a) {
    fp2 acc[D];
#pragma unroll
    for (int d = 0; d < D; d++) acc[d] = {0, 0};
    const fp2 r = a.bind ? fp2{a.r[0], a.r[1]} : fp2{0, 0};
    for (uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; p < a.npairs; p += (uint64_t)gridDim.x * blockDim.x) {
        fp2 prod[D];
#pragma unroll
        for (int d = 0; d < D; d++) prod[d] = {1, 0};
        for (int k = 0; k < a.nt; k++) {
            const bool base = (a.base_mask >> k) & 1;
            fp2 u, v;
            if (a.bind) {
                u = bind_pair(load_entry(a.src[k], base, 4 * p), load_entry(a.src[k], base, 4 * p + 1), r, base);
                v = bind_pair(load_entry(a.src[k], base, 4 * p + 2), load_entry(a.src[k], base, 4 * p + 3), r, base);
                ulonglong2* out = reinterpret_cast<ulonglong2*>(a.dst[k]);
                out[2 * p] = make_ulonglong2(u.c0, u.c1);
                out[2 * p + 1] = make_ulonglong2(v.c0, v.c1);
            } else {
                u = load_entry(a.src[k], base, 2 * p);
                v = load_entry(a.src[k], base, 2 * p + 1);
            }
            const fp2 diff = e_sub(v, u);
            fp2 x = v;
            prod[0] = e_mul(prod[0], u);
#pragma unroll
            for (int d = 1; d < D; d++) {
                x = e_add(x, diff);
                prod[d] = e_mul(prod[d], x);
            }
        }
#pragma unroll
        for (int d = 0; d < D; d++) acc[d] = e_add(acc[d], prod[d]);
    }
    uint64_t words[2 * D];
#pragma unroll
    for (int d = 0; d < D; d++) {
        words[2 * d] = acc[d].c0;
        words[2 * d + 1] = acc[d].c1;
    }
    block_sum<2 * D>(words);
    finish_partials<2 * D, false>(a, words);
}

// Binds the last round (tables of two entries into one): dst[0] = bind(src[0], src[1]).
__global__ void sc_bind_last(ScArgs a) {
    const int k = threadIdx.x;
    if (k >= a.nt) return;
    const bool base = (a.base_mask >> k) & 1;
    const fp2 r = {a.r[0], a.r[1]};
    const fp2 u = bind_pair(load_entry(a.src[k], base, 0), load_entry(a.src[k], base, 1), r, base);
    reinterpret_cast<ulonglong2*>(a.dst[k])[0] = make_ulonglong2(u.c0, u.c1);
}

// Σ_x Π_k T_k[x] over a whole table set (a padded instance's S_i), into a.out as one Fp2.
__global__ void __launch_bounds__(SC_THREADS) sc_product_sum(ScArgs a, uint64_t len) {
    fp2 acc = {0, 0};
    for (uint64_t x = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; x < len; x += (uint64_t)gridDim.x * blockDim.x) {
        fp2 prod = {1, 0};
        for (int k = 0; k < a.nt; k++) prod = e_mul(prod, load_entry(a.src[k], (a.base_mask >> k) & 1, x));
        acc = e_add(acc, prod);
    }
    uint64_t w[2] = {acc.c0, acc.c1};
    block_sum<2>(w);
    finish_partials<2, false>(a, w);
}

// ---- the transcript on the device (one thread) --------------------------------------------------

__device__ void fs_hash(const uint32_t key[8], const uint8_t* msg, uint32_t len, uint8_t out[32]) {
    uint32_t h[8];
    for (int i = 0; i < 8; i++) h[i] = key[i];
    const uint32_t nb = len == 0 ? 1 : (len + 63) / 64;
    for (uint32_t b = 0; b < nb; b++) {
        uint32_t m[16];
        for (int i = 0; i < 16; i++) {
            uint32_t w = 0;
            for (int k = 0; k < 4; k++) {
                const uint32_t at = 64 * b + 4 * i + k;
                if (at < len) w |= (uint32_t)msg[at] << (8 * k);
            }
            m[i] = w;
        }
        const bool last = b + 1 == nb;
        b3::compress_cv(h, m, 0, last ? len - 64 * b : 64,
                        b3::DERIVE_KEY_MATERIAL | (b == 0 ? b3::CHUNK_START : 0) | (last ? (b3::CHUNK_END | b3::ROOT) : 0));
    }
    for (int i = 0; i < 32; i++) out[i] = (uint8_t)(h[i / 4] >> (8 * (i % 4)));
}

__device__ __forceinline__ void put64(uint8_t* p, uint64_t v) {
    for (int i = 0; i < 8; i++) p[i] = (uint8_t)(v >> (8 * i));
}

// state ‖ u64 len(label) ‖ label, label = prefix ‖ tail ‖ decimal j; returns the length.
__device__ uint32_t fs_begin(const FsState* t, const FsLabel& pre, const char* tail, int j, uint8_t* buf) {
    char lab[256];
    int n = 0;
    for (int i = 0; i < pre.len; i++) lab[n++] = pre.text[i];
    for (const char* c = tail; *c; c++) lab[n++] = *c;
    char digits[12];
    int nd = 0;
    do {
        digits[nd++] = (char)('0' + j % 10);
        j /= 10;
    } while (j > 0);
    while (nd > 0) lab[n++] = digits[--nd];
    for (int i = 0; i < 32; i++) buf[i] = t->state[i];
    put64(buf + 32, (uint64_t)n);
    for (int i = 0; i < n; i++) buf[40 + i] = (uint8_t)lab[i];
    return 40 + n;
}

// Round j's message: Σ over instances of w_i·(own sums, or 2^{pad_i − j − 1}·S_i while padded),
// absorbed as TCE Vec<Fp2> under <prefix>/round/j; then r_j = challenge_fp2(<prefix>/r/j).
__global__ void sc_fs_round(FsState* t, FsKeys keys, FsLabel pre, int j, int degree, int ninst, const uint64_t* w,
                            const int* pad, const uint64_t* S, const uint64_t* msgbuf, uint64_t* rounds_out,
                            uint64_t* chal_out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    fp2 msg[8];
    for (int x = 0; x < degree; x++) msg[x] = {0, 0};
    for (int i = 0; i < ninst; i++) {
        const fp2 wi = {w[2 * i], w[2 * i + 1]};
        if (j < pad[i]) {
            const fp2 v = e_mul(wi, e_scale(fp2{S[2 * i], S[2 * i + 1]}, (1ull << (pad[i] - j - 1)) % P));
            for (int x = 0; x < degree; x++) msg[x] = e_add(msg[x], v);
        } else {
            const uint64_t* m = msgbuf + (size_t)i * 2 * degree;
            for (int x = 0; x < degree; x++) msg[x] = e_add(msg[x], e_mul(wi, fp2{m[2 * x], m[2 * x + 1]}));
        }
    }
    uint8_t buf[512];
    uint32_t len = fs_begin(t, pre, "/round/", j, buf);
    put64(buf + len, (uint64_t)degree);
    len += 8;
    for (int x = 0; x < degree; x++) {
        put64(buf + len, msg[x].c0);
        put64(buf + len + 8, msg[x].c1);
        len += 16;
        rounds_out[(size_t)j * 2 * degree + 2 * x] = msg[x].c0;
        rounds_out[(size_t)j * 2 * degree + 2 * x + 1] = msg[x].c1;
    }
    fs_hash(keys.absorb, buf, len, t->state);
    for (int tries = 0; tries < FS_MAX_TRIES; tries++) {
        len = fs_begin(t, pre, "/r/", j, buf);
        put64(buf + len, t->counter);
        uint8_t out[32];
        fs_hash(keys.squeeze, buf, len + 8, out);
        t->counter += 1;
        uint8_t rb[64];
        for (int i = 0; i < 32; i++) {
            rb[i] = t->state[i];
            rb[32 + i] = out[i];
        }
        fs_hash(keys.ratchet, rb, 64, t->state);
        uint64_t c0 = 0, c1 = 0;
        for (int i = 7; i >= 0; i--) {
            c0 = (c0 << 8) | out[i];
            c1 = (c1 << 8) | out[8 + i];
        }
        if (c0 < P && c1 < P) {
            t->r[0] = c0;
            t->r[1] = c1;
            chal_out[2 * j] = c0;
            chal_out[2 * j + 1] = c1;
            return;
        }
    }
    t->err = 1;
}

// Each table's single entry after the last bind (public factors left out), as Fp2 words.
__global__ void sc_gather_evals(const uint64_t* const* ptrs, const int* is_base, int n, uint64_t* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    out[2 * i] = ptrs[i][0];
    out[2 * i + 1] = is_base[i] ? 0 : ptrs[i][1];
}

// ---- host driver -----------------------------------------------------------------------------

static int grid_for(uint64_t items, const Device* d) {
    uint64_t g = (items + SC_THREADS - 1) / SC_THREADS;
    const uint64_t cap = std::min<uint64_t>(SC_MAX_BLOCKS, (uint64_t)d->sm_count * 4);
    if (g > cap) g = cap;
    return (int)(g ? g : 1);
}

struct ScTable {
    const uint64_t* src = nullptr;  // original entries (device)
    bool base = false, is_public = false;
    uint64_t* buf[2] = {nullptr, nullptr};  // ping-pong bound tables
    const uint64_t* cur = nullptr;          // current entries
    bool cur_base = false;
};

struct ScInstance {
    int vars = 0;
    std::vector<ScTable> tables;
};

static void fill_args(ScArgs& a, const ScInstance& in, int degree) {
    memset(&a, 0, sizeof a);
    a.nt = (int)in.tables.size();
    a.degree = degree;
    for (int k = 0; k < a.nt; k++) {
        a.src[k] = in.tables[k].cur;
        if (in.tables[k].cur_base) a.base_mask |= 1u << k;
    }
}

// A bump allocator over one device buffer, 256-byte aligned pieces.
struct Arena {
    size_t used = 0;
    uint8_t* base = nullptr;
    size_t take(size_t bytes) {
        const size_t at = used;
        used += (bytes + 255) & ~(size_t)255;
        return at;
    }
    template <typename T>
    T* at(size_t off) const {
        return reinterpret_cast<T*>(base + off);
    }
};

template <typename F>
static int with_degree(int degree, F&& f) {
    switch (degree) {
        case 1: return f(std::integral_constant<int, 1>{});
        case 2: return f(std::integral_constant<int, 2>{});
        case 3: return f(std::integral_constant<int, 3>{});
        case 4: return f(std::integral_constant<int, 4>{});
        case 5: return f(std::integral_constant<int, 5>{});
        case 6: return f(std::integral_constant<int, 6>{});
        default: return f(std::integral_constant<int, 7>{});
    }
}

}  // namespace tg

using namespace tg;

extern "C" int tg_prove_batch(tg_device* dev, tg_transcript* t, const char* prefix, int degree, const tg_instance* inst,
                              int ninst, int tables_on_device, uint64_t gamma[2], uint64_t* rounds, uint64_t* challenges,
                              uint64_t* final_evals, size_t* n_evals) {
    Device* d = reinterpret_cast<Device*>(dev);
    if (!d || !t || !prefix || !gamma || !n_evals) return fail(TG_ERR_INVALID, "tg_prove_batch: null argument");
    // check_batch (prover.rs:1196-1218), in its order: degree, instances, then each instance.
    if (degree < 1 || degree > 7) return fail(TG_ERR_INVALID, "degree %d outside 1..=7", degree);
    if (ninst < 1 || !inst) return fail(TG_ERR_INVALID, "a batch needs at least one instance");
    int n_max = 0;
    for (int i = 0; i < ninst; i++) {
        if (inst[i].ntables < 1 || !inst[i].tables) return fail(TG_ERR_INVALID, "instance %d has no table", i);
        if (inst[i].ntables > degree)
            return fail(TG_ERR_INVALID, "instance %d: a product of %d tables exceeds degree %d", i, inst[i].ntables, degree);
        if (inst[i].vars < 0 || inst[i].vars > 40) return fail(TG_ERR_INVALID, "instance %d: %d variables", i, inst[i].vars);
        for (int k = 0; k < inst[i].ntables; k++)
            if (!inst[i].tables[k].values) return fail(TG_ERR_INVALID, "instance %d table %d: null values", i, k);
        n_max = std::max(n_max, inst[i].vars);
    }
    const size_t plen = strlen(prefix);
    if (plen > 160) return fail(TG_ERR_INVALID, "prefix longer than 160 characters");
    std::lock_guard<std::mutex> lock(d->mu);
    cudaStream_t s = d->stream;
    const std::string pre(prefix);
    uint64_t g[2];
    int rc = tg_transcript_challenge_fp2(t, (pre + "/gamma").c_str(), g);
    if (rc) return rc;
    gamma[0] = g[0];
    gamma[1] = g[1];
    const fp2 gam = {g[0], g[1]};

    // ---- device memory: one arena for tables, state and outputs
    Arena ar;
    std::vector<ScInstance> st(ninst);
    std::vector<size_t> up_off, buf_off;  // per table, in order
    int nevals = 0;
    for (int i = 0; i < ninst; i++) {
        const size_t len = (size_t)1 << inst[i].vars;
        for (int k = 0; k < inst[i].ntables; k++) {
            const tg_table& src = inst[i].tables[k];
            up_off.push_back(tables_on_device ? 0 : ar.take(len * (src.is_ext ? 16 : 8)));
            buf_off.push_back(inst[i].vars >= 1 ? ar.take(std::max<size_t>(len / 2, 1) * 16) : 0);
            buf_off.push_back(inst[i].vars >= 2 ? ar.take(std::max<size_t>(len / 4, 1) * 16) : 0);
            if (!src.is_public) nevals++;
        }
    }
    const size_t off_fs = ar.take(sizeof(FsState));
    const size_t off_w = ar.take(16 * ninst), off_pad = ar.take(4 * ninst), off_S = ar.take(16 * ninst);
    const size_t off_msg = ar.take((size_t)16 * degree * ninst);
    const size_t off_rounds = ar.take((size_t)16 * degree * std::max(n_max, 1));
    const size_t off_chal = ar.take((size_t)16 * std::max(n_max, 1));
    const size_t off_partials = ar.take((size_t)SC_MAX_BLOCKS * 16 * 8);
    const size_t off_counter = ar.take(16);
    const size_t off_evals = ar.take((size_t)16 * std::max(nevals, 1));
    const size_t off_eptr = ar.take(sizeof(uint64_t*) * std::max(nevals, 1));
    const size_t off_ebase = ar.take(4 * std::max(nevals, 1));
    rc = d->scratch_sc.ensure(ar.used);
    if (rc) return rc;
    ar.base = (uint8_t*)d->scratch_sc.ptr;

    // tables
    std::vector<fp2> w(ninst);
    std::vector<int> pad(ninst);
    fp2 acc = {1, 0};
    size_t ti = 0;
    for (int i = 0; i < ninst; i++) {
        w[i] = acc;
        acc = e_mul(acc, gam);
        st[i].vars = inst[i].vars;
        pad[i] = n_max - inst[i].vars;
        const size_t len = (size_t)1 << inst[i].vars;
        for (int k = 0; k < inst[i].ntables; k++, ti++) {
            const tg_table& src = inst[i].tables[k];
            ScTable tb;
            tb.base = !src.is_ext;
            tb.is_public = src.is_public != 0;
            if (tables_on_device) {
                tb.src = src.values;
            } else {
                uint64_t* dst = ar.at<uint64_t>(up_off[ti]);
                TG_CUDA(cudaMemcpyAsync(dst, src.values, len * (tb.base ? 8 : 16), cudaMemcpyHostToDevice, s));
                tb.src = dst;
            }
            tb.buf[0] = inst[i].vars >= 1 ? ar.at<uint64_t>(buf_off[2 * ti]) : nullptr;
            tb.buf[1] = inst[i].vars >= 2 ? ar.at<uint64_t>(buf_off[2 * ti + 1]) : nullptr;
            tb.cur = tb.src;
            tb.cur_base = tb.base;
            st[i].tables.push_back(tb);
        }
    }
    // transcript state, weights, padding
    FsState fs0;
    memset(&fs0, 0, sizeof fs0);
    memcpy(fs0.state, t->state, 32);
    fs0.counter = t->counter;
    FsState* fs = ar.at<FsState>(off_fs);
    TG_CUDA(cudaMemcpyAsync(fs, &fs0, sizeof fs0, cudaMemcpyHostToDevice, s));
    std::vector<uint64_t> wv(2 * ninst);
    for (int i = 0; i < ninst; i++) {
        wv[2 * i] = w[i].c0;
        wv[2 * i + 1] = w[i].c1;
    }
    uint64_t* dw = ar.at<uint64_t>(off_w);
    int* dpad = ar.at<int>(off_pad);
    uint64_t* dS = ar.at<uint64_t>(off_S);
    uint64_t* dmsg = ar.at<uint64_t>(off_msg);
    uint64_t* drounds = ar.at<uint64_t>(off_rounds);
    uint64_t* dchal = ar.at<uint64_t>(off_chal);
    TG_CUDA(cudaMemcpyAsync(dw, wv.data(), 16 * ninst, cudaMemcpyHostToDevice, s));
    TG_CUDA(cudaMemcpyAsync(dpad, pad.data(), 4 * ninst, cudaMemcpyHostToDevice, s));
    TG_CUDA(cudaMemsetAsync(ar.at<unsigned>(off_counter), 0, 16, s));
    FsKeys keys;
    context_key("transcript-absorb", keys.absorb);
    context_key("transcript-squeeze", keys.squeeze);
    context_key("transcript-ratchet", keys.ratchet);
    FsLabel label;
    memset(&label, 0, sizeof label);
    memcpy(label.text, prefix, plen);
    label.len = (int)plen;

    auto base_args = [&](ScArgs& a, uint64_t* out) {
        a.r = fs->r;
        a.partials = ar.at<uint64_t>(off_partials);
        a.counter = ar.at<unsigned>(off_counter);
        a.out = out;
    };

    // padded instances' full sums S_i
    for (int i = 0; i < ninst; i++) {
        if (st[i].vars >= n_max) continue;
        ScArgs a;
        fill_args(a, st[i], degree);
        base_args(a, dS + 2 * i);
        const uint64_t len = 1ull << st[i].vars;
        const int grid = grid_for(len, d);
        Launch L(d, s, "sumcheck_product_sum", 1, len);
        sc_product_sum<<<grid, SC_THREADS, 0, s>>>(a, len);
        TG_CUDA(cudaGetLastError());
    }

    std::vector<int> pending(ninst, 0);  // own rounds whose challenge is not bound yet
    for (int j = 0; j < n_max; j++) {
        for (int i = 0; i < ninst; i++) {
            if (j < pad[i]) continue;
            const int own = j - pad[i];
            ScInstance& in = st[i];
            ScArgs a;
            fill_args(a, in, degree);
            base_args(a, dmsg + (size_t)i * 2 * degree);
            a.npairs = 1ull << (in.vars - own - 1);
            bool all_base = true;
            for (auto& tb : in.tables) all_base &= tb.cur_base;
            if (pending[i]) {
                a.bind = 1;
                for (int k = 0; k < a.nt; k++) a.dst[k] = in.tables[k].buf[(own - 1) & 1];
            }
            const int grid = grid_for(a.npairs, d);
            {
                Launch L(d, s, "sumcheck_round", 1, a.npairs);
                with_degree(degree, [&](auto D_) {
                    constexpr int D = decltype(D_)::value;
                    if (all_base && !a.bind)
                        sc_round_base<D><<<grid, SC_THREADS, 0, s>>>(a);
                    else
                        sc_round_ext<D><<<grid, SC_THREADS, 0, s>>>(a);
                    return 0;
                });
            }
            TG_CUDA(cudaGetLastError());
            if (a.bind) {
                for (int k = 0; k < a.nt; k++) {
                    in.tables[k].cur = a.dst[k];
                    in.tables[k].cur_base = false;
                }
            }
            pending[i] = 1;
        }
        {
            Launch L(d, s, "sumcheck_transcript", 1, 1);
            sc_fs_round<<<1, 32, 0, s>>>(fs, keys, label, j, degree, ninst, dw, dpad, dS, dmsg, drounds, dchal);
        }
        TG_CUDA(cudaGetLastError());
    }
    // the last own round's challenge, bound into one entry per table
    for (int i = 0; i < ninst; i++) {
        ScInstance& in = st[i];
        if (!pending[i]) continue;
        ScArgs a;
        fill_args(a, in, degree);
        base_args(a, nullptr);
        for (int k = 0; k < a.nt; k++) a.dst[k] = in.tables[k].buf[(in.vars - 1) & 1];
        {
            Launch L(d, s, "sumcheck_bind_last", 1, 1);
            sc_bind_last<<<1, 32, 0, s>>>(a);
        }
        TG_CUDA(cudaGetLastError());
        for (int k = 0; k < a.nt; k++) {
            in.tables[k].cur = a.dst[k];
            in.tables[k].cur_base = false;
        }
    }
    // final evaluations: each table's single entry, public factors left out
    std::vector<const uint64_t*> eptr;
    std::vector<int> ebase;
    for (int i = 0; i < ninst; i++)
        for (auto& tb : st[i].tables)
            if (!tb.is_public) {
                eptr.push_back(tb.cur);
                ebase.push_back(tb.cur_base ? 1 : 0);
            }
    uint64_t* devals = ar.at<uint64_t>(off_evals);
    if (nevals) {
        TG_CUDA(cudaMemcpyAsync(ar.at<uint64_t*>(off_eptr), eptr.data(), sizeof(uint64_t*) * nevals, cudaMemcpyHostToDevice, s));
        TG_CUDA(cudaMemcpyAsync(ar.at<int>(off_ebase), ebase.data(), 4 * nevals, cudaMemcpyHostToDevice, s));
        Launch L(d, s, "sumcheck_evals", 1, nevals);
        sc_gather_evals<<<(nevals + 127) / 128, 128, 0, s>>>(ar.at<const uint64_t* const>(off_eptr), ar.at<int>(off_ebase),
                                                              nevals, devals);
        TG_CUDA(cudaGetLastError());
    }
    // one trip back: transcript, rounds, challenges, evaluations
    FsState fs1;
    std::vector<uint64_t> hr((size_t)2 * degree * n_max), hc((size_t)2 * n_max), he((size_t)2 * nevals);
    TG_CUDA(cudaMemcpyAsync(&fs1, fs, sizeof fs1, cudaMemcpyDeviceToHost, s));
    if (n_max) {
        TG_CUDA(cudaMemcpyAsync(hr.data(), drounds, hr.size() * 8, cudaMemcpyDeviceToHost, s));
        TG_CUDA(cudaMemcpyAsync(hc.data(), dchal, hc.size() * 8, cudaMemcpyDeviceToHost, s));
    }
    if (nevals) TG_CUDA(cudaMemcpyAsync(he.data(), devals, he.size() * 8, cudaMemcpyDeviceToHost, s));
    TG_CUDA(cudaStreamSynchronize(s));
    if (fs1.err) return fail(TG_ERR_STATE, "a transcript challenge found no canonical Fp2 in %d squeezes", FS_MAX_TRIES);
    memcpy(t->state, fs1.state, 32);
    t->counter = fs1.counter;
    if (rounds && n_max) memcpy(rounds, hr.data(), hr.size() * 8);
    if (challenges && n_max) memcpy(challenges, hc.data(), hc.size() * 8);
    *n_evals = (size_t)nevals;
    if (final_evals && nevals) memcpy(final_evals, he.data(), he.size() * 8);
    return tg_transcript_absorb_fp2s(t, (pre + "/evals").c_str(), he.data(), (size_t)nevals);
}
