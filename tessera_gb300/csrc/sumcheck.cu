// SPDX-License-Identifier: Apache-2.0 OR MIT
//
// Batched sumcheck of products of multilinear tables on the device: the reference's prove_batch
// (crates/tessera-sumcheck/src/prover.rs:1122-1421) with its round sums and binds
// (crates/tessera-sumcheck/src/kernel.rs:90-101, 292-355, 591-633). Conventions (RFC-0010 as the
// reference applies them): x_1 is the index's least significant bit; round j binds x_j; the
// message is p(0), p(2), …, p(d); instance i weighs γ^i; an instance on fewer variables than the
// batch is front-padded and contributes 2^{n_max − n_i − j − 1}·S_i to each of its padding rounds.
//
// Each own round is one fused kernel: it binds the previous round's challenge into the tables
// (t'[i] = t[2i] + r·(t[2i+1] − t[2i])) and, in the same pass over the pairs of the new table,
// accumulates the d node sums; a first round over prime-field tables multiplies in the prime
// field only. Block partials are reduced in a second kernel, and the d sums go to the host
// transcript, which draws the next challenge.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <memory>
#include <string>
#include <vector>

#include "gl.cuh"
#include "internal.h"

namespace tg {

constexpr int SC_MAX_TABLES = 7;
constexpr int SC_THREADS = 256;
constexpr int SC_MAX_BLOCKS = 1024;

struct ScArgs {
    const uint64_t* src[SC_MAX_TABLES];  // current tables (or the tables to bind first)
    uint64_t* dst[SC_MAX_TABLES];        // bound tables (when bind)
    uint32_t base_mask;                  // bit k: table k's source holds prime-field words
    int nt;
    int degree;
    int bind;       // bind src by r into dst first
    fp2 r;
    uint64_t npairs;  // pairs of the (bound) table
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

// Block-level sum of `nwords` per-thread words in shared memory; thread 0 writes the result.
__device__ void block_sum_words(uint64_t* vals, int nwords, uint64_t* out) {
    extern __shared__ uint64_t red[];  // blockDim.x * nwords
    for (int w = 0; w < nwords; w++) red[w * blockDim.x + threadIdx.x] = vals[w];
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s)
            for (int w = 0; w < nwords; w++)
                red[w * blockDim.x + threadIdx.x] = add(red[w * blockDim.x + threadIdx.x], red[w * blockDim.x + threadIdx.x + s]);
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int w = 0; w < nwords; w++) out[w] = red[w * blockDim.x];
}

// All tables in the prime field and nothing to bind: products and sums in the prime field.
// partials: gridDim.x x degree words.
__global__ void __launch_bounds__(SC_THREADS) sc_round_base(ScArgs a, uint64_t* partials) {
    uint64_t acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; p < a.npairs; p += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t prod[8];
        for (int d = 0; d < a.degree; d++) prod[d] = 1;
        for (int k = 0; k < a.nt; k++) {
            const ulonglong2 v = reinterpret_cast<const ulonglong2*>(a.src[k])[p];
            const uint64_t diff = sub(v.y, v.x);
            uint64_t x = v.y;  // value at node 1
            prod[0] = mul(prod[0], v.x);
            for (int d = 1; d < a.degree; d++) {  // nodes 2..degree
                x = add(x, diff);
                prod[d] = mul(prod[d], x);
            }
        }
        for (int d = 0; d < a.degree; d++) acc[d] = add(acc[d], prod[d]);
    }
    block_sum_words(acc, a.degree, partials + (size_t)blockIdx.x * a.degree);
}

// General round: Fp2 values (tables may mix prime-field and extension sources), optionally
// binding first. partials: gridDim.x x 2·degree words.
__global__ void __launch_bounds__(SC_THREADS) sc_round_ext(ScArgs a, uint64_t* partials) {
    fp2 acc[8];
    for (int d = 0; d < 8; d++) acc[d] = {0, 0};
    for (uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; p < a.npairs; p += (uint64_t)gridDim.x * blockDim.x) {
        fp2 prod[8];
        for (int d = 0; d < a.degree; d++) prod[d] = {1, 0};
        for (int k = 0; k < a.nt; k++) {
            const bool base = (a.base_mask >> k) & 1;
            fp2 u, v;
            if (a.bind) {
                u = bind_pair(load_entry(a.src[k], base, 4 * p), load_entry(a.src[k], base, 4 * p + 1), a.r, base);
                v = bind_pair(load_entry(a.src[k], base, 4 * p + 2), load_entry(a.src[k], base, 4 * p + 3), a.r, base);
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
            for (int d = 1; d < a.degree; d++) {
                x = e_add(x, diff);
                prod[d] = e_mul(prod[d], x);
            }
        }
        for (int d = 0; d < a.degree; d++) acc[d] = e_add(acc[d], prod[d]);
    }
    uint64_t words[16];
    for (int d = 0; d < a.degree; d++) {
        words[2 * d] = acc[d].c0;
        words[2 * d + 1] = acc[d].c1;
    }
    block_sum_words(words, 2 * a.degree, partials + (size_t)blockIdx.x * 2 * a.degree);
}

// Binds the last round (tables of two entries into one): dst[0] = bind(src[0], src[1]).
__global__ void sc_bind_last(ScArgs a) {
    const int k = threadIdx.x;
    if (k >= a.nt) return;
    const bool base = (a.base_mask >> k) & 1;
    const fp2 u = bind_pair(load_entry(a.src[k], base, 0), load_entry(a.src[k], base, 1), a.r, base);
    reinterpret_cast<ulonglong2*>(a.dst[k])[0] = make_ulonglong2(u.c0, u.c1);
}

// Σ_x Π_k T_k[x] over a whole table set (a padded instance's S_i). partials: grid x 2 words.
__global__ void __launch_bounds__(SC_THREADS) sc_product_sum(ScArgs a, uint64_t len, uint64_t* partials) {
    fp2 acc = {0, 0};
    for (uint64_t x = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; x < len; x += (uint64_t)gridDim.x * blockDim.x) {
        fp2 prod = {1, 0};
        for (int k = 0; k < a.nt; k++) prod = e_mul(prod, load_entry(a.src[k], (a.base_mask >> k) & 1, x));
        acc = e_add(acc, prod);
    }
    uint64_t w[2] = {acc.c0, acc.c1};
    block_sum_words(w, 2, partials + 2 * (size_t)blockIdx.x);
}

// Sums `nblocks` rows of `nwords` words.
__global__ void sc_reduce(const uint64_t* partials, int nblocks, int nwords, uint64_t* out) {
    uint64_t v[16];
    for (int w = 0; w < nwords; w++) v[w] = 0;
    for (int b = threadIdx.x; b < nblocks; b += blockDim.x)
        for (int w = 0; w < nwords; w++) v[w] = add(v[w], partials[(size_t)b * nwords + w]);
    block_sum_words(v, nwords, out);
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
    DevBuf upload;        // the host table's copy, when the caller passed host memory
    DevBuf buf[2];        // ping-pong bound tables
    const uint64_t* cur = nullptr;  // current entries
    bool cur_base = false;
};

struct ScInstance {
    int vars = 0;
    std::vector<std::unique_ptr<ScTable>> tables;
};

static int reduce_to_host(Device* d, cudaStream_t s, uint64_t* partials, int grid, int nwords, uint64_t* host_out) {
    uint64_t* dev_out = partials + (size_t)grid * nwords;
    Launch L(d, s, "sumcheck_reduce", 1, grid);
    sc_reduce<<<1, SC_THREADS, SC_THREADS * nwords * 8, s>>>(partials, grid, nwords, dev_out);
    TG_CUDA(cudaGetLastError());
    TG_CUDA(cudaMemcpyAsync(host_out, dev_out, nwords * 8, cudaMemcpyDeviceToHost, s));
    TG_CUDA(cudaStreamSynchronize(s));
    return TG_OK;
}

static void fill_args(ScArgs& a, const ScInstance& in, int degree) {
    memset(&a, 0, sizeof a);
    a.nt = (int)in.tables.size();
    a.degree = degree;
    for (int k = 0; k < a.nt; k++) {
        a.src[k] = in.tables[k]->cur;
        if (in.tables[k]->cur_base) a.base_mask |= 1u << k;
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
    std::lock_guard<std::mutex> lock(d->mu);
    cudaStream_t s = d->stream;
    const std::string pre(prefix);
    uint64_t g[2];
    int rc = tg_transcript_challenge_fp2(t, (pre + "/gamma").c_str(), g);
    if (rc) return rc;
    gamma[0] = g[0];
    gamma[1] = g[1];
    const fp2 gam = {g[0], g[1]};

    // device state
    std::vector<ScInstance> st(ninst);
    std::vector<fp2> w(ninst), padsum(ninst, fp2{0, 0});
    fp2 acc = {1, 0};
    for (int i = 0; i < ninst; i++) {
        w[i] = acc;
        acc = e_mul(acc, gam);
        st[i].vars = inst[i].vars;
        const size_t len = (size_t)1 << inst[i].vars;
        for (int k = 0; k < inst[i].ntables; k++) {
            auto tb = std::make_unique<ScTable>();
            const tg_table& src = inst[i].tables[k];
            tb->base = !src.is_ext;
            tb->is_public = src.is_public != 0;
            const size_t bytes = len * (tb->base ? 8 : 16);
            if (tables_on_device) {
                tb->src = src.values;
            } else {
                rc = tb->upload.ensure(bytes);
                if (rc) return rc;
                TG_CUDA(cudaMemcpyAsync(tb->upload.ptr, src.values, bytes, cudaMemcpyHostToDevice, s));
                tb->src = (const uint64_t*)tb->upload.ptr;
            }
            if (inst[i].vars >= 1) {
                rc = tb->buf[0].ensure(std::max<size_t>(len / 2, 1) * 16);
                if (rc) return rc;
                if (inst[i].vars >= 2) {
                    rc = tb->buf[1].ensure(std::max<size_t>(len / 4, 1) * 16);
                    if (rc) return rc;
                }
            }
            tb->cur = tb->src;
            tb->cur_base = tb->base;
            st[i].tables.push_back(std::move(tb));
        }
    }
    rc = d->scratch_misc.ensure((size_t)(SC_MAX_BLOCKS + 1) * 16 * 8);
    if (rc) return rc;
    uint64_t* partials = (uint64_t*)d->scratch_misc.ptr;

    // padded instances' full sums S_i
    for (int i = 0; i < ninst; i++) {
        if (st[i].vars >= n_max) continue;
        ScArgs a;
        fill_args(a, st[i], degree);
        const uint64_t len = 1ull << st[i].vars;
        const int grid = grid_for(len, d);
        Launch L(d, s, "sumcheck_product_sum", 1, len);
        sc_product_sum<<<grid, SC_THREADS, SC_THREADS * 2 * 8, s>>>(a, len, partials);
        TG_CUDA(cudaGetLastError());
        uint64_t h[2];
        rc = reduce_to_host(d, s, partials, grid, 2, h);
        if (rc) return rc;
        padsum[i] = {h[0], h[1]};
    }

    std::vector<int> pending(ninst, 0);  // own rounds whose challenge is not bound yet
    fp2 r_prev = {0, 0};
    for (int j = 0; j < n_max; j++) {
        fp2 msg[8];
        for (int x = 0; x < degree; x++) msg[x] = {0, 0};
        for (int i = 0; i < ninst; i++) {
            const int pad = n_max - st[i].vars;
            if (j < pad) {
                const fp2 v = e_mul(w[i], e_scale(padsum[i], (1ull << (pad - j - 1)) % P));
                for (int x = 0; x < degree; x++) msg[x] = e_add(msg[x], v);
                continue;
            }
            const int own = j - pad;  // own round index
            ScInstance& in = st[i];
            ScArgs a;
            fill_args(a, in, degree);
            a.npairs = 1ull << (in.vars - own - 1);
            bool all_base = true;
            for (auto& tb : in.tables) all_base &= tb->cur_base;
            if (pending[i]) {
                a.bind = 1;
                a.r = r_prev;
                for (int k = 0; k < a.nt; k++) a.dst[k] = (uint64_t*)in.tables[k]->buf[(own - 1) & 1].ptr;
            }
            const int grid = grid_for(a.npairs, d);
            uint64_t h[16];
            if (all_base && !a.bind) {
                {
                    Launch L(d, s, "sumcheck_round", 1, a.npairs);
                    sc_round_base<<<grid, SC_THREADS, SC_THREADS * degree * 8, s>>>(a, partials);
                }
                TG_CUDA(cudaGetLastError());
                rc = reduce_to_host(d, s, partials, grid, degree, h);
                if (rc) return rc;
                for (int x = 0; x < degree; x++) msg[x] = e_add(msg[x], e_mul_base(w[i], h[x]));
            } else {
                {
                    Launch L(d, s, "sumcheck_round", 1, a.npairs);
                    sc_round_ext<<<grid, SC_THREADS, SC_THREADS * 2 * degree * 8, s>>>(a, partials);
                }
                TG_CUDA(cudaGetLastError());
                rc = reduce_to_host(d, s, partials, grid, 2 * degree, h);
                if (rc) return rc;
                for (int x = 0; x < degree; x++) msg[x] = e_add(msg[x], e_mul(w[i], fp2{h[2 * x], h[2 * x + 1]}));
            }
            if (a.bind) {
                for (int k = 0; k < a.nt; k++) {
                    in.tables[k]->cur = a.dst[k];
                    in.tables[k]->cur_base = false;
                }
            }
            pending[i] = 1;
        }
        uint64_t words[16];
        for (int x = 0; x < degree; x++) {
            words[2 * x] = msg[x].c0;
            words[2 * x + 1] = msg[x].c1;
            if (rounds) {
                rounds[(size_t)j * 2 * degree + 2 * x] = msg[x].c0;
                rounds[(size_t)j * 2 * degree + 2 * x + 1] = msg[x].c1;
            }
        }
        rc = tg_transcript_absorb_fp2s(t, (pre + "/round/" + std::to_string(j)).c_str(), words, (size_t)degree);
        if (rc) return rc;
        uint64_t r[2];
        rc = tg_transcript_challenge_fp2(t, (pre + "/r/" + std::to_string(j)).c_str(), r);
        if (rc) return rc;
        if (challenges) {
            challenges[2 * j] = r[0];
            challenges[2 * j + 1] = r[1];
        }
        r_prev = {r[0], r[1]};
    }
    // the last own round's challenge, bound into one entry per table
    for (int i = 0; i < ninst; i++) {
        ScInstance& in = st[i];
        if (!pending[i]) continue;
        ScArgs a;
        fill_args(a, in, degree);
        a.r = r_prev;
        for (int k = 0; k < a.nt; k++) a.dst[k] = (uint64_t*)in.tables[k]->buf[(in.vars - 1) & 1].ptr;
        {
            Launch L(d, s, "sumcheck_bind_last", 1, 1);
            sc_bind_last<<<1, 32, 0, s>>>(a);
        }
        TG_CUDA(cudaGetLastError());
        for (int k = 0; k < a.nt; k++) {
            in.tables[k]->cur = a.dst[k];
            in.tables[k]->cur_base = false;
        }
    }
    // final evaluations: each table's single entry, public factors left out
    std::vector<uint64_t> evals;
    for (int i = 0; i < ninst; i++) {
        for (auto& tb : st[i].tables) {
            if (tb->is_public) continue;
            uint64_t v[2] = {0, 0};
            TG_CUDA(cudaMemcpyAsync(v, tb->cur, tb->cur_base ? 8 : 16, cudaMemcpyDeviceToHost, s));
            TG_CUDA(cudaStreamSynchronize(s));
            evals.push_back(v[0]);
            evals.push_back(tb->cur_base ? 0 : v[1]);
        }
    }
    *n_evals = evals.size() / 2;
    if (final_evals) memcpy(final_evals, evals.data(), evals.size() * 8);
    rc = tg_transcript_absorb_fp2s(t, (pre + "/evals").c_str(), evals.data(), evals.size() / 2);
    if (rc) return rc;
    TG_CUDA(cudaStreamSynchronize(s));
    return TG_OK;
}
