// SPDX-License-Identifier: Apache-2.0 OR MIT
//
// Offloaded tree-level rounds: the reference's LevelOffload/DeviceLevel seam
// (crates/tessera-sumcheck/src/offload.rs:17-79), which its window prover calls once a resident
// fraction or product level's tables are folded to Fp2. sums() returns Σ_p w(p)·P(line_x(p)) for
// x ∈ {0, 2, 3} with the split eq weight w(p) = low[p mod 2^low_bits]·high[p >> low_bits];
// bind(r) folds every table's lowest variable; firsts() reads each table's entry 0.
//
// The first sums() after a bind runs fused with it: one pass reads the 4 entries of each
// new pair from the unbound tables, writes the 2 bound entries, and accumulates the sums.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <memory>
#include <vector>

#include "gl.cuh"
#include "internal.h"

namespace tg {

constexpr int LV_THREADS = 256;
constexpr int LV_MAX_BLOCKS = 1024;

struct LvArgs {
    const uint64_t* src[4];
    uint64_t* dst[4];
    int nt;       // 4 fraction, 2 product
    int bind;     // fold src by r into dst before summing
    fp2 r;
    fp2 lambda;
    const uint64_t* low;   // 2^low_bits Fp2
    const uint64_t* high;  // Fp2
    uint32_t low_bits;
    uint64_t npairs;
};

__device__ __forceinline__ fp2 ld2(const uint64_t* t, uint64_t i) {
    const ulonglong2 v = reinterpret_cast<const ulonglong2*>(t)[i];
    return {v.x, v.y};
}

__device__ void lv_block_sum(uint64_t* vals, uint64_t* out) {
    __shared__ uint64_t red[6][LV_THREADS];
    for (int w = 0; w < 6; w++) red[w][threadIdx.x] = vals[w];
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s)
            for (int w = 0; w < 6; w++) red[w][threadIdx.x] = add(red[w][threadIdx.x], red[w][threadIdx.x + s]);
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int w = 0; w < 6; w++) out[w] = red[w][0];
}

__global__ void __launch_bounds__(LV_THREADS) lv_sums(LvArgs a, uint64_t* partials) {
    fp2 s0 = {0, 0}, s2 = {0, 0}, s3 = {0, 0};
    const uint64_t lmask = (1ull << a.low_bits) - 1;
    for (uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; p < a.npairs; p += (uint64_t)gridDim.x * blockDim.x) {
        fp2 v0[4], v2[4], v3[4];
        for (int k = 0; k < a.nt; k++) {
            fp2 u, v;
            if (a.bind) {
                const fp2 x0 = ld2(a.src[k], 4 * p), x1 = ld2(a.src[k], 4 * p + 1);
                const fp2 x2 = ld2(a.src[k], 4 * p + 2), x3 = ld2(a.src[k], 4 * p + 3);
                u = e_add(x0, e_mul(a.r, e_sub(x1, x0)));
                v = e_add(x2, e_mul(a.r, e_sub(x3, x2)));
                ulonglong2* o = reinterpret_cast<ulonglong2*>(a.dst[k]);
                o[2 * p] = make_ulonglong2(u.c0, u.c1);
                o[2 * p + 1] = make_ulonglong2(v.c0, v.c1);
            } else {
                u = ld2(a.src[k], 2 * p);
                v = ld2(a.src[k], 2 * p + 1);
            }
            const fp2 d = e_sub(v, u);
            v0[k] = u;
            v2[k] = e_add(v, d);
            v3[k] = e_add(v2[k], d);
        }
        const fp2 w = e_mul(ld2(a.low, p & lmask), ld2(a.high, p >> a.low_bits));
        fp2 f0, f2, f3;
        if (a.nt == 4) {  // N0 D1 + N1 D0 + λ D0 D1 over [N0, N1, D0, D1]
            f0 = e_add(e_add(e_mul(v0[0], v0[3]), e_mul(v0[1], v0[2])), e_mul(a.lambda, e_mul(v0[2], v0[3])));
            f2 = e_add(e_add(e_mul(v2[0], v2[3]), e_mul(v2[1], v2[2])), e_mul(a.lambda, e_mul(v2[2], v2[3])));
            f3 = e_add(e_add(e_mul(v3[0], v3[3]), e_mul(v3[1], v3[2])), e_mul(a.lambda, e_mul(v3[2], v3[3])));
        } else {  // V0 V1
            f0 = e_mul(v0[0], v0[1]);
            f2 = e_mul(v2[0], v2[1]);
            f3 = e_mul(v3[0], v3[1]);
        }
        s0 = e_add(s0, e_mul(w, f0));
        s2 = e_add(s2, e_mul(w, f2));
        s3 = e_add(s3, e_mul(w, f3));
    }
    uint64_t vals[6] = {s0.c0, s0.c1, s2.c0, s2.c1, s3.c0, s3.c1};
    lv_block_sum(vals, partials + 6 * (size_t)blockIdx.x);
}

__global__ void lv_reduce(const uint64_t* partials, int nblocks, uint64_t* out) {
    uint64_t v[6] = {0, 0, 0, 0, 0, 0};
    for (int b = threadIdx.x; b < nblocks; b += blockDim.x)
        for (int w = 0; w < 6; w++) v[w] = add(v[w], partials[6 * (size_t)b + w]);
    lv_block_sum(v, out);
}

// Binds alone: a.npairs holds the number of bound entries here.
__global__ void lv_bind(LvArgs a) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;  // entry of the bound table
    if (i >= a.npairs) return;
    for (int k = 0; k < a.nt; k++) {
        const fp2 x0 = ld2(a.src[k], 2 * i), x1 = ld2(a.src[k], 2 * i + 1);
        const fp2 u = e_add(x0, e_mul(a.r, e_sub(x1, x0)));
        reinterpret_cast<ulonglong2*>(a.dst[k])[i] = make_ulonglong2(u.c0, u.c1);
    }
}

}  // namespace tg

using namespace tg;

struct tg_level {
    Device* d;
    int nt;
    fp2 lambda;
    size_t len;      // entries per table now
    int cur = 0;     // which of buf[0], buf[1] holds the tables
    bool pending = false;  // a bind waiting to fuse into the next sums()
    fp2 r;
    DevBuf buf[2][4];
    DevBuf weights, partials;
    uint64_t bytes;
    std::mutex mu;
};

static std::mutex g_level_budget_mu;
static std::map<Device*, uint64_t> g_level_used;

static int lv_release_budget(tg_level* l) {
    std::lock_guard<std::mutex> g(g_level_budget_mu);
    g_level_used[l->d] -= l->bytes;
    return TG_OK;
}

// Applies a pending bind on its own (for firsts(), or two binds in a row).
static int lv_flush(tg_level* l) {
    if (!l->pending) return TG_OK;
    Device* d = l->d;
    LvArgs a;
    memset(&a, 0, sizeof a);
    a.nt = l->nt;
    a.r = l->r;
    for (int k = 0; k < l->nt; k++) {
        a.src[k] = (const uint64_t*)l->buf[l->cur][k].ptr;
        a.dst[k] = (uint64_t*)l->buf[l->cur ^ 1][k].ptr;
    }
    const uint64_t entries = l->len;  // the bound length (bind() halved it already)
    a.npairs = entries;
    Launch L(d, d->stream, "level_bind", 1, entries);
    lv_bind<<<(unsigned)((entries + 255) / 256), 256, 0, d->stream>>>(a);
    TG_CUDA(cudaGetLastError());
    l->cur ^= 1;
    l->pending = false;
    return TG_OK;
}

extern "C" {

int tg_level_load(tg_device* dev, int shape, const uint64_t lambda[2], const uint64_t* const* tables, int ntables,
                  size_t len, tg_level** out) {
    Device* d = reinterpret_cast<Device*>(dev);
    if (!d || !out || !tables) return fail(TG_ERR_INVALID, "tg_level_load: null argument");
    *out = nullptr;
    const int columns = shape == 0 ? 4 : (shape == 1 ? 2 : -1);
    if (columns < 0) return fail(TG_ERR_INVALID, "unknown level shape %d", shape);
    if (shape == 0 && !lambda) return fail(TG_ERR_INVALID, "a fraction level needs its lambda");
    // load() declines these (crates/tessera-gpu/src/level.rs:74-90)
    if (ntables != columns || len < d->cfg.level_min_entries || len < 2 || (len & (len - 1))) return TG_DECLINED;
    for (int k = 0; k < ntables; k++)
        if (!tables[k]) return fail(TG_ERR_INVALID, "tg_level_load: null table %d", k);
    const uint64_t bytes = (uint64_t)columns * (len + len / 2) * 16;
    {
        std::lock_guard<std::mutex> g(g_level_budget_mu);
        if (g_level_used[d] + bytes > d->cfg.level_budget_bytes) return TG_DECLINED;
        g_level_used[d] += bytes;
    }
    tg_level* l = new tg_level();
    l->d = d;
    l->nt = columns;
    l->lambda = shape == 0 ? fp2{lambda[0], lambda[1]} : fp2{0, 0};
    l->len = len;
    l->bytes = bytes;
    int rc = TG_OK;
    for (int k = 0; k < columns && !rc; k++) {
        rc = l->buf[0][k].ensure(len * 16);
        if (!rc) rc = l->buf[1][k].ensure(std::max<size_t>(len / 2, 1) * 16);
        if (!rc) host_prefault(tables[k], len * 16);
        if (!rc && cudaMemcpyAsync(l->buf[0][k].ptr, tables[k], len * 16, cudaMemcpyHostToDevice, d->stream) != cudaSuccess)
            rc = fail(TG_ERR_CUDA, "level table upload failed");
    }
    if (!rc) rc = l->partials.ensure((LV_MAX_BLOCKS + 1) * 6 * 8);
    if (!rc && cudaStreamSynchronize(d->stream) != cudaSuccess) rc = fail(TG_ERR_CUDA, "level upload failed");
    if (rc) {
        lv_release_budget(l);
        delete l;
        return rc;
    }
    *out = l;
    return TG_OK;
}

int tg_level_sums(tg_level* l, const uint64_t* low, const uint64_t* high, size_t nhigh, uint32_t low_bits, uint64_t out[6]) {
    if (!l || !low || !high || !out) return fail(TG_ERR_INVALID, "tg_level_sums: null argument");
    std::lock_guard<std::mutex> g(l->mu);
    Device* d = l->d;
    // the pairs of the tables after any pending bind (len is already the bound length)
    const uint64_t npairs = l->len / 2;
    if (npairs == 0) return fail(TG_ERR_STATE, "a level of one entry has no pairs");
    if (low_bits > 40) return fail(TG_ERR_INVALID, "low_bits %u too large", low_bits);
    if (((npairs - 1) >> low_bits) >= nhigh) return fail(TG_ERR_INVALID, "the high weights cover %zu of %llu", nhigh, (unsigned long long)((npairs - 1) >> low_bits) + 1);
    const size_t nlow = (size_t)1 << low_bits;
    std::lock_guard<std::mutex> dl(d->mu);
    int rc = l->weights.ensure((nlow + nhigh) * 16);
    if (rc) return rc;
    cudaStream_t s = d->stream;
    TG_CUDA(cudaMemcpyAsync(l->weights.ptr, low, nlow * 16, cudaMemcpyHostToDevice, s));
    TG_CUDA(cudaMemcpyAsync((uint8_t*)l->weights.ptr + nlow * 16, high, nhigh * 16, cudaMemcpyHostToDevice, s));
    LvArgs a;
    memset(&a, 0, sizeof a);
    a.nt = l->nt;
    a.lambda = l->lambda;
    a.low = (const uint64_t*)l->weights.ptr;
    a.high = (const uint64_t*)l->weights.ptr + 2 * nlow;
    a.low_bits = low_bits;
    a.npairs = npairs;
    if (l->pending) {
        a.bind = 1;
        a.r = l->r;
        for (int k = 0; k < l->nt; k++) {
            a.src[k] = (const uint64_t*)l->buf[l->cur][k].ptr;
            a.dst[k] = (uint64_t*)l->buf[l->cur ^ 1][k].ptr;
        }
    } else {
        for (int k = 0; k < l->nt; k++) a.src[k] = (const uint64_t*)l->buf[l->cur][k].ptr;
    }
    uint64_t blocks = (npairs + LV_THREADS - 1) / LV_THREADS;
    blocks = std::min<uint64_t>(blocks, std::min<uint64_t>(LV_MAX_BLOCKS, (uint64_t)d->sm_count * 4));
    const int grid = (int)std::max<uint64_t>(blocks, 1);
    uint64_t* partials = (uint64_t*)l->partials.ptr;
    {
        Launch L(d, s, "level_sums", 2, npairs);
        lv_sums<<<grid, LV_THREADS, 0, s>>>(a, partials);
        lv_reduce<<<1, LV_THREADS, 0, s>>>(partials, grid, partials + 6 * (size_t)grid);
    }
    TG_CUDA(cudaGetLastError());
    TG_CUDA(cudaMemcpyAsync(out, partials + 6 * (size_t)grid, 48, cudaMemcpyDeviceToHost, s));
    TG_CUDA(cudaStreamSynchronize(s));
    if (l->pending) {
        l->cur ^= 1;
        l->pending = false;
    }
    return TG_OK;
}

int tg_level_bind(tg_level* l, const uint64_t r[2]) {
    if (!l || !r) return fail(TG_ERR_INVALID, "tg_level_bind: null argument");
    std::lock_guard<std::mutex> g(l->mu);
    if (l->len < 2) return fail(TG_ERR_STATE, "every variable is already bound");
    if (l->pending) {  // two binds in a row: apply the first now
        std::lock_guard<std::mutex> dl(l->d->mu);
        int rc = lv_flush(l);
        if (rc) return rc;
    }
    l->r = {r[0], r[1]};
    l->pending = true;
    l->len /= 2;
    return TG_OK;
}

int tg_level_firsts(tg_level* l, uint64_t* out) {
    if (!l || !out) return fail(TG_ERR_INVALID, "tg_level_firsts: null argument");
    std::lock_guard<std::mutex> g(l->mu);
    std::lock_guard<std::mutex> dl(l->d->mu);
    int rc = lv_flush(l);
    if (rc) return rc;
    cudaStream_t s = l->d->stream;
    for (int k = 0; k < l->nt; k++)
        TG_CUDA(cudaMemcpyAsync(out + 2 * k, l->buf[l->cur][k].ptr, 16, cudaMemcpyDeviceToHost, s));
    TG_CUDA(cudaStreamSynchronize(s));
    return TG_OK;
}

int tg_level_free(tg_level* l) {
    if (!l) return TG_OK;
    cudaStreamSynchronize(l->d->stream);
    lv_release_budget(l);
    delete l;
    return TG_OK;
}

}  // extern "C"
