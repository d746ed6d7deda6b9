// SPDX-License-Identifier: Apache-2.0 OR MIT
//
// Reed–Solomon low-degree extension of Goldilocks rows on the device: the computation of the
// reference's RowEncoder::encode_rows (crates/tessera-pcs/src/encoding.rs:257-313). Row i holds
// f(ω_k^t), t < k; codeword symbol j is g(7·ω_n^j), g = f + (X^k − 1)·m, n = 2^r·k.
//
// GB300 design. Symbol q·2^r + e of the codeword is NTT_k(c_e)[q], where c_e[i] = s_e^i·(a_i +
// m_i·(s_e^k − 1)), s_e = 7·ω_n^e and a = iNTT_k(row): the 2^r cosets of the subgroup of order k,
// interleaved. With k = K1·K2 the work runs as three passes over HBM-resident rows, each a batch
// of small transforms in shared memory:
//
//   pass A  inverse size-K2 transforms down the strided columns t1 (stride K1), × ω_k^{−j2·t1};
//   pass M  per j2: inverse size-K1 transform, then per coset e the scale s_e^i/k (+ mask) and a
//           forward size-K1 transform, × ω_k^{v2·j2};
//   pass C  per v2 and coset: forward size-K2 transform, written interleaved into the codeword.
//
// The inverse transform's last step and the forward transform's first step share their data
// grouping (fixed j2, all j1), which is why they fuse into pass M. Rows go through in groups of
// scratch (k + n words per row, lde_group_bytes in all: 32 rows at k = 2^20), so that every pass's
// grid spans many waves; the scratch is written with an L2 evict-last hint, and the part still in
// L2 when the next pass reads it saves HBM reads. Rows of k ≤ 2^11 take one CTA each, all in
// shared memory.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <vector>

#include "gl.cuh"
#include "internal.h"
#include "lde_fast.cuh"

namespace tg {

// ---- in-CTA radix-2 transforms ---------------------------------------------------------------
//
// `cols` columns of length L = 2^lg live in shared memory, element (c, t) at base[c*cs + t*ts].
// tw[m] = w^m for m < L/2, w the transform's root.

// Gentleman–Sande: natural order in, bit-reversed order out (position p holds X[rev(p)]).
template <bool C_FAST>
__device__ __forceinline__ void dif_smem(uint64_t* base, int lg, int lgcols, int cs, int ts, const uint64_t* tw) {
    const int half = 1 << (lg - 1);
    const int nb = half << lgcols;
    for (int s = 0; s < lg; s++) {
        const int lh = lg - 1 - s;
        const int h = 1 << lh;
        for (int b = threadIdx.x; b < nb; b += blockDim.x) {
            int c, bf;
            if (C_FAST) {
                c = b & ((1 << lgcols) - 1);
                bf = b >> lgcols;
            } else {
                bf = b & (half - 1);
                c = b >> (lg - 1);
            }
            const int o = bf & (h - 1);
            const int i0 = ((bf >> lh) << (lh + 1)) + o;
            uint64_t* p0 = base + c * cs + i0 * ts;
            uint64_t* p1 = p0 + h * ts;
            const uint64_t u = *p0, v = *p1;
            *p0 = add(u, v);
            *p1 = mul(sub(u, v), tw[o << s]);
        }
        __syncthreads();
    }
}

// Cooley–Tukey: bit-reversed order in, natural order out.
template <bool C_FAST>
__device__ __forceinline__ void dit_smem(uint64_t* base, int lg, int lgcols, int cs, int ts, const uint64_t* tw) {
    const int half = 1 << (lg - 1);
    const int nb = half << lgcols;
    for (int s = 0; s < lg; s++) {
        const int h = 1 << s;
        for (int b = threadIdx.x; b < nb; b += blockDim.x) {
            int c, bf;
            if (C_FAST) {
                c = b & ((1 << lgcols) - 1);
                bf = b >> lgcols;
            } else {
                bf = b & (half - 1);
                c = b >> (lg - 1);
            }
            const int o = bf & (h - 1);
            const int i0 = ((bf >> s) << (s + 1)) + o;
            uint64_t* p0 = base + c * cs + i0 * ts;
            uint64_t* p1 = p0 + h * ts;
            const uint64_t u = *p0;
            const uint64_t v = mul(*p1, tw[o << (lg - 1 - s)]);
            *p0 = add(u, v);
            *p1 = sub(u, v);
        }
        __syncthreads();
    }
}

__device__ __forceinline__ uint32_t brev(uint32_t x, int bits) { return bits ? (__brev(x) >> (32 - bits)) : 0; }

// ω_L^{±m} for m < L from the table pw[m] = ω_n^m (n = 2^lgn, L = 2^lg ≤ n).
__device__ __forceinline__ uint64_t root_pow(const uint64_t* pw, int lgn, int lg, uint32_t m, bool inverse) {
    const uint64_t n = 1ull << lgn;
    uint64_t e = (uint64_t)m << (lgn - lg);
    if (inverse) e = (n - e) & (n - 1);
    return pw[e];
}

__device__ void load_twiddles(uint64_t* tw, const uint64_t* pw, int lgn, int lg, bool inverse) {
    for (int m = threadIdx.x; m < (1 << (lg - 1)); m += blockDim.x) tw[m] = root_pow(pw, lgn, lg, m, inverse);
}

struct LdeArgs {
    const uint64_t* rows;   // group's rows: g x k
    const uint64_t* masks;  // g x P, or null
    uint64_t* y;            // scratch: g x k
    uint64_t* z;            // scratch: g x n (2^r slabs of k per row)
    uint64_t* out;          // codewords: g x n
    const uint64_t* pw;     // ω_n^m, m < n
    const uint64_t* pow7k;  // 7^i / k, i < k
    uint64_t mk[16];        // k (7^k ω_{2^r}^e − 1), per coset e
    int lgk, lgr, lgk1, lgk2, lgw, P;
};

// Pass A: tile of 2^lgw consecutive t1 columns, all K2 rows t2. smem layout [t2][W].
__global__ void __launch_bounds__(512) lde_pass_a(LdeArgs a) {
    extern __shared__ uint64_t sm[];
    const int lgw = a.lgw, W = 1 << lgw, K1 = 1 << a.lgk1, K2 = 1 << a.lgk2;
    const int lgn = a.lgk + a.lgr;
    uint64_t* buf = sm;
    uint64_t* tw = sm + (W << a.lgk2);
    const int t1_0 = blockIdx.x << lgw;
    const uint64_t* src = a.rows + ((size_t)blockIdx.y << a.lgk);
    for (int i = threadIdx.x; i < (W << a.lgk2); i += blockDim.x) {
        const int c = i & (W - 1), t2 = i >> lgw;
        buf[i] = src[t1_0 + c + ((size_t)t2 << a.lgk1)];
    }
    load_twiddles(tw, a.pw, lgn, a.lgk2, true);
    __syncthreads();
    dif_smem<true>(buf, a.lgk2, lgw, 1, W, tw);
    // position p holds j2 = rev(p); multiply by ω_k^{−j2·t1}, store Y[j2][t1]
    uint64_t* y = a.y + ((size_t)blockIdx.y << a.lgk);
    for (int i = threadIdx.x; i < (W << a.lgk2); i += blockDim.x) {
        const int c = i & (W - 1), p = i >> lgw;
        const uint32_t j2 = brev(p, a.lgk2);
        const uint32_t t1 = t1_0 + c;
        const uint64_t w = root_pow(a.pw, lgn, a.lgk, (j2 * t1) & ((1u << a.lgk) - 1), true);
        y[((size_t)j2 << a.lgk1) + t1] = mul(buf[i], w);
    }
    (void)K1;
    (void)K2;
}

// Pass M: tile of W consecutive j2, each a column of K1 values (t1). smem: a[W][K1+1], b[W][K1+1].
__global__ void __launch_bounds__(512) lde_pass_m(LdeArgs a) {
    extern __shared__ uint64_t sm[];
    const int lgw = a.lgw, W = 1 << lgw, K1 = 1 << a.lgk1, K2 = 1 << a.lgk2;
    const int cs = K1 + 1;
    const int lgn = a.lgk + a.lgr;
    uint64_t* abuf = sm;
    uint64_t* bbuf = sm + W * cs;
    uint64_t* twi = bbuf + W * cs;
    uint64_t* twf = twi + K1 / 2;
    const int j2_0 = blockIdx.x << lgw;
    const size_t row = blockIdx.y;
    const uint64_t* y = a.y + (row << a.lgk);
    for (int i = threadIdx.x; i < (W << a.lgk1); i += blockDim.x) {
        const int t1 = i & (K1 - 1), c = i >> a.lgk1;
        abuf[c * cs + t1] = y[((size_t)(j2_0 + c) << a.lgk1) + t1];
    }
    load_twiddles(twi, a.pw, lgn, a.lgk1, true);
    load_twiddles(twf, a.pw, lgn, a.lgk1, false);
    __syncthreads();
    dif_smem<false>(abuf, a.lgk1, lgw, cs, 1, twi);
    // abuf[c][p] = k·a_i, i = j2 + K2·rev(p)
    const uint64_t* masks = a.masks ? a.masks + row * (size_t)a.P : nullptr;
    for (int e = 0; e < (1 << a.lgr); e++) {
        for (int i = threadIdx.x; i < (W << a.lgk1); i += blockDim.x) {
            const int p = i & (K1 - 1), c = i >> a.lgk1;
            const uint32_t j1 = brev(p, a.lgk1);
            const uint32_t idx = (uint32_t)(j2_0 + c) + ((uint32_t)j1 << a.lgk2);
            uint64_t v = abuf[c * cs + p];
            if ((int)idx < a.P) v = add(v, mul(masks[idx], a.mk[e]));
            // s_e^i / k = (7^i / k) · ω_n^{e·i}
            uint64_t sc = a.pow7k[idx];
            if (e) sc = mul(sc, a.pw[((uint64_t)e * idx) & ((1ull << lgn) - 1)]);
            bbuf[c * cs + p] = mul(v, sc);
        }
        __syncthreads();
        dit_smem<false>(bbuf, a.lgk1, lgw, cs, 1, twf);
        // bbuf[c][v2] natural; × ω_k^{v2·j2}; store Z_e[v2][j2]
        uint64_t* z = a.z + (row << lgn) + ((size_t)e << a.lgk);
        for (int i = threadIdx.x; i < (W << a.lgk1); i += blockDim.x) {
            const int c = i & (W - 1), v2 = i >> lgw;
            const uint32_t j2 = j2_0 + c;
            const uint64_t w = root_pow(a.pw, lgn, a.lgk, (j2 * (uint32_t)v2) & ((1u << a.lgk) - 1), false);
            z[((size_t)v2 << a.lgk2) + j2] = mul(bbuf[c * cs + v2], w);
        }
        __syncthreads();
    }
    (void)K2;
}

// Pass C: tile of W consecutive v2, all cosets; each a column of K2 values (j2).
// smem: 2^r buffers of [W][K2+1].
__global__ void __launch_bounds__(512) lde_pass_c(LdeArgs a) {
    extern __shared__ uint64_t sm[];
    const int lgw = a.lgw, W = 1 << lgw, K1 = 1 << a.lgk1, K2 = 1 << a.lgk2;
    const int cs = K2 + 1;
    const int R = 1 << a.lgr;
    const int lgn = a.lgk + a.lgr;
    uint64_t* tw = sm + (size_t)R * W * cs;
    const int v2_0 = blockIdx.x << lgw;
    const size_t row = blockIdx.y;
    const uint64_t* z = a.z + (row << lgn);
    for (int i = threadIdx.x; i < (R * W) << a.lgk2; i += blockDim.x) {
        const int j2 = i & (K2 - 1), ce = i >> a.lgk2;  // ce = e * W + c
        const int c = ce & (W - 1), e = ce >> lgw;
        sm[ce * cs + j2] = z[((size_t)e << a.lgk) + ((size_t)(v2_0 + c) << a.lgk2) + j2];
    }
    load_twiddles(tw, a.pw, lgn, a.lgk2, false);
    __syncthreads();
    dif_smem<false>(sm, a.lgk2, lgw + a.lgr, cs, 1, tw);
    // sm[e*W + c][p] = out_e[v2 + K1·rev(p)]; codeword position (v2 + K1·v1)·2^r + e
    uint64_t* out = a.out + (row << lgn);
    for (int i = threadIdx.x; i < (R * W) << a.lgk2; i += blockDim.x) {
        const int e = i & (R - 1), c = (i >> a.lgr) & (W - 1), v1 = i >> (a.lgr + lgw);
        const int p = brev(v1, a.lgk2);
        const size_t q = (size_t)(v2_0 + c) + ((size_t)v1 << a.lgk1);
        out[(q << a.lgr) + e] = sm[(e * W + c) * cs + p];
    }
    (void)K1;
}

// Small rows (k ≤ 2^11): one CTA per row, everything in shared memory.
__global__ void __launch_bounds__(512) lde_small(LdeArgs a) {
    extern __shared__ uint64_t sm[];
    const int K = 1 << a.lgk, R = 1 << a.lgr;
    const int lgn = a.lgk + a.lgr;
    uint64_t* abuf = sm;
    uint64_t* bbuf = sm + K;
    uint64_t* twi = bbuf + K;
    uint64_t* twf = twi + (K > 1 ? K / 2 : 1);
    const size_t row = blockIdx.x;
    const uint64_t* src = a.rows + (row << a.lgk);
    for (int i = threadIdx.x; i < K; i += blockDim.x) abuf[i] = src[i];
    if (a.lgk > 0) {
        load_twiddles(twi, a.pw, lgn, a.lgk, true);
        load_twiddles(twf, a.pw, lgn, a.lgk, false);
    }
    __syncthreads();
    if (a.lgk > 0) dif_smem<false>(abuf, a.lgk, 0, 0, 1, twi);
    const uint64_t* masks = a.masks ? a.masks + row * (size_t)a.P : nullptr;
    uint64_t* out = a.out + (row << lgn);
    for (int e = 0; e < R; e++) {
        for (int p = threadIdx.x; p < K; p += blockDim.x) {
            const uint32_t idx = brev(p, a.lgk);
            uint64_t v = abuf[p];
            if ((int)idx < a.P) v = add(v, mul(masks[idx], a.mk[e]));
            uint64_t sc = a.pow7k[idx];
            if (e) sc = mul(sc, a.pw[((uint64_t)e * idx) & ((1ull << lgn) - 1)]);
            bbuf[p] = mul(v, sc);
        }
        __syncthreads();
        if (a.lgk > 0) dit_smem<false>(bbuf, a.lgk, 0, 0, 1, twf);
        for (int q = threadIdx.x; q < K; q += blockDim.x) out[((size_t)q << a.lgr) + e] = bbuf[q];
        __syncthreads();
    }
}

// ---- tables ----------------------------------------------------------------------------------

__global__ void fill_powers(uint64_t* out, size_t n, uint64_t base, uint64_t scale, uint32_t chunk_log) {
    // out[i] = scale · base^i: each thread starts its chunk with one exponentiation.
    const size_t chunk = (size_t)1 << chunk_log;
    const size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t start = c * chunk;
    if (start >= n) return;
    uint64_t v = mul(scale, pow(base, start));
    const size_t end = start + chunk < n ? start + chunk : n;
    for (size_t i = start; i < end; i++) {
        out[i] = v;
        v = mul(v, base);
    }
}

static uint64_t root_of_unity(uint32_t lg) { return pow(7, (P - 1) >> lg); }

int Device::get_tables(uint32_t lgn, uint32_t lgk, const Tables** out) {
    const uint64_t key = ((uint64_t)lgn << 32) | lgk;
    auto it = tables.find(key);
    if (it != tables.end()) {
        *out = &it->second;
        return TG_OK;
    }
    Tables t;
    t.lgn = lgn;
    t.lgk = lgk;
    const size_t n = (size_t)1 << lgn, k = (size_t)1 << lgk;
    TG_CUDA(cudaMalloc(&t.pw, n * 8));
    cudaError_t e = cudaMalloc(&t.pow7k, k * 8);
    if (e != cudaSuccess) {
        cudaFree(t.pw);
        return cuda_fail(e, "cudaMalloc(pow7k)");
    }
    const uint32_t cl = 6;
    const size_t threads_n = (n + (1u << cl) - 1) >> cl, threads_k = (k + (1u << cl) - 1) >> cl;
    launches += 2;
    fill_powers<<<(unsigned)((threads_n + 255) / 256), 256, 0, stream>>>(t.pw, n, root_of_unity(lgn), 1, cl);
    const uint64_t inv_k = inv(k % P);
    fill_powers<<<(unsigned)((threads_k + 255) / 256), 256, 0, stream>>>(t.pow7k, k, 7, inv_k, cl);
    TG_CUDA(cudaGetLastError());
    TG_CUDA(cudaStreamSynchronize(stream));
    tables[key] = t;
    *out = &tables[key];
    return TG_OK;
}

// ---- register-resident passes (lde_fast.cuh) for 2^14 <= k <= 2^20 ---------------------------

static int set_smem(const void* fn, int words) {
    TG_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, words * 8));
    return TG_OK;
}

// Launches pass `which` (0 = A, 1 = M1, 2 = M2, 3 = C) for a column length 2^lg.
static int fast_pass(int which, int lg, dim3 grid, const fast::Args& a, cudaStream_t s) {
    using namespace fast;
#define TG_FAST_CASE(LG, RA, RB)                                                                   \
    case LG: {                                                                                     \
        const void* fns[4] = {(const void*)pass_a<RA, RB>, (const void*)pass_m1<RA, RB>,          \
                              (const void*)pass_m2<RA, RB>, (const void*)pass_c<RA, RB>};          \
        const int words = Shape<RA, RB>::WORDS + RA * RB;                                          \
        int rc = set_smem(fns[which], words);                                                      \
        if (rc) return rc;                                                                         \
        if (which == 0) pass_a<RA, RB><<<grid, THREADS, words * 8, s>>>(a);                        \
        else if (which == 1) pass_m1<RA, RB><<<grid, THREADS, words * 8, s>>>(a);                  \
        else if (which == 2) pass_m2<RA, RB><<<grid, THREADS, words * 8, s>>>(a);                  \
        else pass_c<RA, RB><<<grid, THREADS, words * 8, s>>>(a);                                   \
        return TG_OK;                                                                              \
    }
    switch (lg) {
        TG_FAST_CASE(6, 8, 8)
        TG_FAST_CASE(7, 16, 8)
        TG_FAST_CASE(8, 16, 16)
        TG_FAST_CASE(9, 32, 16)
        TG_FAST_CASE(10, 32, 32)
        TG_FAST_CASE(11, 64, 32)
        default:
            return fail(TG_ERR_INVALID, "no register-resident transform of length 2^%d", lg);
    }
#undef TG_FAST_CASE
}

static bool fast_shape(uint32_t lgk) { return lgk >= 13 && lgk <= 22; }

// RB, the second radix of the register-resident transform of length 2^lg (fast_pass's cases).
static int fast_rb(int lg) { return lg <= 7 ? 8 : lg <= 9 ? 16 : 32; }

// Words of one CTA's tile: 8,192 for every column length (32 elements per thread).
static uint64_t fast_tile(int) { return 8192; }

bool encode_split_valid(uint32_t lgk, int lgk1) {
    const int lgk2 = (int)lgk - lgk1;
    return fast_shape(lgk) && lgk1 >= 6 && lgk1 <= 11 && lgk2 >= 6 && lgk2 <= 11;
}

// Encodes rows in groups through the four register-resident passes; y/z hold `group` rows. The
// row's transform of length k = K1·K2 splits as K1 = 2^lgk1 (passes M1, M2) by K2 (passes A, C);
// lgk1 = 0 takes the default, K1 = 2^ceil(lgk/2).
static int fast_encode(Device* d, uint32_t lgk, uint32_t lgr, uint32_t P_, const uint64_t* rows, size_t npolys,
                       const uint64_t* masks, uint64_t* codewords, cudaStream_t s, const uint64_t* pw,
                       const uint64_t* pow7k, uint64_t* y, uint64_t* z, size_t group, int lgk1) {
    if (lgk1 == 0) lgk1 = (int)(lgk + 1) / 2;
    if (!encode_split_valid(lgk, lgk1))
        return fail(TG_ERR_INVALID, "no split of 2^%u into 2^%d columns of 2^%d", lgk, lgk1, (int)lgk - lgk1);
    fast::Args a = {};
    a.pw = pw;
    a.pow7k = pow7k;
    a.lgk = (int)lgk;
    a.lgr = (int)lgr;
    a.P = (int)P_;
    a.lgk1 = lgk1;
    a.lgk2 = (int)lgk - lgk1;
    a.y = y;
    a.z = z;
    const uint32_t lgn = lgk + lgr;
    const uint64_t k = 1ull << lgk;
    const uint64_t pow7_k = pow(7, k);
    const uint64_t w_r = root_of_unity(lgr), w_n = root_of_unity(lgn);
    // pass M's chain step s_e^{K2·RB}, RB the second radix of the length-K1 transform
    const uint64_t m = (uint64_t)fast_rb(a.lgk1) << a.lgk2;
    uint64_t we = 1;
    for (int e = 0; e < (1 << lgr); e++) {
        a.mk[e] = mul(k % P, sub(mul(pow7_k, we), 1));
        a.sstep[e] = mul(pow(7, m), pow(w_n, ((uint64_t)e * m) & ((1ull << lgn) - 1)));
        we = mul(we, w_r);
    }
    const size_t tiles_k2 = k / fast_tile(a.lgk2), tiles_k1 = k / fast_tile(a.lgk1);
    group = std::min<size_t>(std::max<size_t>(group, 1), 65535);
    for (size_t r0 = 0; r0 < npolys; r0 += group) {
        const unsigned g = (unsigned)std::min(group, npolys - r0);
        a.rows = rows + (r0 << lgk);
        a.masks = masks ? masks + r0 * P_ : nullptr;
        a.out = codewords + (r0 << lgn);
        int rc;
        {
            Launch L(d, s, "lde_pass_a", 1, g);
            rc = fast_pass(0, a.lgk2, dim3((unsigned)tiles_k2, g), a, s);
        }
        if (rc) return rc;
        {
            Launch L(d, s, "lde_pass_m1", 1, g);
            rc = fast_pass(1, a.lgk1, dim3((unsigned)tiles_k1, g), a, s);
        }
        if (rc) return rc;
        if (P_ > 0 && masks) {
            Launch L(d, s, "lde_mask_fixup", 1, g);
            const unsigned threads = (unsigned)P_ << lgr;
            fast::mask_fixup<<<dim3((threads + 255) / 256, g), 256, 0, s>>>(a);
        }
        {
            Launch L(d, s, "lde_pass_m2", 1, g);
            rc = fast_pass(2, a.lgk1, dim3((unsigned)(tiles_k1 << lgr), g), a, s);
        }
        if (rc) return rc;
        {
            Launch L(d, s, "lde_pass_c", 1, g);
            rc = fast_pass(3, a.lgk2, dim3((unsigned)(tiles_k2 << lgr), g), a, s);
        }
        if (rc) return rc;
    }
    TG_CUDA(cudaGetLastError());
    return TG_OK;
}

// ---- launcher --------------------------------------------------------------------------------

static int smem_limit(Device* d) { return (int)std::min<size_t>(d->smem_optin, 227 * 1024); }

int lde_encode(Device* d, uint32_t lgk, uint32_t lgr, uint32_t P_, const uint64_t* rows, size_t npolys,
               const uint64_t* masks, uint64_t* codewords, cudaStream_t s) {
    if (lgr < 1 || lgr > 4) return fail(TG_ERR_INVALID, "log2 inverse rate %u outside 1..4", lgr);
    if (lgk > 24) return fail(TG_ERR_INVALID, "log2 k %u above 24", lgk);
    if ((size_t)P_ > ((size_t)1 << lgk)) return fail(TG_ERR_INVALID, "%u mask coefficients exceed k", P_);
    if (P_ > 0 && !masks) return fail(TG_ERR_INVALID, "mask coefficients requested without masks");
    if (npolys == 0) return TG_OK;
    const Tables* t;
    int rc = d->get_tables(lgk + lgr, lgk, &t);
    if (rc) return rc;
    // Rows of k > 2^11 go through scratch: k + n words per row, rows in groups of about the
    // configured budget, so that every pass's grid spans many waves.
    size_t group = 0;
    uint64_t *y = nullptr, *z = nullptr;
    if (lgk > 11) {
        const size_t k = (size_t)1 << lgk;
        group = std::max<size_t>(1, d->cfg.lde_group_bytes / ((k + (k << lgr)) * 8));
        group = std::min<size_t>(group, std::min<size_t>(npolys, 65535));
        rc = d->scratch_y.ensure(group * k * 8);
        if (rc) return rc;
        rc = d->scratch_z.ensure(group * (k << lgr) * 8);
        if (rc) return rc;
        y = (uint64_t*)d->scratch_y.ptr;
        z = (uint64_t*)d->scratch_z.ptr;
    }
    return lde_encode_into(d, lgk, lgr, P_, rows, npolys, masks, codewords, s, t->pw, t->pow7k, false, y, z, group);
}

}  // namespace tg

namespace tg {

// The encoder over caller-owned tables and scratch (lde_encode's launcher, and the
// allocation-free entry point's): it allocates nothing. When `build_tables` is set it first
// writes pw (n words, ω_n^m) and pow7k (k words, 7^i/k) on stream s; y and z hold `group` rows
// of scratch (k and n words per row; unused for k <= 2^11).
int lde_encode_into(Device* d, uint32_t lgk, uint32_t lgr, uint32_t P_, const uint64_t* rows, size_t npolys,
                    const uint64_t* masks, uint64_t* codewords, cudaStream_t s, uint64_t* pw, uint64_t* pow7k,
                    bool build_tables, uint64_t* y, uint64_t* z, size_t group, int lgk1) {
    const uint32_t lgn = lgk + lgr;
    const uint64_t k = 1ull << lgk, n = 1ull << lgn;
    if (build_tables) {
        const uint32_t cl = 6;
        const size_t threads_n = (n + (1u << cl) - 1) >> cl, threads_k = (k + (1u << cl) - 1) >> cl;
        Launch L(d, s, "tables", 2, n + k);
        fill_powers<<<(unsigned)((threads_n + 255) / 256), 256, 0, s>>>(pw, n, root_of_unity(lgn), 1, cl);
        fill_powers<<<(unsigned)((threads_k + 255) / 256), 256, 0, s>>>(pow7k, k, 7, inv(k % P), cl);
        TG_CUDA(cudaGetLastError());
    }
    if (npolys == 0) return TG_OK;
    LdeArgs a = {};
    a.pw = pw;
    a.pow7k = pow7k;
    a.lgk = (int)lgk;
    a.lgr = (int)lgr;
    a.P = (int)P_;
    const uint64_t pow7_k = pow(7, k);
    const uint64_t w_r = root_of_unity(lgr);
    uint64_t we = 1;
    for (int e = 0; e < (1 << lgr); e++) {
        a.mk[e] = mul(k % P, sub(mul(pow7_k, we), 1));
        we = mul(we, w_r);
    }
    const int limit = smem_limit(d);
    if (lgk <= 11) {
        const size_t K = (size_t)1 << lgk;
        const size_t smem = (2 * K + 2 * std::max<size_t>(K / 2, 1)) * 8;
        TG_CUDA(cudaFuncSetAttribute(lde_small, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        const int threads = (int)std::min<size_t>(512, std::max<size_t>(32, K / 2));
        for (size_t r0 = 0; r0 < npolys; r0 += 65535) {
            const size_t g = std::min<size_t>(65535, npolys - r0);
            a.rows = rows + (r0 << lgk);
            a.masks = masks ? masks + r0 * P_ : nullptr;
            a.out = codewords + (r0 << lgn);
            Launch L(d, s, "lde_small", 1, g);
            lde_small<<<(unsigned)g, threads, smem, s>>>(a);
        }
        TG_CUDA(cudaGetLastError());
        return TG_OK;
    }
    if (fast_shape(lgk)) {
        if (group < 1) return fail(TG_ERR_INVALID, "no scratch for one row");
        return fast_encode(d, lgk, lgr, P_, rows, npolys, masks, codewords, s, pw, pow7k, y, z, group, lgk1);
    }
    a.lgk1 = (int)(lgk + 1) / 2;
    a.lgk2 = (int)lgk / 2;
    const size_t K1 = (size_t)1 << a.lgk1, K2 = (size_t)1 << a.lgk2;
    const size_t R = (size_t)1 << lgr;
    int lgw_a = 4, lgw_m = 3, lgw_c = 3;
    while (lgw_a > 0 && ((K2 << lgw_a) * 8 > 128 * 1024)) lgw_a--;
    while (lgw_m > 0 && (2 * ((K1 + 1) << lgw_m) * 8 + K1 * 8 > (size_t)limit)) lgw_m--;
    while (lgw_c > 0 && (R * ((K2 + 1) << lgw_c) * 8 + K2 * 4 > (size_t)limit)) lgw_c--;
    const size_t smem_a = ((K2 << lgw_a) + K2 / 2) * 8;
    const size_t smem_m = (2 * ((K1 + 1) << lgw_m) + K1) * 8;
    const size_t smem_c = (R * ((K2 + 1) << lgw_c) + K2 / 2) * 8;
    if (smem_m > (size_t)limit || smem_c > (size_t)limit)
        return fail(TG_ERR_INVALID, "row length 2^%u at rate 1/2^%u exceeds shared memory", lgk, lgr);
    TG_CUDA(cudaFuncSetAttribute(lde_pass_a, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_a));
    TG_CUDA(cudaFuncSetAttribute(lde_pass_m, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_m));
    TG_CUDA(cudaFuncSetAttribute(lde_pass_c, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_c));
    if (group < 1) return fail(TG_ERR_INVALID, "no scratch for one row");
    group = std::min<size_t>(group, 65535);
    a.y = y;
    a.z = z;
    for (size_t r0 = 0; r0 < npolys; r0 += group) {
        const unsigned g = (unsigned)std::min(group, npolys - r0);
        a.rows = rows + (r0 << lgk);
        a.masks = masks ? masks + r0 * P_ : nullptr;
        a.out = codewords + (r0 << lgn);
        a.lgw = lgw_a;
        {
            Launch L(d, s, "lde_pass_a", 1, g);
            lde_pass_a<<<dim3((unsigned)(K1 >> lgw_a), g), 512, smem_a, s>>>(a);
        }
        a.lgw = lgw_m;
        {
            Launch L(d, s, "lde_pass_m", 1, g);
            lde_pass_m<<<dim3((unsigned)(K2 >> lgw_m), g), 512, smem_m, s>>>(a);
        }
        a.lgw = lgw_c;
        {
            Launch L(d, s, "lde_pass_c", 1, g);
            lde_pass_c<<<dim3((unsigned)(K1 >> lgw_c), g), 512, smem_c, s>>>(a);
        }
    }
    TG_CUDA(cudaGetLastError());
    return TG_OK;
}

}  // namespace tg

namespace tg {

// ---- standalone transforms: NttPlan::{ntt, intt, coset_ntt, coset_intt} ----------------------
//
// The reference's plan transforms one row in place, natural order on both sides
// (crates/tessera-pcs/src/ntt.rs:461-516). Here many rows go at once. Rows of n ≤ 2^12 take one
// CTA each in shared memory; rows of 2^13..2^22 run through the encoder's register-resident
// passes with a one-coset (rate 1) setting: the forward transform is passes M2 and C (the
// coefficients laid out as the encoder's C_0, natural order), the inverse passes A and M1 with
// M1's per-element scale taken from a table of shift^{−i}/n instead of the coset powers.

// values[i] *= scale[i mod n] over g rows of n = 2^lgn.
__global__ void ntt_scale(uint64_t* values, uint32_t lgn, size_t total, const uint64_t* scale) {
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    const size_t mask = ((size_t)1 << lgn) - 1;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += stride)
        values[i] = mul(values[i], scale[i & mask]);
}

// One row per CTA: forward — x_i·scale[i] (when scale is set), DIF with ω_n, written back in
// natural order; inverse — DIF with ω_n^{−1}, each output c_j times scale[j] (shift^{−j}/n).
__global__ void __launch_bounds__(512) ntt_small(uint64_t* values, int lgn, const uint64_t* pw, const uint64_t* scale,
                                                  int inverse) {
    extern __shared__ uint64_t sm[];
    const int n = 1 << lgn;
    uint64_t* buf = sm;
    uint64_t* tw = sm + n;
    uint64_t* row = values + ((size_t)blockIdx.x << lgn);
    for (int i = threadIdx.x; i < n; i += blockDim.x) buf[i] = (!inverse && scale) ? mul(row[i], scale[i]) : row[i];
    load_twiddles(tw, pw, lgn, lgn, inverse != 0);
    __syncthreads();
    dif_smem<false>(buf, lgn, 0, 0, 1, tw);
    for (int p = threadIdx.x; p < n; p += blockDim.x) {
        const uint32_t j = brev(p, lgn);
        row[j] = inverse ? mul(buf[p], scale[j]) : buf[p];
    }
}

int ntt_rows(Device* d, int kind, uint32_t lgn, uint64_t shift, uint64_t* values, size_t nrows, cudaStream_t s) {
    const bool inverse = kind == NTT_INVERSE || kind == NTT_COSET_INVERSE;
    const bool coset = kind == NTT_COSET_FORWARD || kind == NTT_COSET_INVERSE;
    if (kind < NTT_FORWARD || kind > NTT_COSET_INVERSE) return fail(TG_ERR_INVALID, "unknown transform kind %d", kind);
    if (lgn > 22) return fail(TG_ERR_INVALID, "transforms of 2^%u points: the device transforms go up to 2^22", lgn);
    if (coset && (shift == 0 || shift >= P)) return fail(TG_ERR_INVALID, "coset shift %llu is zero or not canonical",
                                                          (unsigned long long)shift);
    if (nrows == 0 || lgn == 0) return TG_OK;  // a transform of one point is the identity
    const size_t n = (size_t)1 << lgn;
    const Tables* t;
    int rc = d->get_tables(lgn, lgn, &t);
    if (rc) return rc;
    // the scale table: forward shift^i (coset only); inverse shift^{−i}/n (shift 1 for the plain inverse)
    const bool scaled = inverse || coset;
    uint64_t* scale = nullptr;
    if (scaled) {
        rc = d->scratch_z.ensure(n * 8);
        if (rc) return rc;
        scale = (uint64_t*)d->scratch_z.ptr;
        const uint64_t base = inverse ? (coset ? inv(shift) : 1) : shift;
        const uint64_t first = inverse ? inv(n % P) : 1;
        const uint32_t cl = 6;
        const size_t threads = (n + (1u << cl) - 1) >> cl;
        Launch L(d, s, "ntt_tables", 1, n);
        fill_powers<<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(scale, n, base, first, cl);
    }
    if (lgn <= 12) {
        const size_t smem = (n + n / 2) * 8;
        const int threads = (int)std::min<size_t>(512, std::max<size_t>(32, n / 2));
        for (size_t r0 = 0; r0 < nrows; r0 += 65535) {
            const size_t g = std::min<size_t>(65535, nrows - r0);
            Launch L(d, s, "ntt_small", 1, g);
            ntt_small<<<(unsigned)g, threads, smem, s>>>(values + (r0 << lgn), (int)lgn, t->pw, scale, inverse);
        }
        TG_CUDA(cudaGetLastError());
        return TG_OK;
    }
    fast::Args a = {};
    a.pw = t->pw;
    a.pow7k = scale;
    a.lgk = (int)lgn;
    a.lgr = 0;
    a.P = 0;
    a.lgk1 = (int)(lgn + 1) / 2;
    a.lgk2 = (int)lgn / 2;
    if (inverse) {
        // pass M1's running scale steps by base^m along a thread's elements, m = RB·K2
        const uint64_t base = coset ? inv(shift) : 1;
        a.sstep[0] = pow(base, (uint64_t)fast_rb(a.lgk1) << a.lgk2);
    }
    size_t group = std::max<size_t>(1, d->cfg.lde_group_bytes / (n * 8));
    group = std::min<size_t>(group, std::min<size_t>(nrows, 65535));
    rc = d->scratch_y.ensure(group * n * 8);
    if (rc) return rc;
    uint64_t* tmp = (uint64_t*)d->scratch_y.ptr;
    const size_t tiles_k2 = n / fast_tile(a.lgk2), tiles_k1 = n / fast_tile(a.lgk1);
    for (size_t r0 = 0; r0 < nrows; r0 += group) {
        const unsigned g = (unsigned)std::min(group, nrows - r0);
        uint64_t* rows = values + (r0 << lgn);
        if (inverse) {
            a.rows = rows;
            a.y = tmp;
            a.z = rows;  // the coefficients land in place
            {
                Launch L(d, s, "ntt_pass_a", 1, g);
                rc = fast_pass(0, a.lgk2, dim3((unsigned)tiles_k2, g), a, s);
            }
            if (rc) return rc;
            {
                Launch L(d, s, "ntt_pass_m1", 1, g);
                rc = fast_pass(1, a.lgk1, dim3((unsigned)tiles_k1, g), a, s);
            }
            if (rc) return rc;
        } else {
            if (coset) {
                const size_t total = (size_t)g << lgn;
                Launch L(d, s, "ntt_scale", 1, g);
                ntt_scale<<<(unsigned)std::min<size_t>((total + 255) / 256, (size_t)d->sm_count * 16), 256, 0, s>>>(
                    rows, lgn, total, scale);
            }
            a.z = rows;  // pass M2 works in place
            a.out = tmp;
            {
                Launch L(d, s, "ntt_pass_m2", 1, g);
                rc = fast_pass(2, a.lgk1, dim3((unsigned)tiles_k1, g), a, s);
            }
            if (rc) return rc;
            {
                Launch L(d, s, "ntt_pass_c", 1, g);
                rc = fast_pass(3, a.lgk2, dim3((unsigned)tiles_k2, g), a, s);
            }
            if (rc) return rc;
            TG_CUDA(cudaMemcpyAsync(rows, tmp, ((size_t)g << lgn) * 8, cudaMemcpyDeviceToDevice, s));
        }
    }
    TG_CUDA(cudaGetLastError());
    return TG_OK;
}

}  // namespace tg
