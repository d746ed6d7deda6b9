// SPDX-License-Identifier: Apache-2.0 OR MIT
//
// The opening's device steps: the ColumnSink of the reference (crates/tessera-pcs/src/streaming/
// opening.rs:845-884; its GPU form is ColumnsSink, crates/tessera-prover/src/gpu.rs:196-398).
// P5 re-encodes the advice rows block by block (with their replayed masks) and keeps only the
// queried columns' symbols; P4, in the same pass over the rows, accumulates the combined rows
// Σ_r c[g][r]·row_r (one Fp2 row of k per group g) on the device until the opening collects them.
//
// The reference also interleaves two rate-1/2 cosets into a rate-1/4 codeword (its interleave2);
// here the encoder writes the 2^r cosets interleaved for any rate, so no such step exists.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "gl.cuh"
#include "internal.h"

namespace tg {

// out[r·m + q] = codewords[r·n + columns[q]], and 0 for a column at or past n (an index past
// the codeword reads nothing, as the reference's gather does).
__global__ void gather_columns_kernel(const uint64_t* cw, uint64_t n, uint32_t rows, const uint64_t* columns,
                                      uint32_t m, uint64_t* out) {
    const uint64_t total = (uint64_t)rows * m;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += stride) {
        const uint64_t r = i / m, c = columns[i % m];
        out[i] = c < n ? cw[r * n + c] : 0;
    }
}

constexpr int CR_GROUPS = 8;  // groups whose sums one pass keeps in registers

// acc[g][i] += Σ_r coeff[g][r]·values[r][i] over the block's rows, in Fp2 = (c0, c1) word pairs:
// each thread owns columns i, so no two threads write one sum; groups go CR_GROUPS at a time so
// that each value is read once per CR_GROUPS groups.
__global__ void combine_rows_kernel(const uint64_t* values, uint32_t rows, uint64_t k, const uint64_t* coeff,
                                    uint32_t groups, uint64_t* acc) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < k; i += stride) {
        for (uint32_t g0 = 0; g0 < groups; g0 += CR_GROUPS) {
            const uint32_t gs = min(groups - g0, (uint32_t)CR_GROUPS);
            fp2 s[CR_GROUPS];
#pragma unroll
            for (int g = 0; g < CR_GROUPS; g++)
                if (g < (int)gs) {
                    const ulonglong2 v = reinterpret_cast<const ulonglong2*>(acc)[(uint64_t)(g0 + g) * k + i];
                    s[g] = {v.x, v.y};
                }
            for (uint32_t r = 0; r < rows; r++) {
                const uint64_t x = values[(uint64_t)r * k + i];
#pragma unroll
                for (int g = 0; g < CR_GROUPS; g++)
                    if (g < (int)gs) {
                        const ulonglong2 c = __ldg(reinterpret_cast<const ulonglong2*>(coeff) + (uint64_t)(g0 + g) * rows + r);
                        s[g] = e_add(s[g], fp2{mul(c.x, x), mul(c.y, x)});
                    }
            }
#pragma unroll
            for (int g = 0; g < CR_GROUPS; g++)
                if (g < (int)gs)
                    reinterpret_cast<ulonglong2*>(acc)[(uint64_t)(g0 + g) * k + i] = make_ulonglong2(s[g].c0, s[g].c1);
        }
    }
}

// An answer to column queries on resident data: cols[q·rows + r] = cw[r·n + idx[q]] (each queried
// column's symbols of every row, in row order) and sib[t] = nodes[node[t]] (32-byte digests).
__global__ void gather_answer_kernel(const uint64_t* cw, uint64_t n, uint32_t rows, const uint64_t* idx, uint32_t m,
                                     uint64_t* cols, const uint64_t* nodes, const uint64_t* node, uint32_t ns,
                                     uint64_t* sib) {
    const uint64_t ncols = (uint64_t)rows * m, total = ncols + 4ull * ns;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += stride) {
        if (i < ncols) {
            const uint64_t q = i / rows, r = i % rows;
            cols[i] = cw[r * n + idx[q]];
        } else {
            const uint64_t j = i - ncols;
            sib[j] = nodes[4 * node[j >> 2] + (j & 3)];
        }
    }
}

int gather_answer(Device* d, const uint64_t* cw, uint64_t n, uint32_t rows, const uint64_t* idx, uint32_t m,
                  uint64_t* cols, const uint8_t* nodes, const uint64_t* node, uint32_t ns, uint8_t* sib,
                  cudaStream_t s) {
    const uint64_t total = (uint64_t)rows * m + 4ull * ns;
    if (total == 0) return TG_OK;
    const uint64_t blocks = std::min<uint64_t>((total + 255) / 256, (uint64_t)d->sm_count * 8);
    Launch L(d, s, "gather_answer", 1, total);
    gather_answer_kernel<<<(unsigned)blocks, 256, 0, s>>>(cw, n, rows, idx, m, cols, (const uint64_t*)nodes, node, ns,
                                                          (uint64_t*)sib);
    TG_CUDA(cudaGetLastError());
    return TG_OK;
}

static void zero(DevBuf& b, cudaStream_t s) {
    if (b.ptr) cudaMemsetAsync(b.ptr, 0, b.bytes, s);
}

}  // namespace tg

using namespace tg;

struct tg_column_sink {
    Device* d = nullptr;
    uint32_t lgk = 0, lgr = 0, P = 0, B = 0;
    uint64_t n = 0, m = 0;
    DevBuf columns, rows, masks, cw, out, coeff, sums;
    uint32_t groups = 0;  // 0 until the first combining block
};

extern "C" int tg_column_sink_open(tg_device* dev, uint32_t log_k, uint32_t log_inv_rate, uint32_t mask_coeffs,
                                   uint32_t block, const uint64_t* columns, size_t ncolumns, tg_column_sink** out) {
    Device* d = reinterpret_cast<Device*>(dev);
    if (!d || !out || (ncolumns && !columns)) return fail(TG_ERR_INVALID, "tg_column_sink_open: null argument");
    *out = nullptr;
    if (log_inv_rate < 1 || log_inv_rate > 4 || log_k > 24)
        return fail(TG_ERR_INVALID, "unsupported shape 2^%u rate 1/2^%u", log_k, log_inv_rate);
    if ((uint64_t)mask_coeffs > (1ull << log_k)) return fail(TG_ERR_INVALID, "%u mask coefficients exceed k", mask_coeffs);
    if (block == 0 || block > 65535) return fail(TG_ERR_INVALID, "a block of %u rows", block);
    if (ncolumns > 0xFFFFFFFFull) return fail(TG_ERR_INVALID, "too many columns");
    tg_column_sink* sk = new tg_column_sink();
    sk->d = d;
    sk->lgk = log_k;
    sk->lgr = log_inv_rate;
    sk->P = mask_coeffs;
    sk->B = block;
    sk->n = 1ull << (log_k + log_inv_rate);
    sk->m = ncolumns;
    const size_t k = (size_t)1 << log_k;
    int rc = sk->columns.ensure(std::max<size_t>(ncolumns, 1) * 8);
    if (!rc) rc = sk->rows.ensure(block * k * 8);
    if (!rc) rc = sk->masks.ensure(std::max<size_t>((size_t)block * mask_coeffs, 1) * 8);
    if (!rc) rc = sk->cw.ensure(block * sk->n * 8);
    if (!rc) rc = sk->out.ensure(std::max<size_t>((size_t)block * ncolumns, 1) * 8);
    if (!rc && ncolumns) {
        const cudaError_t e = cudaMemcpy(sk->columns.ptr, columns, ncolumns * 8, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) rc = cuda_fail(e, "columns");
    }
    if (rc) {
        delete sk;
        return rc;
    }
    *out = sk;
    return TG_OK;
}

// Encodes the block and gathers its queried symbols; with coefficients, first adds the block's
// combined rows to the sums.
static int sink_run(tg_column_sink* sk, const uint64_t* rows, size_t nrows, const uint64_t* masks,
                    const uint64_t* coefficients, size_t groups, uint64_t* out) {
    if (!sk || (nrows && !rows) || (sk->P && nrows && !masks) || (nrows && sk->m && !out))
        return fail(TG_ERR_INVALID, "column sink: null argument");
    if (nrows == 0 || nrows > sk->B) return fail(TG_ERR_INVALID, "a block of whole rows: 1 to %u, not %zu", sk->B, nrows);
    Device* d = sk->d;
    cudaStream_t s = d->stream;
    const size_t k = (size_t)1 << sk->lgk;
    if (coefficients) {
        if (groups == 0 || groups > 4096) return fail(TG_ERR_INVALID, "%zu groups", groups);
        if (sk->groups && sk->groups != groups) return fail(TG_ERR_STATE, "one group count per opening");
        if (!sk->groups) {
            int rc = sk->sums.ensure(groups * k * 16);
            if (rc) return rc;
            TG_CUDA(cudaMemsetAsync(sk->sums.ptr, 0, groups * k * 16, s));
            sk->groups = (uint32_t)groups;
        }
        int rc = sk->coeff.ensure(groups * nrows * 16);
        if (rc) return rc;
        TG_CUDA(cudaMemcpyAsync(sk->coeff.ptr, coefficients, groups * nrows * 16, cudaMemcpyHostToDevice, s));
    }
    host_prefault(rows, nrows * k * 8);
    TG_CUDA(cudaMemcpyAsync(sk->rows.ptr, rows, nrows * k * 8, cudaMemcpyHostToDevice, s));
    if (sk->P) host_prefault(masks, nrows * sk->P * 8);
    if (sk->P) TG_CUDA(cudaMemcpyAsync(sk->masks.ptr, masks, nrows * sk->P * 8, cudaMemcpyHostToDevice, s));
    std::lock_guard<std::mutex> lock(d->mu);
    if (coefficients) {
        const uint64_t blocks = std::min<uint64_t>((k + 255) / 256, (uint64_t)d->sm_count * 8);
        Launch L(d, s, "combine_rows", 1, k * nrows * groups);
        combine_rows_kernel<<<(unsigned)blocks, 256, 0, s>>>((const uint64_t*)sk->rows.ptr, (uint32_t)nrows, k,
                                                            (const uint64_t*)sk->coeff.ptr, (uint32_t)groups,
                                                            (uint64_t*)sk->sums.ptr);
        TG_CUDA(cudaGetLastError());
    }
    int rc = lde_encode(d, sk->lgk, sk->lgr, sk->P, (const uint64_t*)sk->rows.ptr, nrows,
                        sk->P ? (const uint64_t*)sk->masks.ptr : nullptr, (uint64_t*)sk->cw.ptr, s);
    if (rc) return rc;
    if (sk->m) {
        const uint64_t total = nrows * sk->m;
        const uint64_t blocks = std::min<uint64_t>((total + 255) / 256, (uint64_t)d->sm_count * 8);
        Launch L(d, s, "gather_columns", 1, total);
        gather_columns_kernel<<<(unsigned)blocks, 256, 0, s>>>((const uint64_t*)sk->cw.ptr, sk->n, (uint32_t)nrows,
                                                              (const uint64_t*)sk->columns.ptr, (uint32_t)sk->m,
                                                              (uint64_t*)sk->out.ptr);
        TG_CUDA(cudaGetLastError());
        TG_CUDA(cudaMemcpyAsync(out, sk->out.ptr, total * 8, cudaMemcpyDeviceToHost, s));
    }
    TG_CUDA(cudaStreamSynchronize(s));
    return TG_OK;
}

extern "C" int tg_column_sink_select(tg_column_sink* sk, const uint64_t* rows, size_t nrows, const uint64_t* masks,
                                     uint64_t* out) {
    return sink_run(sk, rows, nrows, masks, nullptr, 0, out);
}

extern "C" int tg_column_sink_select_combining(tg_column_sink* sk, const uint64_t* rows, size_t nrows,
                                               const uint64_t* masks, const uint64_t* coefficients, size_t groups,
                                               uint64_t* out) {
    if (!coefficients) return fail(TG_ERR_INVALID, "tg_column_sink_select_combining: null coefficients");
    return sink_run(sk, rows, nrows, masks, coefficients, groups, out);
}

extern "C" int tg_column_sink_combined(tg_column_sink* sk, uint64_t* out, size_t groups) {
    if (!sk) return fail(TG_ERR_INVALID, "tg_column_sink_combined: null sink");
    if (!sk->groups) return TG_OK;  // nothing combined
    if (!out || groups != sk->groups) return fail(TG_ERR_INVALID, "one combined row per group (%u)", sk->groups);
    const size_t k = (size_t)1 << sk->lgk;
    std::vector<uint64_t> w(groups * k * 2);
    cudaStream_t s = sk->d->stream;
    TG_CUDA(cudaMemcpyAsync(w.data(), sk->sums.ptr, w.size() * 8, cudaMemcpyDeviceToHost, s));
    zero(sk->sums, s);  // secret-class sums are cleared once collected
    TG_CUDA(cudaStreamSynchronize(s));
    sk->groups = 0;
    for (size_t i = 0; i < w.size(); i++) out[i] = add(out[i] % P, w[i]);
    memset(w.data(), 0, w.size() * 8);
    return TG_OK;
}

extern "C" int tg_column_sink_close(tg_column_sink* sk) {
    if (!sk) return TG_OK;
    cudaStream_t s = sk->d->stream;
    for (DevBuf* b : {&sk->rows, &sk->masks, &sk->cw, &sk->out, &sk->coeff, &sk->sums}) zero(*b, s);
    cudaStreamSynchronize(s);
    delete sk;
    return TG_OK;
}
