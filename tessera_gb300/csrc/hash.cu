// SPDX-License-Identifier: Apache-2.0 OR MIT
//
// Column chains and Merkle trees on the device: the reference's ColumnChains
// (crates/tessera-hash/src/columns.rs:72-104), MerkleTree (crates/tessera-hash/src/merkle.rs:10-16,
// 93-113) and the column-merge leaves of merge_segments (crates/tessera-pcs/src/streaming.rs:
// 382-438). Every hash is H(domain, x) = BLAKE3 derive-key-material under the domain's context
// key, one chunk long, so a digest is a chain of compressions over x's 64-byte blocks.
//
// One thread owns one column (or one tree node): it streams its message words straight from
// HBM, where consecutive threads read consecutive symbols of a row, so every load is coalesced,
// and its 8-word chaining value never leaves registers.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include "b3.cuh"
#include "internal.h"

namespace tg {

struct Key {
    uint32_t w[8];
};

// H(domain, id ‖ u64 j) for column j: 40 bytes, one block.
__global__ void column_init_kernel(Key key, Key id, uint64_t ncols, uint32_t* chains) {
    const uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= ncols) return;
    uint32_t m[16];
#pragma unroll
    for (int i = 0; i < 8; i++) m[i] = id.w[i];
    m[8] = (uint32_t)j;
    m[9] = (uint32_t)(j >> 32);
#pragma unroll
    for (int i = 10; i < 16; i++) m[i] = 0;
    uint32_t cv[8];
#pragma unroll
    for (int i = 0; i < 8; i++) cv[i] = key.w[i];
    b3::compress_cv(cv, m, 0, 40, b3::CHUNK_START | b3::CHUNK_END | b3::ROOT | b3::DERIVE_KEY_MATERIAL);
    uint4* out = reinterpret_cast<uint4*>(chains + 8 * j);
    out[0] = make_uint4(cv[0], cv[1], cv[2], cv[3]);
    out[1] = make_uint4(cv[4], cv[5], cv[6], cv[7]);
}

// d_j ← H("column-step", d_j ‖ symbols of `cnt` rows) for every block of `block` rows, in order.
// rows: count x ncols, row r of the group at rows + r*ld. The message of one step is 8 chain
// words then 2 words per symbol; it is consumed 16 words (one BLAKE3 block) at a time.
__global__ void __launch_bounds__(128) column_absorb_kernel(Key key, uint64_t ncols, const uint64_t* rows, size_t ld,
                                                            uint32_t count, uint32_t block, uint32_t* chains) {
    const uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= ncols) return;
    uint32_t cv[8];
    {
        const uint4* in = reinterpret_cast<const uint4*>(chains + 8 * j);
        uint4 a = in[0], b = in[1];
        cv[0] = a.x, cv[1] = a.y, cv[2] = a.z, cv[3] = a.w, cv[4] = b.x, cv[5] = b.y, cv[6] = b.z, cv[7] = b.w;
    }
    for (uint32_t r0 = 0; r0 < count; r0 += block) {
        const uint32_t cnt = count - r0 < block ? count - r0 : block;
        const uint32_t words = 8 + 2 * cnt;  // ≤ 256 words (one chunk) since cnt ≤ 124
        const uint32_t nblocks = (words + 15) / 16;
        uint32_t h[8];
#pragma unroll
        for (int i = 0; i < 8; i++) h[i] = key.w[i];
        const uint64_t* col = rows + (size_t)r0 * ld + j;
        for (uint32_t b = 0; b < nblocks; b++) {
            uint32_t m[16];
            if (b == 0) {
#pragma unroll
                for (int i = 0; i < 8; i++) m[i] = cv[i];
#pragma unroll
                for (int s = 0; s < 4; s++) {
                    const uint64_t v = (uint32_t)s < cnt ? col[(size_t)s * ld] : 0;
                    m[8 + 2 * s] = (uint32_t)v;
                    m[9 + 2 * s] = (uint32_t)(v >> 32);
                }
            } else {
                const uint32_t s0 = 8 * b - 4;  // first symbol of this block
#pragma unroll
                for (int s = 0; s < 8; s++) {
                    const uint64_t v = s0 + s < cnt ? col[(size_t)(s0 + s) * ld] : 0;
                    m[2 * s] = (uint32_t)v;
                    m[2 * s + 1] = (uint32_t)(v >> 32);
                }
            }
            const bool last = b + 1 == nblocks;
            const uint32_t len = last ? 4 * (words - 16 * b) : 64;
            const uint32_t flags = b3::DERIVE_KEY_MATERIAL | (b == 0 ? b3::CHUNK_START : 0) |
                                   (last ? (b3::CHUNK_END | b3::ROOT) : 0);
            b3::compress_cv(h, m, 0, len, flags);
        }
#pragma unroll
        for (int i = 0; i < 8; i++) cv[i] = h[i];
    }
    uint4* out = reinterpret_cast<uint4*>(chains + 8 * j);
    out[0] = make_uint4(cv[0], cv[1], cv[2], cv[3]);
    out[1] = make_uint4(cv[4], cv[5], cv[6], cv[7]);
}

// H("merkle-node", L ‖ R) of a 64-byte message: one compression.
__device__ __forceinline__ void merkle_pair(const Key& key, const uint32_t* l, const uint32_t* r, uint32_t* out) {
    uint32_t m[16];
#pragma unroll
    for (int i = 0; i < 8; i++) {
        m[i] = l[i];
        m[8 + i] = r[i];
    }
    uint32_t cv[8];
#pragma unroll
    for (int i = 0; i < 8; i++) cv[i] = key.w[i];
    b3::compress_cv(cv, m, 0, 64, b3::CHUNK_START | b3::CHUNK_END | b3::ROOT | b3::DERIVE_KEY_MATERIAL);
#pragma unroll
    for (int i = 0; i < 8; i++) out[i] = cv[i];
}

// Up to `levels` levels of the tree above `width` nodes at `in`: each CTA of T threads takes 2T
// nodes and climbs while it still has pairs, writing every level it makes to `out` (the
// level's offset within the node array is level_off[ℓ]). The climb stays in shared memory.
__global__ void __launch_bounds__(256) merkle_levels_kernel(Key key, const uint32_t* in, uint64_t width,
                                                            uint32_t* nodes, uint64_t out_off0, int levels) {
    __shared__ uint32_t sm[256 * 8];
    const uint64_t base = (uint64_t)blockIdx.x * 2 * blockDim.x;  // first input node of this CTA
    uint64_t lvl_width = width / 2;                                  // nodes at the next level
    uint64_t off = out_off0;                                         // where the next level starts
    int active = blockDim.x;
    const uint64_t pair = base / 2 + threadIdx.x;
    if (pair < lvl_width) {
        uint32_t o[8];
        merkle_pair(key, in + 16 * pair, in + 16 * pair + 8, o);
#pragma unroll
        for (int i = 0; i < 8; i++) {
            sm[threadIdx.x * 8 + i] = o[i];
            nodes[8 * (off + pair) + i] = o[i];
        }
    }
    __syncthreads();
    uint64_t first = base / 2;  // index of this CTA's first node at the current level
    for (int l = 1; l < levels && lvl_width > 1 && active > 1; l++) {
        off += lvl_width;
        lvl_width /= 2;
        active /= 2;
        first /= 2;
        const uint64_t idx = first + threadIdx.x;
        uint32_t o[8];
        const bool live = threadIdx.x < (unsigned)active && idx < lvl_width;
        if (live) merkle_pair(key, sm + 16 * threadIdx.x, sm + 16 * threadIdx.x + 8, o);
        __syncthreads();
        if (live) {
#pragma unroll
            for (int i = 0; i < 8; i++) {
                sm[threadIdx.x * 8 + i] = o[i];
                nodes[8 * (off + idx) + i] = o[i];
            }
        }
        __syncthreads();
    }
}

// leaf_j = H("column-merge", d_j^(1) ‖ … ‖ d_j^(S)), segs: S x n digests.
__global__ void column_merge_kernel(Key key, const uint32_t* segs, uint32_t nseg, uint64_t n, uint32_t* leaves) {
    const uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const uint32_t words = 8 * nseg;
    const uint32_t nblocks = words == 0 ? 1 : (words + 15) / 16;
    uint32_t h[8];
#pragma unroll
    for (int i = 0; i < 8; i++) h[i] = key.w[i];
    for (uint32_t b = 0; b < nblocks; b++) {
        uint32_t m[16];
#pragma unroll
        for (int i = 0; i < 16; i++) {
            const uint32_t w = 16 * b + i;
            m[i] = w < words ? segs[8 * ((size_t)(w / 8) * n + j) + (w % 8)] : 0;
        }
        const bool last = b + 1 == nblocks;
        const uint32_t len = last ? 4 * (words - 16 * b) : 64;
        b3::compress_cv(h, m, 0, len,
                        b3::DERIVE_KEY_MATERIAL | (b == 0 ? b3::CHUNK_START : 0) | (last ? (b3::CHUNK_END | b3::ROOT) : 0));
    }
#pragma unroll
    for (int i = 0; i < 8; i++) leaves[8 * j + i] = h[i];
}

static Key key_of(const char* name) {
    Key k;
    context_key(name, k.w);
    return k;
}

static Key words_of(const uint8_t b[32]) {
    Key k;
    for (int i = 0; i < 8; i++) k.w[i] = b3::le32(b + 4 * i);
    return k;
}

int column_init(Device* d, const uint8_t id[32], uint64_t ncols, uint8_t* chains, cudaStream_t s) {
    if (ncols == 0) return TG_OK;
    static const Key key = key_of("column-init");
    Launch L(d, s, "column_init", 1, ncols);
    column_init_kernel<<<(unsigned)((ncols + 255) / 256), 256, 0, s>>>(key, words_of(id), ncols, (uint32_t*)chains);
    TG_CUDA(cudaGetLastError());
    return TG_OK;
}

int column_absorb(Device* d, uint8_t* chains, uint64_t ncols, const uint64_t* rows, size_t ld, size_t count,
                  uint32_t block, cudaStream_t s) {
    if (ncols == 0 || count == 0) return TG_OK;
    if (block == 0 || block > 124)
        return fail(TG_ERR_INVALID, "row block %u outside 1..124 (one BLAKE3 chunk per step)", block);
    static const Key key = key_of("column-step");
    Launch L(d, s, "column_absorb", 1, ncols * count);
    column_absorb_kernel<<<(unsigned)((ncols + 127) / 128), 128, 0, s>>>(key, ncols, rows, ld, (uint32_t)count, block,
                                                                         (uint32_t*)chains);
    TG_CUDA(cudaGetLastError());
    return TG_OK;
}

int merkle_tree(Device* d, const uint8_t* leaves, size_t n, uint8_t* nodes, cudaStream_t s) {
    if (n == 0 || (n & (n - 1))) return fail(TG_ERR_INVALID, "a Merkle tree needs a power-of-two number of leaves, not %zu", n);
    static const Key key = key_of("merkle-node");
    if (leaves != nodes) TG_CUDA(cudaMemcpyAsync(nodes, leaves, n * 32, cudaMemcpyDeviceToDevice, s));
    uint64_t width = n, in_off = 0;
    const int T = 256, per_launch = 9;  // 2T = 512 nodes climb 9 levels in one CTA
    while (width > 1) {
        const uint64_t pairs = width / 2;
        const unsigned grid = (unsigned)((pairs + T - 1) / T);
        const int threads = pairs < (uint64_t)T ? (int)pairs : T;
        int levels = 0;
        for (uint64_t w = width, a = 2 * (uint64_t)threads; w > 1 && a > 1 && levels < per_launch; w /= 2, a /= 2) levels++;
        Launch L(d, s, "merkle", 1, pairs);
        merkle_levels_kernel<<<grid, threads, 0, s>>>(key, (const uint32_t*)nodes + 8 * in_off, width, (uint32_t*)nodes,
                                                      in_off + width, levels);
        for (int l = 0; l < levels; l++) {
            in_off += width;
            width /= 2;
        }
    }
    TG_CUDA(cudaGetLastError());
    return TG_OK;
}

int column_merge(Device* d, const uint8_t* segs, size_t nseg, uint64_t n, uint8_t* leaves, cudaStream_t s) {
    if (n == 0) return TG_OK;
    if (nseg > 32) return fail(TG_ERR_INVALID, "%zu segments exceed one BLAKE3 chunk of digests (32)", nseg);
    static const Key key = key_of("column-merge");
    Launch L(d, s, "column_merge", 1, n);
    column_merge_kernel<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(key, (const uint32_t*)segs, (uint32_t)nseg, n,
                                                                    (uint32_t*)leaves);
    TG_CUDA(cudaGetLastError());
    return TG_OK;
}

// ---- the advice mask stream (crates/tessera-hash/src/domain.rs:83-127, ProverDomain::AdviceMasks)
//
// The stream is BLAKE3's extended output of H("advice-masks", seed) in derive-key mode: output
// block t (64 bytes, eight little-endian words) is the root compression of the seed's one block at
// counter t. The masks are its words below p, in order (rejection sampling). Output blocks are
// independent, so each thread makes one; the words kept are placed by a count, a scan of the
// per-CTA counts, and a second pass that recomputes and scatters.

constexpr int MASK_THREADS = 256;

struct MaskSeed {
    uint32_t key[8];
    uint32_t m[16];
    uint32_t len;
};

__device__ __forceinline__ void mask_block(const MaskSeed& ms, uint64_t t, uint64_t w[8]) {
    uint32_t out[16];
    b3::compress_full(ms.key, ms.m, t, ms.len,
                      b3::DERIVE_KEY_MATERIAL | b3::CHUNK_START | b3::CHUNK_END | b3::ROOT, out);
#pragma unroll
    for (int i = 0; i < 8; i++) w[i] = (uint64_t)out[2 * i] | ((uint64_t)out[2 * i + 1] << 32);
}

// counts[b]: the words below p among CTA b's output blocks (one a thread).
__global__ void __launch_bounds__(MASK_THREADS) mask_count_kernel(MaskSeed ms, uint64_t nblocks, uint32_t* counts) {
    __shared__ uint32_t part[MASK_THREADS / 32];
    const uint64_t t = (uint64_t)blockIdx.x * MASK_THREADS + threadIdx.x;
    uint32_t c = 0;
    if (t < nblocks) {
        uint64_t w[8];
        mask_block(ms, t, w);
#pragma unroll
        for (int i = 0; i < 8; i++) c += w[i] < P;
    }
    for (int o = 16; o; o >>= 1) c += __shfl_down_sync(0xFFFFFFFFu, c, o);
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t sum = 0;
        for (int i = 0; i < MASK_THREADS / 32; i++) sum += part[i];
        counts[blockIdx.x] = sum;
    }
}

// offsets[b] = Σ_{b' < b} counts[b'], offsets[n] the total; one CTA, in chunks of its width.
__global__ void __launch_bounds__(1024) mask_scan_kernel(const uint32_t* counts, uint32_t n, uint64_t* offsets) {
    __shared__ uint64_t warp_sum[32];
    __shared__ uint64_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (uint32_t base = 0; base < n; base += 1024) {
        const uint32_t i = base + threadIdx.x;
        const uint64_t v = i < n ? counts[i] : 0;
        uint64_t x = v;  // inclusive scan within the warp
        for (int o = 1; o < 32; o <<= 1) {
            const uint64_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
            if ((threadIdx.x & 31) >= (unsigned)o) x += y;
        }
        if ((threadIdx.x & 31) == 31) warp_sum[threadIdx.x >> 5] = x;
        __syncthreads();
        if (threadIdx.x < 32) {
            uint64_t ws = warp_sum[threadIdx.x];
            for (int o = 1; o < 32; o <<= 1) {
                const uint64_t y = __shfl_up_sync(0xFFFFFFFFu, ws, o);
                if (threadIdx.x >= (unsigned)o) ws += y;
            }
            warp_sum[threadIdx.x] = ws;  // inclusive over warps
        }
        __syncthreads();
        const uint64_t before = carry + ((threadIdx.x >> 5) ? warp_sum[(threadIdx.x >> 5) - 1] : 0) + x - v;
        if (i < n) offsets[i] = before;
        __syncthreads();
        if (threadIdx.x == 0) carry += warp_sum[31];
        __syncthreads();
    }
    if (threadIdx.x == 0) offsets[n] = carry;
}

// The kept words of CTA b's blocks, in order, from position offsets[b]; those at positions in
// [first, first + count) land in out[position − first].
__global__ void __launch_bounds__(MASK_THREADS) mask_scatter_kernel(MaskSeed ms, uint64_t nblocks,
                                                                    const uint64_t* offsets, uint64_t first,
                                                                    uint64_t count, uint64_t* out) {
    __shared__ uint32_t part[MASK_THREADS / 32];
    const uint64_t t = (uint64_t)blockIdx.x * MASK_THREADS + threadIdx.x;
    uint64_t w[8];
    uint32_t c = 0;
    if (t < nblocks) {
        mask_block(ms, t, w);
#pragma unroll
        for (int i = 0; i < 8; i++) c += w[i] < P;
    }
    // exclusive prefix of c over the CTA
    uint32_t x = c;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
        if ((threadIdx.x & 31) >= (unsigned)o) x += y;
    }
    if ((threadIdx.x & 31) == 31) part[threadIdx.x >> 5] = x;
    __syncthreads();
    uint32_t warps_before = 0;
    for (int i = 0; i < (int)(threadIdx.x >> 5); i++) warps_before += part[i];
    if (t >= nblocks) return;
    uint64_t pos = offsets[blockIdx.x] + warps_before + x - c;
#pragma unroll
    for (int i = 0; i < 8; i++) {
        if (w[i] < P) {
            if (pos >= first && pos - first < count) out[pos - first] = w[i];
            pos++;
        }
    }
}

int advice_masks(Device* d, const uint8_t* seed, size_t seed_len, uint64_t first, uint64_t count, uint64_t* out,
                 cudaStream_t s) {
    if (seed_len > 64) return fail(TG_ERR_INVALID, "a seed of %zu bytes: at most one BLAKE3 block (64)", seed_len);
    if (count == 0) return TG_OK;
    MaskSeed ms;
    context_key("advice-masks", ms.key);
    uint8_t block[64] = {0};
    memcpy(block, seed, seed_len);
    for (int i = 0; i < 16; i++) ms.m[i] = b3::le32(block + 4 * i);
    ms.len = (uint32_t)seed_len;
    // words drawn: the values wanted and some slack for rejected words (each word is rejected with
    // probability below 2^-32); drawn again with more if the slack ran out
    for (uint64_t slack = 64;; slack *= 16) {
        const uint64_t words = first + count + slack;
        const uint64_t nblocks = (words + 7) / 8;
        const uint64_t ctas = (nblocks + MASK_THREADS - 1) / MASK_THREADS;
        if (ctas > 0xFFFFFFFFull) return fail(TG_ERR_INVALID, "%llu mask values", (unsigned long long)(first + count));
        int rc = d->scratch_aux.ensure(ctas * 4 + (ctas + 1) * 8 + 8);
        if (rc) return rc;
        uint64_t* offsets = (uint64_t*)d->scratch_aux.ptr;
        uint32_t* counts = (uint32_t*)(offsets + ctas + 1);
        {
            Launch L(d, s, "advice_masks", 3, words);
            mask_count_kernel<<<(unsigned)ctas, MASK_THREADS, 0, s>>>(ms, nblocks, counts);
            mask_scan_kernel<<<1, 1024, 0, s>>>(counts, (uint32_t)ctas, offsets);
            mask_scatter_kernel<<<(unsigned)ctas, MASK_THREADS, 0, s>>>(ms, nblocks, offsets, first, count, out);
        }
        TG_CUDA(cudaGetLastError());
        uint64_t total = 0;
        TG_CUDA(cudaMemcpyAsync(&total, offsets + ctas, 8, cudaMemcpyDeviceToHost, s));
        TG_CUDA(cudaStreamSynchronize(s));
        if (total >= first + count) return TG_OK;
    }
}

}  // namespace tg
