// SPDX-License-Identifier: Apache-2.0 OR MIT
//
// The C ABI of libtessera_gb300: device handles, errors, the encoding and hashing entry
// points, the resident commitment, and the two streaming sinks (BlockSink, MatrixSink) that
// stand in for the reference's AdviceSink and GpuWeights (crates/tessera-prover/src/gpu.rs).
#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>
#include <unistd.h>

#include <algorithm>
#include <string>
#include <vector>

#include "b3.cuh"
#include "gl.cuh"
#include "internal.h"

namespace tg {

static thread_local std::string g_last_error;

int fail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return code;
}

int cuda_fail(cudaError_t e, const char* what) {
    const int code = (e == cudaErrorMemoryAllocation) ? TG_ERR_NOMEM : TG_ERR_CUDA;
    return fail(code, "%s: %s", what, cudaGetErrorString(e));
}

int DevBuf::ensure(size_t want) {
    if (want <= bytes && ptr) return TG_OK;
    release();
    if (want == 0) want = 16;
    cudaError_t e = cudaMalloc(&ptr, want);
    if (e != cudaSuccess) {
        ptr = nullptr;
        bytes = 0;
        cudaGetLastError();
        return cuda_fail(e, "cudaMalloc");
    }
    bytes = want;
    return TG_OK;
}

void DevBuf::release() {
    if (ptr && owned) cudaFree(ptr);
    ptr = nullptr;
    bytes = 0;
    owned = true;
}

int readback_ensure(Device* d, size_t bytes) {
    if (d->readback_bytes >= bytes) return TG_OK;
    if (d->readback) cudaFreeHost(d->readback);
    d->readback = nullptr;
    d->readback_bytes = 0;
    const size_t want = std::max<size_t>(bytes, 64 << 10);
    TG_CUDA(cudaHostAlloc((void**)&d->readback, want, cudaHostAllocDefault));
    d->readback_bytes = want;
    return TG_OK;
}

int spare_take(Device* d, DevBuf& b, size_t want) {
    if (want == 0) want = 16;
    {
        std::lock_guard<std::mutex> lock(d->spare_mu);
        auto it = d->spare.lower_bound(want);
        if (it != d->spare.end() && it->first / 2 <= want) {
            b.release();
            b.ptr = it->second;
            b.bytes = it->first;
            d->spare_bytes -= it->first;
            d->spare.erase(it);
            return TG_OK;
        }
    }
    if (b.ensure(want) == TG_OK) return TG_OK;
    spare_trim(d);  // the cache gives way to a new allocation
    return b.ensure(want);
}

void spare_give(Device* d, DevBuf& b) {
    bool over = false;
    if (b.ptr && b.owned) {
        std::lock_guard<std::mutex> lock(d->spare_mu);
        d->spare.emplace(b.bytes, b.ptr);
        d->spare_bytes += b.bytes;
        over = d->spare_cap && d->spare_bytes > d->spare_cap;
    }
    b.ptr = nullptr;
    b.bytes = 0;
    b.owned = true;
    if (over) spare_trim(d);
}

void spare_trim(Device* d) {
    std::multimap<size_t, void*> drop;
    {
        std::lock_guard<std::mutex> lock(d->spare_mu);
        drop.swap(d->spare);
        d->spare_bytes = 0;
    }
    if (drop.empty()) return;
    for (auto& kv : drop) cudaMemsetAsync(kv.second, 0, kv.first, d->stream);
    cudaStreamSynchronize(d->stream);
    for (auto& kv : drop) cudaFree(kv.second);
    cudaGetLastError();
}

cudaStream_t pick_stream(Device* d, void* stream) { return stream ? (cudaStream_t)stream : d->stream; }

static cudaEvent_t take_event(Device* d) {
    if (!d->event_pool.empty()) {
        cudaEvent_t e = d->event_pool.back();
        d->event_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
    return e;
}

Launch::Launch(Device* d_, cudaStream_t s_, const char* name, uint64_t nkernels, uint64_t units) : d(d_), s(s_) {
    if (d->capturing) {
        d->captured += nkernels;
        return;
    }
    d->launches += nkernels;
    if (!d->prof_on) return;
    std::lock_guard<std::mutex> g(d->prof_mu);
    ProfRec r{name, take_event(d), take_event(d), units};
    if (!r.begin || !r.end) return;
    cudaEventRecord(r.begin, s);
    d->prof.push_back(r);
    idx = (int)d->prof.size() - 1;
}

Launch::~Launch() {
    if (idx < 0) return;
    std::lock_guard<std::mutex> g(d->prof_mu);
    cudaEventRecord(d->prof[idx].end, s);
}

// Zeroes a secret-class device buffer before it is released (the reference zeroes its device
// copies of rows and masks, crates/tessera-prover/src/gpu.rs:656-665).
static void clear(DevBuf& b, cudaStream_t s) {
    if (b.ptr) cudaMemsetAsync(b.ptr, 0, b.bytes, s);
}

// Gathers the queried symbols of each row: out[r*nq + q] = cw[r*n + queries[q]].
__global__ void gather_kernel(const uint64_t* cw, uint64_t n, const uint64_t* queries, uint64_t nq, uint64_t nrows,
                              uint64_t* out) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nq * nrows) return;
    const uint64_t r = i / nq, q = i % nq;
    out[i] = cw[r * n + queries[q]];
}

// ---- proof of work -----------------------------------------------------------------------------

struct PowMsg {
    uint32_t key[8];
    uint32_t words[64];  // state ‖ u64 len ‖ label ‖ (nonce), zero padded; ≤ 256 bytes
    uint32_t len;        // message bytes
    uint32_t nonce_off;  // byte offset of the nonce
    uint32_t bits;
};

__global__ void grind_kernel(PowMsg msg, uint64_t base, uint64_t count, unsigned long long* found) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t nonce = base + i;
        if (nonce >= *found) return;
        uint32_t h[8];
        for (int w = 0; w < 8; w++) h[w] = msg.key[w];
        const uint32_t nb = (msg.len + 63) / 64;
        for (uint32_t b = 0; b < nb; b++) {
            uint32_t m[16];
            for (int w = 0; w < 16; w++) m[w] = msg.words[16 * b + w];
            for (int k = 0; k < 8; k++) {
                const uint32_t pos = msg.nonce_off + k;
                if (pos >= 64 * b && pos < 64 * b + 64) {
                    const uint32_t byte = (uint32_t)(nonce >> (8 * k)) & 0xFF;
                    m[(pos - 64 * b) / 4] |= byte << (8 * ((pos - 64 * b) % 4));
                }
            }
            const bool last = b + 1 == nb;
            b3::compress_cv(h, m, 0, last ? msg.len - 64 * b : 64,
                            b3::DERIVE_KEY_MATERIAL | (b == 0 ? b3::CHUNK_START : 0) | (last ? (b3::CHUNK_END | b3::ROOT) : 0));
        }
        // leading zero bits, most significant bit of byte 0 first
        uint32_t zeros = 0;
        for (int w = 0; w < 8; w++) {
            const uint32_t be = __byte_perm(h[w], 0, 0x0123);
            if (be) {
                zeros += __clz(be);
                break;
            }
            zeros += 32;
        }
        if (zeros >= msg.bits) atomicMin(found, (unsigned long long)nonce);
    }
}

}  // namespace tg

using namespace tg;

struct tg_sink {
    Device* d;
    uint32_t lgk, lgr, P, B;
    uint64_t n;
    DevBuf chains, rows, masks, cw;
    bool closed = false, finished = false;
};

struct tg_matrix {
    Device* d;
    uint32_t lgk, lgr, B;
    uint64_t n, nq;
    DevBuf chains, rows, cw, queries, answers;
    bool closed = false, finished = false;
};

namespace tg {
void host_prefault(const void* p, size_t bytes) {
    if (!p || !bytes) return;
    static const size_t page = [] {
        const long v = sysconf(_SC_PAGESIZE);
        return v > 0 ? (size_t)v : (size_t)4096;
    }();
    const volatile uint8_t* b = static_cast<const volatile uint8_t*>(p);
    uint8_t acc = 0;
    for (size_t i = 0; i < bytes; i += page) acc ^= b[i];
    acc ^= b[bytes - 1];
    (void)acc;
}
}  // namespace tg

extern "C" {

int tg_version(void) { return 1; }

const char* tg_last_error(void) { return g_last_error.c_str(); }

int tg_device_open(int ordinal, const tg_config* cfg, tg_device** out) {
    if (!out) return fail(TG_ERR_INVALID, "tg_device_open: null out");
    *out = nullptr;
    int count = 0;
    TG_CUDA(cudaGetDeviceCount(&count));
    if (ordinal < 0 || ordinal >= count) return fail(TG_ERR_INVALID, "no CUDA device %d (%d present)", ordinal, count);
    TG_CUDA(cudaSetDevice(ordinal));
    Device* d = new Device();
    d->ordinal = ordinal;
    memset(&d->cfg, 0, sizeof d->cfg);
    if (cfg) d->cfg = *cfg;
    if (!d->cfg.level_budget_bytes) d->cfg.level_budget_bytes = 16ull << 30;
    if (!d->cfg.level_min_entries) d->cfg.level_min_entries = 1ull << 14;
    if (!d->cfg.lde_group_bytes) d->cfg.lde_group_bytes = 768ull << 20;
    cudaError_t e = cudaStreamCreateWithFlags(&d->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete d;
        return cuda_fail(e, "cudaStreamCreate");
    }
    cudaDeviceProp prop;
    e = cudaGetDeviceProperties(&prop, ordinal);
    if (e != cudaSuccess) {
        cudaStreamDestroy(d->stream);
        delete d;
        return cuda_fail(e, "cudaGetDeviceProperties");
    }
    if (prop.major * 10 + prop.minor < 100) {
        cudaStreamDestroy(d->stream);
        delete d;
        return fail(TG_ERR_INVALID, "device %d is sm_%d%d; this library is built for sm_103a", ordinal, prop.major,
                    prop.minor);
    }
    d->sm_count = prop.multiProcessorCount;
    d->smem_optin = prop.sharedMemPerBlockOptin;
    d->spare_cap = prop.totalGlobalMem / 2;
    *out = reinterpret_cast<tg_device*>(d);
    return TG_OK;
}

int tg_device_close(tg_device* dev) {
    Device* d = reinterpret_cast<Device*>(dev);
    if (!d) return TG_OK;
    cudaSetDevice(d->ordinal);
    cudaStreamSynchronize(d->stream);
    for (auto& r : d->prof) {
        cudaEventDestroy(r.begin);
        cudaEventDestroy(r.end);
    }
    for (auto e : d->event_pool) cudaEventDestroy(e);
    for (auto& kv : d->tables) {
        cudaFree(kv.second.pw);
        cudaFree(kv.second.pow7k);
    }
    clear(d->scratch_y, d->stream);
    clear(d->scratch_z, d->stream);
    cudaStreamSynchronize(d->stream);
    if (d->copy_stream) {
        cudaStreamSynchronize(d->copy_stream);
        cudaStreamDestroy(d->copy_stream);
    }
    for (int b = 0; b < 2; b++) {
        if (d->staged[b]) cudaEventDestroy(d->staged[b]);
        if (d->consumed[b]) cudaEventDestroy(d->consumed[b]);
    }
    for (cudaEvent_t& e : d->ramp)
        if (e) cudaEventDestroy(e);
    if (d->readback) cudaFreeHost(d->readback);
    d->stage_rows.release();
    d->stage_cw.release();
    d->stage_nodes.release();
    for (Worker* w : d->workers) {
        cudaStreamSynchronize(w->s);
        cudaStreamDestroy(w->s);
        cudaEventDestroy(w->done);
        delete w;
    }
    if (d->fork) cudaEventDestroy(d->fork);
    d->batch_roots.release();
    spare_trim(d);
    d->scratch_y.release();
    d->scratch_z.release();
    d->scratch_misc.release();
    d->scratch_aux.release();
    d->scratch_sc.release();
    d->err.release();
    cudaStreamDestroy(d->stream);
    delete d;
    return TG_OK;
}

int tg_profile_enable(tg_device* dev, int on) {
    Device* d = reinterpret_cast<Device*>(dev);
    if (!d) return fail(TG_ERR_INVALID, "null device");
    d->prof_on = on != 0;
    return TG_OK;
}

int tg_profile_read(tg_device* dev, char* names, size_t names_len, double* ms, uint64_t* launches, uint64_t* units,
                    size_t cap, size_t* count) {
    Device* d = reinterpret_cast<Device*>(dev);
    if (!d || !count) return fail(TG_ERR_INVALID, "tg_profile_read: null argument");
    std::lock_guard<std::mutex> g(d->prof_mu);
    std::vector<std::string> keys;
    std::vector<double> tot;
    std::vector<uint64_t> cnt, un;
    for (auto& r : d->prof) {
        float t = 0;
        TG_CUDA(cudaEventSynchronize(r.end));
        TG_CUDA(cudaEventElapsedTime(&t, r.begin, r.end));
        size_t i = 0;
        while (i < keys.size() && keys[i] != r.name) i++;
        if (i == keys.size()) {
            keys.push_back(r.name);
            tot.push_back(0);
            cnt.push_back(0);
            un.push_back(0);
        }
        tot[i] += t;
        cnt[i] += 1;
        un[i] += r.units;
        d->event_pool.push_back(r.begin);
        d->event_pool.push_back(r.end);
    }
    d->prof.clear();
    *count = keys.size();
    std::string joined;
    for (size_t i = 0; i < keys.size(); i++) {
        if (i < cap) {
            if (ms) ms[i] = tot[i];
            if (launches) launches[i] = cnt[i];
            if (units) units[i] = un[i];
        }
        joined += keys[i];
        joined += '\n';
    }
    if (names && names_len) {
        const size_t m = std::min(names_len - 1, joined.size());
        memcpy(names, joined.data(), m);
        names[m] = 0;
    }
    return TG_OK;
}

int tg_device_stream(tg_device* dev, void** stream) {
    Device* d = reinterpret_cast<Device*>(dev);
    if (!d || !stream) return fail(TG_ERR_INVALID, "tg_device_stream: null argument");
    *stream = (void*)d->stream;
    return TG_OK;
}

int tg_device_launches(tg_device* dev, uint64_t* launches) {
    Device* d = reinterpret_cast<Device*>(dev);
    if (!d || !launches) return fail(TG_ERR_INVALID, "tg_device_launches: null argument");
    *launches = d->launches.load();
    return TG_OK;
}

int tg_device_trim(tg_device* dev) {
    Device* d = reinterpret_cast<Device*>(dev);
    if (!d) return fail(TG_ERR_INVALID, "null device");
    spare_trim(d);
    return TG_OK;
}

int tg_host_prefault(const void* p, size_t bytes) {
    if (!p && bytes) return fail(TG_ERR_INVALID, "tg_host_prefault: null buffer");
    host_prefault(p, bytes);
    return TG_OK;
}

int tg_device_sync(tg_device* dev) {
    Device* d = reinterpret_cast<Device*>(dev);
    if (!d) return fail(TG_ERR_INVALID, "null device");
    TG_CUDA(cudaStreamSynchronize(d->stream));
    return TG_OK;
}

int tg_encode_rows_dev(tg_device* dev, uint32_t log_k, uint32_t log_inv_rate, uint32_t mask_coeffs, const uint64_t* rows,
                       size_t nrows, const uint64_t* masks, uint64_t* codewords, void* stream) {
    Device* d = reinterpret_cast<Device*>(dev);
    if (!d || (nrows && (!rows || !codewords))) return fail(TG_ERR_INVALID, "tg_encode_rows_dev: null argument");
    std::lock_guard<std::mutex> lock(d->mu);
    return lde_encode(d, log_k, log_inv_rate, mask_coeffs, rows, nrows, masks, codewords, pick_stream(d, stream));
}

int tg_encode_rows(tg_device* dev, uint32_t log_k, uint32_t log_inv_rate, uint32_t mask_coeffs, const uint64_t* rows,
                   size_t nrows, const uint64_t* masks, uint64_t* codewords) {
    Device* d = reinterpret_cast<Device*>(dev);
    if (!d || (nrows && (!rows || !codewords))) return fail(TG_ERR_INVALID, "tg_encode_rows: null argument");
    if (log_inv_rate < 1 || log_inv_rate > 4 || log_k > 24) return fail(TG_ERR_INVALID, "unsupported shape 2^%u rate 1/2^%u", log_k, log_inv_rate);
    if (nrows == 0) return TG_OK;
    const size_t k = (size_t)1 << log_k, n = k << log_inv_rate;
    DevBuf r, m, c;
    int rc = r.ensure(nrows * k * 8);
    if (!rc && mask_coeffs) rc = m.ensure(nrows * mask_coeffs * 8);
    if (!rc) rc = c.ensure(nrows * n * 8);
    if (rc) return rc;
    cudaStream_t s = d->stream;
    host_prefault(rows, nrows * k * 8);
    TG_CUDA(cudaMemcpyAsync(r.ptr, rows, nrows * k * 8, cudaMemcpyHostToDevice, s));
    if (mask_coeffs) host_prefault(masks, nrows * mask_coeffs * 8);
    if (mask_coeffs) TG_CUDA(cudaMemcpyAsync(m.ptr, masks, nrows * mask_coeffs * 8, cudaMemcpyHostToDevice, s));
    {
        std::lock_guard<std::mutex> lock(d->mu);
        rc = lde_encode(d, log_k, log_inv_rate, mask_coeffs, (const uint64_t*)r.ptr, nrows,
                        mask_coeffs ? (const uint64_t*)m.ptr : nullptr, (uint64_t*)c.ptr, s);
    }
    if (rc) return rc;
    TG_CUDA(cudaMemcpyAsync(codewords, c.ptr, nrows * n * 8, cudaMemcpyDeviceToHost, s));
    clear(r, s);
    clear(m, s);
    clear(c, s);
    TG_CUDA(cudaStreamSynchronize(s));
    return TG_OK;
}

static int ntt_dev(tg_device* dev, int kind, uint32_t log_n, uint64_t shift, uint64_t* values, size_t nrows, void* stream) {
    Device* d = reinterpret_cast<Device*>(dev);
    if (!d || (nrows && !values)) return fail(TG_ERR_INVALID, "transform: null argument");
    std::lock_guard<std::mutex> lock(d->mu);
    return ntt_rows(d, kind, log_n, shift, values, nrows, pick_stream(d, stream));
}

static int ntt_host(tg_device* dev, int kind, uint32_t log_n, uint64_t shift, uint64_t* values, size_t nrows) {
    Device* d = reinterpret_cast<Device*>(dev);
    if (!d || (nrows && !values)) return fail(TG_ERR_INVALID, "transform: null argument");
    if (log_n > 22) return fail(TG_ERR_INVALID, "transforms of 2^%u points: the device transforms go up to 2^22", log_n);
    if (nrows == 0) return TG_OK;
    const size_t bytes = (nrows << log_n) * 8;
    DevBuf v;
    int rc = v.ensure(bytes);
    if (rc) return rc;
    cudaStream_t s = d->stream;
    host_prefault(values, bytes);
    TG_CUDA(cudaMemcpyAsync(v.ptr, values, bytes, cudaMemcpyHostToDevice, s));
    {
        std::lock_guard<std::mutex> lock(d->mu);
        rc = ntt_rows(d, kind, log_n, shift, (uint64_t*)v.ptr, nrows, s);
    }
    if (rc) return rc;
    TG_CUDA(cudaMemcpyAsync(values, v.ptr, bytes, cudaMemcpyDeviceToHost, s));
    TG_CUDA(cudaStreamSynchronize(s));
    return TG_OK;
}

int tg_ntt_dev(tg_device* dev, uint32_t log_n, uint64_t* values, size_t nrows, void* stream) {
    return ntt_dev(dev, NTT_FORWARD, log_n, 1, values, nrows, stream);
}
int tg_intt_dev(tg_device* dev, uint32_t log_n, uint64_t* values, size_t nrows, void* stream) {
    return ntt_dev(dev, NTT_INVERSE, log_n, 1, values, nrows, stream);
}
int tg_coset_ntt_dev(tg_device* dev, uint32_t log_n, uint64_t shift, uint64_t* values, size_t nrows, void* stream) {
    return ntt_dev(dev, NTT_COSET_FORWARD, log_n, shift, values, nrows, stream);
}
int tg_coset_intt_dev(tg_device* dev, uint32_t log_n, uint64_t shift, uint64_t* values, size_t nrows, void* stream) {
    return ntt_dev(dev, NTT_COSET_INVERSE, log_n, shift, values, nrows, stream);
}
int tg_ntt(tg_device* dev, uint32_t log_n, uint64_t* values, size_t nrows) {
    return ntt_host(dev, NTT_FORWARD, log_n, 1, values, nrows);
}
int tg_intt(tg_device* dev, uint32_t log_n, uint64_t* values, size_t nrows) {
    return ntt_host(dev, NTT_INVERSE, log_n, 1, values, nrows);
}
int tg_coset_ntt(tg_device* dev, uint32_t log_n, uint64_t shift, uint64_t* values, size_t nrows) {
    return ntt_host(dev, NTT_COSET_FORWARD, log_n, shift, values, nrows);
}
int tg_coset_intt(tg_device* dev, uint32_t log_n, uint64_t shift, uint64_t* values, size_t nrows) {
    return ntt_host(dev, NTT_COSET_INVERSE, log_n, shift, values, nrows);
}

int tg_advice_masks_dev(tg_device* dev, const uint8_t* seed, size_t seed_len, uint64_t first, size_t count,
                        uint64_t* out, void* stream) {
    Device* d = reinterpret_cast<Device*>(dev);
    if (!d || (seed_len && !seed) || (count && !out)) return fail(TG_ERR_INVALID, "tg_advice_masks_dev: null argument");
    std::lock_guard<std::mutex> lock(d->mu);
    return advice_masks(d, seed, seed_len, first, count, out, pick_stream(d, stream));
}

int tg_advice_masks(tg_device* dev, const uint8_t* seed, size_t seed_len, uint64_t first, size_t count, uint64_t* out) {
    Device* d = reinterpret_cast<Device*>(dev);
    if (!d || (seed_len && !seed) || (count && !out)) return fail(TG_ERR_INVALID, "tg_advice_masks: null argument");
    if (count == 0) return TG_OK;
    DevBuf v;
    int rc = v.ensure(count * 8);
    if (rc) return rc;
    cudaStream_t s = d->stream;
    {
        std::lock_guard<std::mutex> lock(d->mu);
        rc = advice_masks(d, seed, seed_len, first, count, (uint64_t*)v.ptr, s);
    }
    if (rc) return rc;
    TG_CUDA(cudaMemcpyAsync(out, v.ptr, count * 8, cudaMemcpyDeviceToHost, s));
    clear(v, s);  // secret-class values are cleared before the memory is released
    TG_CUDA(cudaStreamSynchronize(s));
    return TG_OK;
}

int tg_column_init_dev(tg_device* dev, const uint8_t commitment_id[32], uint64_t ncols, uint8_t* chains, void* stream) {
    Device* d = reinterpret_cast<Device*>(dev);
    if (!d || !commitment_id || (ncols && !chains)) return fail(TG_ERR_INVALID, "tg_column_init_dev: null argument");
    return column_init(d, commitment_id, ncols, chains, pick_stream(d, stream));
}

int tg_column_absorb_dev(tg_device* dev, uint8_t* chains, uint64_t ncols, const uint64_t* rows, size_t count,
                         uint32_t row_block, void* stream) {
    Device* d = reinterpret_cast<Device*>(dev);
    if (!d || (ncols && count && (!chains || !rows))) return fail(TG_ERR_INVALID, "tg_column_absorb_dev: null argument");
    return column_absorb(d, chains, ncols, rows, ncols, count, row_block, pick_stream(d, stream));
}

int tg_merkle_tree_dev(tg_device* dev, const uint8_t* leaves, size_t n, uint8_t* nodes, void* stream) {
    Device* d = reinterpret_cast<Device*>(dev);
    if (!d || !leaves || !nodes) return fail(TG_ERR_INVALID, "tg_merkle_tree_dev: null argument");
    return merkle_tree(d, leaves, n, nodes, pick_stream(d, stream));
}

int tg_column_merge_dev(tg_device* dev, const uint8_t* segment_chains, size_t nsegments, uint64_t n, uint8_t* leaves,
                        void* stream) {
    Device* d = reinterpret_cast<Device*>(dev);
    if (!d || (n && (!leaves || (nsegments && !segment_chains)))) return fail(TG_ERR_INVALID, "tg_column_merge_dev: null argument");
    return column_merge(d, segment_chains, nsegments, n, leaves, pick_stream(d, stream));
}

int tg_commit_unmasked_dev(tg_device* dev, uint32_t log_k, uint32_t log_inv_rate, uint32_t row_block,
                           const uint8_t commitment_id[32], const uint64_t* rows, size_t npolys, uint64_t* codewords,
                           uint8_t* nodes, uint8_t root[32], void* stream) {
    Device* d = reinterpret_cast<Device*>(dev);
    if (!d || !commitment_id || !nodes || (npolys && (!rows || !codewords)))
        return fail(TG_ERR_INVALID, "tg_commit_unmasked_dev: null argument");
    // unmasked_shape's checks (commitment.rs:343-357): rate, length, row block
    if (log_inv_rate == 0) return fail(TG_ERR_INVALID, "log2 inverse rate 0 is a code of rate 1");
    if (log_k + log_inv_rate > 32) return fail(TG_ERR_INVALID, "codeword of 2^%u points exceeds 2^32", log_k + log_inv_rate);
    if (row_block == 0 || row_block > 124) return fail(TG_ERR_INVALID, "row block %u outside 1..124", row_block);
    cudaStream_t s = pick_stream(d, stream);
    const uint64_t n = 1ull << (log_k + log_inv_rate);
    std::lock_guard<std::mutex> lock(d->mu);
    int rc = lde_encode(d, log_k, log_inv_rate, 0, rows, npolys, nullptr, codewords, s);
    if (rc) return rc;
    rc = column_init(d, commitment_id, n, nodes, s);
    if (rc) return rc;
    rc = column_absorb(d, nodes, n, codewords, n, npolys, row_block, s);
    if (rc) return rc;
    rc = merkle_tree(d, nodes, n, nodes, s);
    if (rc) return rc;
    if (root) {
        TG_CUDA(cudaMemcpyAsync(root, nodes + 32 * (2 * n - 2), 32, cudaMemcpyDeviceToHost, s));
        TG_CUDA(cudaStreamSynchronize(s));
    }
    return TG_OK;
}

// Host rows in, root (and optionally the leaves) out. The rows travel in chunks of whole row
// blocks: chunk c is copied on the copy stream while chunk c − 1 is encoded and absorbed into the
// column chains on the device stream, so the transfer hides behind the encoder. The staging
// buffers stay with the device handle for the next call and are zeroed once the call ends.
int tg_commit_unmasked(tg_device* dev, uint32_t log_k, uint32_t log_inv_rate, uint32_t row_block,
                       const uint8_t commitment_id[32], const uint64_t* rows, size_t npolys, uint8_t* leaves,
                       uint8_t root[32]) {
    Device* d = reinterpret_cast<Device*>(dev);
    if (!d || !commitment_id || !root || (npolys && !rows)) return fail(TG_ERR_INVALID, "tg_commit_unmasked: null argument");
    if (log_inv_rate == 0 || log_inv_rate > 4 || log_k > 24) return fail(TG_ERR_INVALID, "unsupported shape 2^%u rate 1/2^%u", log_k, log_inv_rate);
    if (row_block == 0 || row_block > 124) return fail(TG_ERR_INVALID, "row block %u outside 1..124", row_block);
    const size_t k = (size_t)1 << log_k, n = k << log_inv_rate;
    // rows per chunk: the encoder's group, rounded down to whole row blocks (at least one block)
    size_t chunk = std::max<size_t>(1, d->cfg.lde_group_bytes / ((k + n) * 8));
    chunk = std::max<size_t>(row_block, chunk / row_block * row_block);
    chunk = std::min<size_t>(chunk, std::max<size_t>(npolys, 1));
    std::lock_guard<std::mutex> lock(d->mu);
    int rc = d->stage_rows.ensure(2 * chunk * k * 8);
    if (!rc) rc = d->stage_cw.ensure(chunk * n * 8);
    if (!rc) rc = d->stage_nodes.ensure((2 * n - 1) * 32);
    if (rc) return rc;
    if (!d->copy_stream) {
        TG_CUDA(cudaStreamCreateWithFlags(&d->copy_stream, cudaStreamNonBlocking));
        for (int b = 0; b < 2; b++) {
            TG_CUDA(cudaEventCreateWithFlags(&d->staged[b], cudaEventDisableTiming));
            TG_CUDA(cudaEventCreateWithFlags(&d->consumed[b], cudaEventDisableTiming));
        }
        for (cudaEvent_t& e : d->ramp) TG_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    }
    cudaStream_t s = d->stream, cs = d->copy_stream;
    uint64_t* stage = (uint64_t*)d->stage_rows.ptr;
    uint64_t* cw = (uint64_t*)d->stage_cw.ptr;
    uint8_t* nodes = (uint8_t*)d->stage_nodes.ptr;
    // the copy stream starts after everything already queued on the device stream
    TG_CUDA(cudaEventRecord(d->consumed[0], s));
    TG_CUDA(cudaEventRecord(d->consumed[1], s));
    rc = column_init(d, commitment_id, n, nodes, s);
    if (rc) return rc;
    for (size_t r0 = 0, c = 0; r0 < npolys; r0 += chunk, c++) {
        const size_t g = std::min(chunk, npolys - r0);
        const int b = (int)(c & 1);
        uint64_t* half = stage + b * chunk * k;
        TG_CUDA(cudaStreamWaitEvent(cs, d->consumed[b], 0));
        if (c == 0 && g >= 2) {
            // the first chunk's copy has nothing to hide behind: it goes in pieces of g/8, g/8,
            // g/4 and the rest, each encoded as soon as it has landed, so that only the first
            // piece's copy is exposed
            size_t piece[4], np = 0, at = 0, want = std::max<size_t>(1, g / 8);
            while (at < g) {
                const size_t take = np == 3 ? g - at : std::min(want, g - at);
                piece[np++] = take;
                at += take;
                if (np >= 2) want *= 2;
            }
            at = 0;
            for (size_t q = 0; q < np; q++) {
                host_prefault(rows + at * k, piece[q] * k * 8);
                TG_CUDA(cudaMemcpyAsync(half + at * k, rows + at * k, piece[q] * k * 8, cudaMemcpyHostToDevice, cs));
                TG_CUDA(cudaEventRecord(d->ramp[q], cs));
                at += piece[q];
            }
            at = 0;
            for (size_t q = 0; q < np; q++) {
                TG_CUDA(cudaStreamWaitEvent(s, d->ramp[q], 0));
                rc = lde_encode(d, log_k, log_inv_rate, 0, half + at * k, piece[q], nullptr, cw + at * n, s);
                if (rc) return rc;
                at += piece[q];
            }
        } else {
            host_prefault(rows + r0 * k, g * k * 8);
            TG_CUDA(cudaMemcpyAsync(half, rows + r0 * k, g * k * 8, cudaMemcpyHostToDevice, cs));
            TG_CUDA(cudaEventRecord(d->staged[b], cs));
            TG_CUDA(cudaStreamWaitEvent(s, d->staged[b], 0));
            rc = lde_encode(d, log_k, log_inv_rate, 0, half, g, nullptr, cw, s);
            if (rc) return rc;
        }
        TG_CUDA(cudaEventRecord(d->consumed[b], s));
        rc = column_absorb(d, nodes, n, cw, n, g, row_block, s);
        if (rc) return rc;
    }
    rc = merkle_tree(d, nodes, n, nodes, s);
    if (rc) return rc;
    if (leaves) TG_CUDA(cudaMemcpyAsync(leaves, nodes, n * 32, cudaMemcpyDeviceToHost, s));
    TG_CUDA(cudaMemcpyAsync(root, nodes + 32 * (2 * n - 2), 32, cudaMemcpyDeviceToHost, s));
    clear(d->stage_rows, s);
    clear(d->stage_cw, s);
    TG_CUDA(cudaStreamSynchronize(s));
    return TG_OK;
}

int tg_merge_segments(tg_device* dev, const uint8_t* segment_chains, size_t nsegments, uint64_t n, uint8_t* leaves,
                      uint8_t root[32]) {
    Device* d = reinterpret_cast<Device*>(dev);
    if (!d || !root || (nsegments && !segment_chains)) return fail(TG_ERR_INVALID, "tg_merge_segments: null argument");
    if (nsegments == 0) return fail(TG_ERR_INVALID, "merge_segments needs at least one segment");
    if (n < 2 || (n & (n - 1))) return fail(TG_ERR_INVALID, "%llu columns is not a power of two", (unsigned long long)n);
    DevBuf sg, nd;
    int rc = sg.ensure(nsegments * n * 32);
    if (!rc) rc = nd.ensure((2 * n - 1) * 32);
    if (rc) return rc;
    cudaStream_t s = d->stream;
    TG_CUDA(cudaMemcpyAsync(sg.ptr, segment_chains, nsegments * n * 32, cudaMemcpyHostToDevice, s));
    rc = column_merge(d, (const uint8_t*)sg.ptr, nsegments, n, (uint8_t*)nd.ptr, s);
    if (!rc) rc = merkle_tree(d, (const uint8_t*)nd.ptr, n, (uint8_t*)nd.ptr, s);
    if (rc) return rc;
    if (leaves) TG_CUDA(cudaMemcpyAsync(leaves, nd.ptr, n * 32, cudaMemcpyDeviceToHost, s));
    TG_CUDA(cudaMemcpyAsync(root, (uint8_t*)nd.ptr + 32 * (2 * n - 2), 32, cudaMemcpyDeviceToHost, s));
    TG_CUDA(cudaStreamSynchronize(s));
    return TG_OK;
}

// ---- BlockSink --------------------------------------------------------------------------------

int tg_advice_sink_open(tg_device* dev, uint32_t log_k, uint32_t log_inv_rate, uint32_t mask_coeffs, uint32_t row_block,
                        const uint8_t commitment_id[32], tg_sink** out) {
    Device* d = reinterpret_cast<Device*>(dev);
    if (!d || !commitment_id || !out) return fail(TG_ERR_INVALID, "tg_advice_sink_open: null argument");
    *out = nullptr;
    if (log_inv_rate < 1 || log_inv_rate > 4 || log_k > 24) return fail(TG_ERR_INVALID, "unsupported shape 2^%u rate 1/2^%u", log_k, log_inv_rate);
    if ((uint64_t)mask_coeffs > (1ull << log_k)) return fail(TG_ERR_INVALID, "%u mask coefficients exceed k", mask_coeffs);
    if (row_block == 0 || row_block > 124) return fail(TG_ERR_INVALID, "row block %u outside 1..124", row_block);
    tg_sink* sk = new tg_sink();
    sk->d = d;
    sk->lgk = log_k;
    sk->lgr = log_inv_rate;
    sk->P = mask_coeffs;
    sk->B = row_block;
    sk->n = 1ull << (log_k + log_inv_rate);
    const size_t k = (size_t)1 << log_k;
    int rc = sk->chains.ensure(sk->n * 32);
    if (!rc) rc = sk->rows.ensure((size_t)row_block * k * 8);
    if (!rc && mask_coeffs) rc = sk->masks.ensure((size_t)row_block * mask_coeffs * 8);
    if (!rc) rc = sk->cw.ensure((size_t)row_block * sk->n * 8);
    if (!rc) rc = column_init(d, commitment_id, sk->n, (uint8_t*)sk->chains.ptr, d->stream);
    if (rc) {
        delete sk;
        return rc;
    }
    *out = sk;
    return TG_OK;
}

int tg_sink_absorb(tg_sink* sk, const uint64_t* rows, size_t nrows, const uint64_t* masks) {
    if (!sk || (nrows && !rows) || (nrows && sk->P && !masks)) return fail(TG_ERR_INVALID, "tg_sink_absorb: null argument");
    if (sk->finished) return fail(TG_ERR_STATE, "absorb after finish");
    if (sk->closed) return fail(TG_ERR_STATE, "a block followed the short final block");
    if (nrows == 0 || nrows > sk->B) return fail(TG_ERR_INVALID, "a block holds 1 to %u rows, not %zu", sk->B, nrows);
    Device* d = sk->d;
    cudaStream_t s = d->stream;
    const size_t k = (size_t)1 << sk->lgk;
    host_prefault(rows, nrows * k * 8);
    TG_CUDA(cudaMemcpyAsync(sk->rows.ptr, rows, nrows * k * 8, cudaMemcpyHostToDevice, s));
    if (sk->P) host_prefault(masks, nrows * sk->P * 8);
    if (sk->P) TG_CUDA(cudaMemcpyAsync(sk->masks.ptr, masks, nrows * sk->P * 8, cudaMemcpyHostToDevice, s));
    std::lock_guard<std::mutex> lock(d->mu);
    int rc = lde_encode(d, sk->lgk, sk->lgr, sk->P, (const uint64_t*)sk->rows.ptr, nrows,
                        sk->P ? (const uint64_t*)sk->masks.ptr : nullptr, (uint64_t*)sk->cw.ptr, s);
    if (!rc) rc = column_absorb(d, (uint8_t*)sk->chains.ptr, sk->n, (const uint64_t*)sk->cw.ptr, sk->n, nrows, sk->B, s);
    if (rc) return rc;
    // the host buffers may be reused once this returns
    TG_CUDA(cudaStreamSynchronize(s));
    sk->closed = nrows < sk->B;
    return TG_OK;
}

int tg_sink_finish(tg_sink* sk, uint8_t* chains) {
    if (!sk || !chains) return fail(TG_ERR_INVALID, "tg_sink_finish: null argument");
    if (sk->finished) return fail(TG_ERR_STATE, "finish called twice");
    cudaStream_t s = sk->d->stream;
    TG_CUDA(cudaMemcpyAsync(chains, sk->chains.ptr, sk->n * 32, cudaMemcpyDeviceToHost, s));
    TG_CUDA(cudaStreamSynchronize(s));
    sk->finished = true;
    return TG_OK;
}

int tg_sink_close(tg_sink* sk) {
    if (!sk) return TG_OK;
    cudaStream_t s = sk->d->stream;
    clear(sk->rows, s);
    clear(sk->masks, s);
    clear(sk->cw, s);
    cudaStreamSynchronize(s);
    delete sk;
    return TG_OK;
}

// ---- MatrixSink -------------------------------------------------------------------------------

int tg_matrix_open(tg_device* dev, uint32_t log_k, uint32_t log_inv_rate, uint32_t row_block,
                   const uint8_t commitment_id[32], const uint64_t* queries, size_t nqueries, tg_matrix** out) {
    Device* d = reinterpret_cast<Device*>(dev);
    if (!d || !commitment_id || !out || (nqueries && !queries)) return fail(TG_ERR_INVALID, "tg_matrix_open: null argument");
    *out = nullptr;
    if (log_inv_rate < 1 || log_inv_rate > 4 || log_k > 24) return fail(TG_ERR_INVALID, "unsupported shape 2^%u rate 1/2^%u", log_k, log_inv_rate);
    if (row_block == 0 || row_block > 124) return fail(TG_ERR_INVALID, "row block %u outside 1..124", row_block);
    const uint64_t n = 1ull << (log_k + log_inv_rate);
    for (size_t q = 0; q < nqueries; q++) {
        if (queries[q] >= n) return fail(TG_ERR_INVALID, "query %llu outside %llu columns", (unsigned long long)queries[q], (unsigned long long)n);
        if (q && queries[q] <= queries[q - 1]) return fail(TG_ERR_INVALID, "queries must be distinct and increasing");
    }
    tg_matrix* m = new tg_matrix();
    m->d = d;
    m->lgk = log_k;
    m->lgr = log_inv_rate;
    m->B = row_block;
    m->n = n;
    m->nq = nqueries;
    const size_t k = (size_t)1 << log_k;
    int rc = m->chains.ensure(n * 32);
    if (!rc) rc = m->rows.ensure((size_t)row_block * k * 8);
    if (!rc) rc = m->cw.ensure((size_t)row_block * n * 8);
    if (!rc) rc = m->queries.ensure(std::max<size_t>(nqueries, 1) * 8);
    if (!rc) rc = m->answers.ensure(std::max<size_t>(nqueries, 1) * row_block * 8);
    if (!rc && nqueries)
        rc = cudaMemcpyAsync(m->queries.ptr, queries, nqueries * 8, cudaMemcpyHostToDevice, d->stream) == cudaSuccess
                 ? TG_OK
                 : fail(TG_ERR_CUDA, "query upload failed");
    if (!rc) rc = column_init(d, commitment_id, n, (uint8_t*)m->chains.ptr, d->stream);
    if (rc) {
        delete m;
        return rc;
    }
    *out = m;
    return TG_OK;
}

int tg_matrix_absorb(tg_matrix* m, const uint64_t* rows, size_t nrows, uint64_t* answers) {
    if (!m || (nrows && !rows) || (nrows && m->nq && !answers)) return fail(TG_ERR_INVALID, "tg_matrix_absorb: null argument");
    if (m->finished) return fail(TG_ERR_STATE, "absorb after finish");
    if (m->closed) return fail(TG_ERR_STATE, "a block followed the short final block");
    if (nrows == 0 || nrows > m->B) return fail(TG_ERR_INVALID, "a block holds 1 to %u rows, not %zu", m->B, nrows);
    Device* d = m->d;
    cudaStream_t s = d->stream;
    const size_t k = (size_t)1 << m->lgk;
    host_prefault(rows, nrows * k * 8);
    TG_CUDA(cudaMemcpyAsync(m->rows.ptr, rows, nrows * k * 8, cudaMemcpyHostToDevice, s));
    std::lock_guard<std::mutex> lock(d->mu);
    int rc = lde_encode(d, m->lgk, m->lgr, 0, (const uint64_t*)m->rows.ptr, nrows, nullptr, (uint64_t*)m->cw.ptr, s);
    if (!rc) rc = column_absorb(d, (uint8_t*)m->chains.ptr, m->n, (const uint64_t*)m->cw.ptr, m->n, nrows, m->B, s);
    if (rc) return rc;
    if (m->nq) {
        const uint64_t total = m->nq * nrows;
        Launch L(d, s, "gather", 1, total);
        gather_kernel<<<(unsigned)((total + 255) / 256), 256, 0, s>>>((const uint64_t*)m->cw.ptr, m->n,
                                                                      (const uint64_t*)m->queries.ptr, m->nq, nrows,
                                                                      (uint64_t*)m->answers.ptr);
        TG_CUDA(cudaGetLastError());
        TG_CUDA(cudaMemcpyAsync(answers, m->answers.ptr, total * 8, cudaMemcpyDeviceToHost, s));
    }
    TG_CUDA(cudaStreamSynchronize(s));
    m->closed = nrows < m->B;
    return TG_OK;
}

int tg_matrix_finish(tg_matrix* m, uint8_t* chains) {
    if (!m || !chains) return fail(TG_ERR_INVALID, "tg_matrix_finish: null argument");
    if (m->finished) return fail(TG_ERR_STATE, "finish called twice");
    cudaStream_t s = m->d->stream;
    TG_CUDA(cudaMemcpyAsync(chains, m->chains.ptr, m->n * 32, cudaMemcpyDeviceToHost, s));
    TG_CUDA(cudaStreamSynchronize(s));
    m->finished = true;
    return TG_OK;
}

int tg_matrix_close(tg_matrix* m) {
    if (!m) return TG_OK;
    cudaStream_t s = m->d->stream;
    clear(m->rows, s);
    clear(m->cw, s);
    clear(m->answers, s);
    cudaStreamSynchronize(s);
    delete m;
    return TG_OK;
}

// ---- grind ------------------------------------------------------------------------------------

int tg_transcript_grind(tg_device* dev, tg_transcript* t, const char* label, uint32_t bits, uint64_t* nonce) {
    Device* d = reinterpret_cast<Device*>(dev);
    if (!d || !t || !label || !nonce) return fail(TG_ERR_INVALID, "tg_transcript_grind: null argument");
    const size_t ll = strlen(label);
    if (48 + ll > 256) return fail(TG_ERR_INVALID, "grind label longer than 208 bytes");
    if (bits > 64) return fail(TG_ERR_INVALID, "%u bits of work exceed the nonce space", bits);
    PowMsg msg;
    memset(&msg, 0, sizeof msg);
    context_key("pow", msg.key);
    uint8_t bytes[256] = {0};
    memcpy(bytes, t->state, 32);
    for (int i = 0; i < 8; i++) bytes[32 + i] = (uint8_t)((uint64_t)ll >> (8 * i));
    memcpy(bytes + 40, label, ll);
    msg.nonce_off = (uint32_t)(40 + ll);
    msg.len = (uint32_t)(48 + ll);
    msg.bits = bits;
    for (int i = 0; i < 64; i++) msg.words[i] = b3::le32(bytes + 4 * i);
    std::lock_guard<std::mutex> lock(d->mu);
    int rc = d->scratch_misc.ensure(16 * 8);
    if (rc) return rc;
    unsigned long long* found = (unsigned long long*)d->scratch_misc.ptr;
    cudaStream_t s = d->stream;
    const unsigned long long none = ~0ull;
    const uint64_t chunk = 1ull << 24;
    for (uint64_t base = 0;; base += chunk) {
        TG_CUDA(cudaMemcpyAsync(found, &none, 8, cudaMemcpyHostToDevice, s));
        Launch L(d, s, "grind", 1, chunk);
        grind_kernel<<<d->sm_count * 8, 256, 0, s>>>(msg, base, chunk, found);
        TG_CUDA(cudaGetLastError());
        unsigned long long got = none;
        TG_CUDA(cudaMemcpyAsync(&got, found, 8, cudaMemcpyDeviceToHost, s));
        TG_CUDA(cudaStreamSynchronize(s));
        if (got != none) {
            *nonce = got;
            uint8_t v[8];
            for (int i = 0; i < 8; i++) v[i] = (uint8_t)(got >> (8 * i));
            return tg_transcript_absorb(t, label, v, 8);
        }
        if (base > UINT64_MAX - 2 * chunk) return fail(TG_ERR_STATE, "no nonce meets %u bits", bits);
    }
}

}  // extern "C"
