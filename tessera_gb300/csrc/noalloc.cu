// SPDX-License-Identifier: Apache-2.0 OR MIT
//
// An allocation-free form of the Reed–Solomon encoder, for callers that cannot call cudaMalloc:
// a prover embedded in a host program whose device memory belongs to another allocator (a Rust
// runtime's own pool, a serving loop that reserved all of HBM up front), or a hot loop that must
// not allocate because cudaMalloc and cudaFree synchronize the whole device. Such a caller passes
// its rows, masks and codeword buffers; the encoder's twiddle tables and scratch live in one
// fixed array in this file's device memory instead of being allocated.
//
// The array is NOALLOC_WORDS 64-bit words (32 MiB), and every GPU that loads this library holds
// it until the process exits. A call needs its tables (k + n words) plus, for k >= 2^12, one row
// of scratch (k + n words), so 2·(k + n) <= 2^22 words: k <= 2^19 at rate 1/2, k <= 2^18 at rate
// 1/4. Larger shapes are refused. Every call shares the array, which keeps the last call's tables
// and scratch; nothing in it has to start at zero (each call writes every word it reads). Calls
// that overlap on the GPU (on different streams, or from several threads) race on the array:
// order them on one stream.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <mutex>

#include "internal.h"

namespace tg {
namespace {

constexpr size_t NOALLOC_WORDS = size_t(1) << 22;  // 32 MiB
constexpr int MAX_DEVICES = 64;

static __device__ __align__(256) uint64_t g_noalloc_scratch[NOALLOC_WORDS];

struct PerDevice {
    uint64_t* base = nullptr;  // device address of g_noalloc_scratch on this device
    uint32_t lgn = 0, lgk = 0;  // the shape whose tables the array holds
    bool tables = false;
};

std::mutex g_mu;
PerDevice g_dev[MAX_DEVICES];

// Set-up, once per device with that device current: the array's device address.
int device_base(int ordinal, PerDevice** out) {
    if (ordinal < 0 || ordinal >= MAX_DEVICES) return fail(TG_ERR_INVALID, "device ordinal %d out of range", ordinal);
    PerDevice& pd = g_dev[ordinal];
    if (!pd.base) {
        int cur = -1;
        TG_CUDA(cudaGetDevice(&cur));
        if (cur != ordinal) TG_CUDA(cudaSetDevice(ordinal));
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (cur != ordinal) cudaSetDevice(cur);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
        pd.base = static_cast<uint64_t*>(p);
    }
    *out = &pd;
    return TG_OK;
}

}  // namespace
}  // namespace tg

using namespace tg;

// The encoder of tg_encode_rows_dev with no device allocation (no counterpart in the
// reference). The first call on a device looks up the fixed array's address; make that first
// call before any stream capture.
extern "C" int tg_encode_rows_noalloc_dev(tg_device* dev, uint32_t log_k, uint32_t log_inv_rate, uint32_t mask_coeffs,
                                          const uint64_t* rows, size_t nrows, const uint64_t* masks,
                                          uint64_t* codewords, void* stream) {
    Device* d = reinterpret_cast<Device*>(dev);
    if (!d || (nrows && (!rows || !codewords))) return fail(TG_ERR_INVALID, "tg_encode_rows_noalloc_dev: null argument");
    if (log_inv_rate < 1 || log_inv_rate > 4) return fail(TG_ERR_INVALID, "log2 inverse rate %u outside 1..4", log_inv_rate);
    if (log_k > 24) return fail(TG_ERR_INVALID, "log2 k %u above 24", log_k);
    if ((uint64_t)mask_coeffs > (1ull << log_k)) return fail(TG_ERR_INVALID, "%u mask coefficients exceed k", mask_coeffs);
    if (mask_coeffs > 0 && !masks) return fail(TG_ERR_INVALID, "mask coefficients requested without masks");
    const size_t k = (size_t)1 << log_k, n = k << log_inv_rate;
    const size_t tables = k + n;
    const size_t per_row = log_k >= 12 ? k + n : 0;
    if (tables + per_row > NOALLOC_WORDS)
        return fail(TG_ERR_INVALID,
                    "rows of 2^%u at rate 1/2^%u need %zu words of fixed scratch; the allocation-free encoder holds %zu "
                    "(2 (k + n) <= 2^22)",
                    log_k, log_inv_rate, tables + per_row, NOALLOC_WORDS);
    // The fixed array's address is this device's, so the kernels must launch on this device.
    int cur = -1;
    TG_CUDA(cudaGetDevice(&cur));
    if (cur != d->ordinal)
        return fail(TG_ERR_INVALID, "tg_encode_rows_noalloc_dev: device %d is current, the handle is device %d", cur,
                    d->ordinal);
    std::lock_guard<std::mutex> lock(g_mu);
    PerDevice* pd = nullptr;
    int rc = device_base(d->ordinal, &pd);
    if (rc) return rc;
    const uint32_t lgn = log_k + log_inv_rate;
    cudaStream_t s = pick_stream(d, stream);
    // A call recorded into a CUDA graph runs its kernels only when the graph is launched, maybe
    // after calls of other shapes have rewritten the array: such a call always writes its own
    // tables, and leaves the array's tables marked unknown for the next direct call.
    cudaStreamCaptureStatus capture = cudaStreamCaptureStatusNone;
    TG_CUDA(cudaStreamIsCapturing(s, &capture));
    const bool captured = capture != cudaStreamCaptureStatusNone;
    const bool build = captured || !(pd->tables && pd->lgn == lgn && pd->lgk == log_k);
    uint64_t* pw = pd->base;
    uint64_t* pow7k = pw + n;
    uint64_t* scratch = pow7k + k;
    const size_t group = per_row ? std::min<size_t>((NOALLOC_WORDS - tables) / per_row, std::max<size_t>(nrows, 1)) : 0;
    uint64_t* y = scratch;
    uint64_t* z = scratch + group * k;
    std::lock_guard<std::mutex> dl(d->mu);
    rc = lde_encode_into(d, log_k, log_inv_rate, mask_coeffs, rows, nrows, masks, codewords, s, pw, pow7k, build, y, z,
                         std::max<size_t>(group, 1));
    if (rc || captured) {
        pd->tables = false;
        return rc;
    }
    pd->lgn = lgn;
    pd->lgk = log_k;
    pd->tables = true;
    return TG_OK;
}
