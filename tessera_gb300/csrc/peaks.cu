// SPDX-License-Identifier: Apache-2.0 OR MIT
//
// Integer-pipe peaks of this GPU, measured: the denominators for the kernels that integer
// arithmetic binds (the encoder's butterflies and multiplies, BLAKE3 compressions). Each kernel runs
// independent dependency chains in registers only — no memory traffic but one word per thread at
// the end, so that the compiler keeps the work — over a grid of 8 CTAs of 256 threads per SM.
//
//   imad_wide      mad.wide.u32 (32 × 32 + 64 → 64), the building block of a 64-bit product
//   mulmod         Goldilocks products (tg::lz::mul), the encoder's twiddle multiply
//   butterfly      radix-2 butterflies inside radix-32 transforms with shift twiddles, the
//                  encoder's sub-transforms (80 butterflies per transform)
//   blake3         BLAKE3 compressions (one 64-byte block, seven rounds)
#include <cuda_runtime.h>
#include <stdint.h>

#include "b3.cuh"
#include "gl.cuh"
#include "internal.h"
#include "lde_fast.cuh"

namespace tg {

constexpr int PK_THREADS = 256;

__global__ void __launch_bounds__(PK_THREADS) peak_imad_wide(uint64_t* out, int iters, uint32_t k) {
    uint64_t acc[8];
    for (int c = 0; c < 8; c++) acc[c] = (uint64_t)(threadIdx.x + 1) * (c + 3) + blockIdx.x;
    for (int it = 0; it < iters; it++) {
#pragma unroll
        for (int u = 0; u < 16; u++)
#pragma unroll
            for (int c = 0; c < 8; c++) {
                uint64_t r;
                asm("mad.wide.u32 %0, %1, %2, %3;" : "=l"(r) : "r"((uint32_t)acc[c]), "r"(k), "l"(acc[c]));
                acc[c] = r;
            }
    }
    uint64_t x = 0;
    for (int c = 0; c < 8; c++) x ^= acc[c];
    out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = x;
}

__global__ void __launch_bounds__(PK_THREADS) peak_mulmod(uint64_t* out, int iters, uint64_t k) {
    uint64_t acc[8];
    for (int c = 0; c < 8; c++) acc[c] = (uint64_t)(threadIdx.x + 1) * 0x9E3779B97F4A7C15ull + c + blockIdx.x;
    for (int it = 0; it < iters; it++) {
#pragma unroll
        for (int u = 0; u < 8; u++)
#pragma unroll
            for (int c = 0; c < 8; c++) acc[c] = lz::mul(acc[c], k);
    }
    uint64_t x = 0;
    for (int c = 0; c < 8; c++) x ^= lz::canon(acc[c]);
    out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = x;
}

__global__ void __launch_bounds__(PK_THREADS) peak_butterfly(uint64_t* out, int iters) {
    uint64_t v[32];
    for (int i = 0; i < 32; i++) v[i] = (uint64_t)(threadIdx.x + 1) * 0x9E3779B97F4A7C15ull + i * 0x632BE59BD9B4E019ull + blockIdx.x;
    for (int it = 0; it < iters; it++) fast::dft_dif<32, false, 0>(v);
    uint64_t x = 0;
    for (int i = 0; i < 32; i++) x ^= lz::canon(v[i]) * (i + 1);
    out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = x;
}

__global__ void __launch_bounds__(PK_THREADS) peak_blake3(uint64_t* out, int iters) {
    uint32_t cv[8], m[16];
    for (int i = 0; i < 8; i++) cv[i] = threadIdx.x * 0x9E3779B9u + i + blockIdx.x;
    for (int i = 0; i < 16; i++) m[i] = threadIdx.x * 0x85EBCA6Bu + i;
    for (int it = 0; it < iters; it++) {
        b3::compress_cv(cv, m, (uint64_t)it, 64, b3::CHUNK_START);
        m[it & 15] ^= cv[it & 7];
    }
    uint64_t x = 0;
    for (int i = 0; i < 8; i++) x = x * 0x100000001B3ull ^ cv[i];
    out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = x;
}

}  // namespace tg

using namespace tg;

extern "C" int tg_measure_int_peaks(tg_device* dev, tg_int_peaks* out) {
    Device* d = reinterpret_cast<Device*>(dev);
    if (!d || !out) return fail(TG_ERR_INVALID, "tg_measure_int_peaks: null argument");
    std::lock_guard<std::mutex> lock(d->mu);
    cudaStream_t s = d->stream;
    const int blocks = d->sm_count * 8;
    const size_t threads = (size_t)blocks * PK_THREADS;
    int rc = d->scratch_misc.ensure(threads * 8);
    if (rc) return rc;
    uint64_t* buf = (uint64_t*)d->scratch_misc.ptr;
    struct Events {
        cudaEvent_t e[2] = {nullptr, nullptr};
        ~Events() {
            for (auto x : e)
                if (x) cudaEventDestroy(x);
        }
    } ev;
    TG_CUDA(cudaEventCreate(&ev.e[0]));
    TG_CUDA(cudaEventCreate(&ev.e[1]));
    cudaEvent_t e0 = ev.e[0], e1 = ev.e[1];
    // Runs f once to warm up, then times it; returns the seconds of the timed run.
    auto timed = [&](auto&& f, double* sec) -> int {
        f();
        TG_CUDA(cudaGetLastError());
        TG_CUDA(cudaEventRecord(e0, s));
        f();
        TG_CUDA(cudaEventRecord(e1, s));
        TG_CUDA(cudaEventSynchronize(e1));
        float ms = 0;
        TG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        *sec = ms / 1e3;
        return TG_OK;
    };
    double t = 0;
    const int it_w = 2048, it_m = 512, it_b = 512, it_h = 2048;
    rc = timed([&] { peak_imad_wide<<<blocks, PK_THREADS, 0, s>>>(buf, it_w, 0x9E3779B9u); }, &t);
    if (rc) return rc;
    out->imad_wide_per_s = (double)threads * it_w * 16 * 8 / t;
    rc = timed([&] { peak_mulmod<<<blocks, PK_THREADS, 0, s>>>(buf, it_m, 0x123456789ABCDEFull); }, &t);
    if (rc) return rc;
    out->mulmod_per_s = (double)threads * it_m * 8 * 8 / t;
    rc = timed([&] { peak_butterfly<<<blocks, PK_THREADS, 0, s>>>(buf, it_b); }, &t);
    if (rc) return rc;
    out->butterflies_per_s = (double)threads * it_b * 80 / t;
    rc = timed([&] { peak_blake3<<<blocks, PK_THREADS, 0, s>>>(buf, it_h); }, &t);
    if (rc) return rc;
    out->blake3_compressions_per_s = (double)threads * it_h / t;
    d->launches += 8;
    return TG_OK;
}

// ---- a self-check of the lazy arithmetic on any 64-bit words ----------------------------------

namespace tg {

// Word i's outputs (canonical): see tg_check_lazy_arith in the header for the list.
__global__ void check_lazy_kernel(const uint64_t* w, size_t n, uint64_t* out) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint64_t a = w[i], b = w[(i + 1) % n], c = w[(i + 2) % n], d = w[(i + 3) % n];
    uint64_t* o = out + (size_t)TG_LAZY_CHECK_OUTS * i;
    o[0] = lz::canon(lz::add(a, b));
    o[1] = lz::canon(lz::sub(a, b));
    o[2] = lz::canon(lz::mul(a, b));
    o[3] = lz::canon(lz::mul7(a));
    o[4] = lz::canon(lz::mulp2<5>(a));
    o[5] = lz::canon(lz::mulp2<40>(a));
    o[6] = lz::canon(lz::mulp2<70>(a));
    lz::Acc s = lz::acc_mul(a, b);
    lz::mad(s, c, d);
    o[7] = lz::canon(lz::reduce(s));
    lz::Acc t = lz::acc_of(a);
    lz::mad(t, b, c);
    lz::mad(t, d, a);
    o[8] = lz::canon(lz::reduce(t));
    const fp2 x = {a, b}, y = {c, d}, u = {b, a}, v = {b, d}, z = {a, c};
    const fp2 m = l2_canon(l2_muls(x, y)), f = l2_canon(l2_fma(x, y, lz::mul7(y.c1), u)), g = l2_canon(l2_dot(x, y, v, z));
    o[9] = m.c0, o[10] = m.c1, o[11] = f.c0, o[12] = f.c1, o[13] = g.c0, o[14] = g.c1;
    lz::Acc big = lz::acc_zero();
    for (size_t k = 0; k < 64; k++) lz::mad(big, w[(i + k) % n], w[(i + 2 * k + 1) % n]);
    o[15] = lz::canon(lz::reduce(big));
}

}  // namespace tg

extern "C" int tg_check_lazy_arith(tg_device* dev, const uint64_t* words, size_t n, uint64_t* out) {
    using namespace tg;
    Device* d = reinterpret_cast<Device*>(dev);
    if (!d || !words || !out) return fail(TG_ERR_INVALID, "tg_check_lazy_arith: null argument");
    if (n < 4) return fail(TG_ERR_INVALID, "tg_check_lazy_arith: %zu words, at least 4 needed", n);
    DevBuf in, res;
    int rc = in.ensure(n * 8);
    if (!rc) rc = res.ensure(n * 8 * TG_LAZY_CHECK_OUTS);
    if (rc) return rc;
    cudaStream_t s = d->stream;
    TG_CUDA(cudaMemcpyAsync(in.ptr, words, n * 8, cudaMemcpyHostToDevice, s));
    check_lazy_kernel<<<(unsigned)((n + 127) / 128), 128, 0, s>>>((const uint64_t*)in.ptr, n, (uint64_t*)res.ptr);
    TG_CUDA(cudaGetLastError());
    d->launches += 1;
    TG_CUDA(cudaMemcpyAsync(out, res.ptr, n * 8 * TG_LAZY_CHECK_OUTS, cudaMemcpyDeviceToHost, s));
    TG_CUDA(cudaStreamSynchronize(s));
    return TG_OK;
}

