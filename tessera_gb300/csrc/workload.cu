// SPDX-License-Identifier: Apache-2.0 OR MIT
//
// Synthetic inputs generated where they are used: uniform Goldilocks words from SplitMix64
// (state += 0x9E3779B97F4A7C15, then the mix; outputs at or above p reduced once, as the
// reference benchmark's `from_u64_reduced` does, crates/tessera-bench/benches/primitives.rs:52-69).
// Word i (0-based) is the (i + 1)-th output of the stream started at `seed`, so the device fill
// equals the host generator word for word. Large benchmark inputs (tens of GB) are filled at HBM
// speed instead of being generated on the host and copied.
#include <cuda_runtime.h>
#include <stdint.h>

#include "gl.cuh"
#include "internal.h"

namespace tg {

__global__ void fill_splitmix_kernel(uint64_t* out, uint64_t n, uint64_t seed) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        uint64_t z = seed + (i + 1) * 0x9E3779B97F4A7C15ull;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        out[i] = z >= P ? z - P : z;
    }
}

}  // namespace tg

using namespace tg;

extern "C" int tg_fill_splitmix(tg_device* dev, uint64_t* out, size_t n, uint64_t seed, void* stream) {
    Device* d = reinterpret_cast<Device*>(dev);
    if (!d || (n && !out)) return fail(TG_ERR_INVALID, "tg_fill_splitmix: null argument");
    if (n == 0) return TG_OK;
    cudaStream_t s = pick_stream(d, stream);
    const uint64_t blocks = std::min<uint64_t>((n + 255) / 256, (uint64_t)d->sm_count * 16);
    Launch L(d, s, "splitmix", 1, n);
    fill_splitmix_kernel<<<(unsigned)blocks, 256, 0, s>>>(out, n, seed);
    TG_CUDA(cudaGetLastError());
    return TG_OK;
}

// The reference's fill_counter (crates/tessera-gpu/kernels/commit.cu:27-33): out[i] is
// counter(base + i), the SplitMix64 output for state (base + i + 1)·0x9E3779B97F4A7C15 reduced
// once below p, which is the stream above started at base·0x9E3779B97F4A7C15.
extern "C" int tg_fill_counter(tg_device* dev, uint64_t* out, size_t n, uint64_t base, void* stream) {
    return tg_fill_splitmix(dev, out, n, base * 0x9E3779B97F4A7C15ull, stream);
}
