// SPDX-License-Identifier: Apache-2.0 OR MIT
//
// BASELINE INFRASTRUCTURE ONLY: runs the reference's own CUDA kernels on this GPU, for a same-box
// comparison with the library's. The kernels are the reference's crates/tessera-gpu/kernels/
// commit.cu, compiled from its sources by oracle/Makefile (target `ref`) into
// oracle/_ref/commit.fatbin; this file is the host side the reference writes in Rust
// (crates/tessera-gpu/src/commit.rs, driven by crates/tessera-bench/examples/gpu_unit_costs.rs
// `cc`), restated in C++ over the CUDA driver API: the same tables, passes, launch geometry and
// argument lists, and the same measurement. The product library never links or loads this.
//
//   refgpu_cc: the committed-element cost c_c. Blocks of 32 rows of k = 2^log_k values with P
//   mask coefficients are generated on the device (fill_counter; rows from counter 32·k·block,
//   masks from 2^62 + 32·P·block), encoded at rate 1/2 (ntt_pass DIF passes, encode_low, ntt_pass
//   DIT passes; commit.rs:277-388) and absorbed into the 2k column chains (column_step,
//   commit.rs:458-492). c_c = (generate + encode + hash − generate) / elements, medians of the
//   timed runs after the warm-ups (gpu_unit_costs.rs:93-170). Before timing, block 0's chains
//   are checked against the CPU oracle's encoding and chains, as the reference's benchmark
//   checks them against its CPU crates.
#include <cuda.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <string>
#include <vector>

#include "tessera_oracle.h"

namespace {

constexpr uint64_t P = 0xFFFFFFFF00000001ull;
constexpr uint32_t TILE_LOG = 13, RUN_LOG = 2, PASS_TILE_LOG = 12, LOW_LOG = TILE_LOG - 1;
constexpr uint32_t BLOCK = 32;

uint32_t shared_bytes(uint32_t elements) { return 8 * (elements + elements / 16); }

uint64_t mulm(uint64_t a, uint64_t b) { return (uint64_t)(((unsigned __int128)a * b) % P); }
uint64_t powm(uint64_t b, uint64_t e) {
    uint64_t r = 1;
    while (e) {
        if (e & 1) r = mulm(r, b);
        b = mulm(b, b);
        e >>= 1;
    }
    return r;
}
std::vector<uint64_t> powers(uint64_t w, size_t len) {
    std::vector<uint64_t> out(len);
    uint64_t x = 1;
    for (size_t i = 0; i < len; i++) {
        out[i] = x;
        x = mulm(x, w);
    }
    return out;
}

struct Pass {
    uint32_t lo_bit, c, log_g;
};

// The strided passes over index bits [from, to), each at most a tile of 2^PASS_TILE_LOG
// elements, in increasing bit order (commit.rs:147-158).
std::vector<Pass> passes(uint32_t from, uint32_t to) {
    std::vector<Pass> out;
    for (uint32_t lo = from; lo < to;) {
        const uint32_t log_g = std::min(RUN_LOG, lo);
        const uint32_t c = std::min(to - lo, PASS_TILE_LOG - log_g);
        out.push_back({lo, c, log_g});
        lo += c;
    }
    return out;
}

std::string g_err;

bool ok(CUresult r, const char* what) {
    if (r == CUDA_SUCCESS) return true;
    const char* s = nullptr;
    cuGetErrorString(r, &s);
    g_err = std::string(what) + ": " + (s ? s : "unknown CUDA error");
    return false;
}
#define CK(call)                              \
    do {                                      \
        if (!ok((call), #call)) return false; \
    } while (0)

struct Bench {
    CUcontext ctx = nullptr;
    CUmodule mod = nullptr;
    CUstream s = nullptr;
    CUfunction fill_counter, ntt_pass, encode_low, column_init, column_step;
    uint32_t log_k = 0, P_ = 0;
    uint64_t k = 0, n = 0;
    CUdeviceptr inverse = 0, forward = 0, scale = 0, mask_pow = 0, rows = 0, masks = 0, cw = 0, chains = 0,
                params = 0;
    uint64_t shift_pow_k = 0;
    CUdevice dev = 0;

    bool open(const char* fatbin, uint32_t lgk, uint32_t mask_coeffs) {
        log_k = lgk;
        P_ = mask_coeffs;
        k = 1ull << lgk;
        n = 2 * k;
        CK(cuInit(0));
        CK(cuDeviceGet(&dev, 0));
        CK(cuDevicePrimaryCtxRetain(&ctx, dev));
        CK(cuCtxSetCurrent(ctx));
        CK(cuModuleLoad(&mod, fatbin));
        CK(cuModuleGetFunction(&fill_counter, mod, "fill_counter"));
        CK(cuModuleGetFunction(&ntt_pass, mod, "ntt_pass"));
        CK(cuModuleGetFunction(&encode_low, mod, "encode_low"));
        CK(cuModuleGetFunction(&column_init, mod, "column_init"));
        CK(cuModuleGetFunction(&column_step, mod, "column_step"));
        for (CUfunction f : {ntt_pass, encode_low})
            CK(cuFuncSetAttribute(f, CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, shared_bytes(1u << TILE_LOG)));
        CK(cuStreamCreate(&s, CU_STREAM_NON_BLOCKING));
        // The rate-1/2 encoder's tables on the coset 7·L (commit.rs:200-249).
        const uint64_t omega = powm(7, (P - 1) / n), omega_inv = powm(omega, P - 2), k_inv = powm(k % P, P - 2);
        std::vector<uint64_t> shift_powers = powers(7, k), sc(k);
        for (uint64_t t = 0; t < k; t++) {
            uint64_t r = 0;
            for (uint32_t b = 0; b < lgk; b++) r |= ((t >> b) & 1) << (lgk - 1 - b);
            sc[t] = mulm(shift_powers[r], k_inv);
        }
        std::vector<uint64_t> mp = P_ ? std::vector<uint64_t>(shift_powers.begin(), shift_powers.begin() + P_)
                                     : std::vector<uint64_t>{0};
        shift_pow_k = powm(7, k);
        if (!upload(&inverse, powers(omega_inv, k)) || !upload(&forward, powers(omega, k)) || !upload(&scale, sc) ||
            !upload(&mask_pow, mp))
            return false;
        CK(cuMemAlloc(&rows, BLOCK * k * 8));
        CK(cuMemAlloc(&masks, std::max<uint64_t>(1, (uint64_t)BLOCK * P_) * 8));
        CK(cuMemAlloc(&cw, BLOCK * n * 8));
        CK(cuMemAlloc(&chains, n * 32));
        // column_init / column_step parameters: the two context keys and the commitment id
        // (commit.rs:428-436), id [0x5A; 32] as the reference's benchmark uses.
        uint8_t words[96];
        or_context_key("column-init", words);
        or_context_key("column-step", words + 32);
        memset(words + 64, 0x5A, 32);
        CK(cuMemAlloc(&params, 96));
        CK(cuMemcpyHtoD(params, words, 96));
        return true;
    }

    bool upload(CUdeviceptr* p, const std::vector<uint64_t>& v) {
        CK(cuMemAlloc(p, v.size() * 8));
        CK(cuMemcpyHtoD(*p, v.data(), v.size() * 8));
        return true;
    }

    bool fill(CUdeviceptr out, uint64_t len, uint64_t base) {
        // cudarc's LaunchConfig::for_num_elems: 1,024 threads a block
        void* args[] = {&out, &len, &base};
        const uint32_t blocks = (uint32_t)((len + 1023) / 1024);
        CK(cuLaunchKernel(fill_counter, blocks, 1, 1, 1024, 1, 1, 0, s, args, nullptr));
        return true;
    }

    bool generate(uint64_t block) {
        if (!fill(rows, BLOCK * k, block * BLOCK * k)) return false;
        return !P_ || fill(masks, BLOCK * P_, (1ull << 62) + block * BLOCK * P_);
    }

    bool pass(CUdeviceptr data, uint64_t row_stride, uint32_t log_n, const Pass& p, CUdeviceptr table,
              uint32_t log_table, uint32_t dit) {
        const uint32_t size = 1u << (p.c + p.log_g);
        void* args[] = {&data, &row_stride, &log_n, (void*)&p.lo_bit, (void*)&p.c, (void*)&p.log_g, &table,
                        &log_table, &dit};
        const uint32_t threads = std::min<uint32_t>(128, std::max<uint32_t>(1, size / 32));
        CK(cuLaunchKernel(ntt_pass, 1u << (log_n - p.c - p.log_g), BLOCK, 1, threads, 1, 1, shared_bytes(size), s,
                          args, nullptr));
        return true;
    }

    // Device::encode_rows (commit.rs:277-349): rows are scratch.
    bool encode() {
        const uint32_t cx = std::min(log_k, LOW_LOG), log_n = log_k + 1;
        std::vector<Pass> high = passes(cx, log_k);
        for (auto it = high.rbegin(); it != high.rend(); ++it)
            if (!pass(rows, k, log_k, *it, inverse, log_n, 0)) return false;
        const uint32_t tile = 1u << cx;
        uint32_t lgk = log_k, cxa = cx, mc = P_;
        uint64_t spk = shift_pow_k;
        void* args[] = {&rows, &cw, &lgk, &cxa, &inverse, &forward, &scale, &masks, &mask_pow, &spk, &mc};
        CK(cuLaunchKernel(encode_low, 1u << (log_k - cx), BLOCK, 1, std::max<uint32_t>(1, tile >> 4), 1, 1,
                          shared_bytes(2 * tile), s, args, nullptr));
        for (const Pass& p : passes(cx + 1, log_n))
            if (!pass(cw, n, log_n, p, forward, log_n, 1)) return false;
        return true;
    }

    bool init_chains() {
        uint64_t nn = n;
        void* args[] = {&chains, &nn, &params};
        CK(cuLaunchKernel(column_init, (uint32_t)((n + 1023) / 1024), 1, 1, 1024, 1, 1, 0, s, args, nullptr));
        return true;
    }

    bool absorb() {
        uint64_t nn = n;
        uint32_t count = BLOCK;
        void* args[] = {&chains, &cw, &nn, &count, &params};
        CK(cuLaunchKernel(column_step, (uint32_t)((n + 127) / 128), 1, 1, 128, 1, 1, 0, s, args, nullptr));
        return true;
    }

    // One timed run of `blocks` blocks (mode 0: generate; 1: generate + encode; 2: + hash), seconds.
    bool run(uint64_t blocks, int mode, double* seconds) {
        CUevent e0, e1;
        CK(cuEventCreate(&e0, CU_EVENT_DEFAULT));
        CK(cuEventCreate(&e1, CU_EVENT_DEFAULT));
        CK(cuEventRecord(e0, s));
        if (mode == 2 && !init_chains()) return false;
        for (uint64_t b = 0; b < blocks; b++) {
            if (!generate(b)) return false;
            if (mode >= 1 && !encode()) return false;
            if (mode == 2 && !absorb()) return false;
        }
        CK(cuEventRecord(e1, s));
        CK(cuEventSynchronize(e1));
        float ms = 0;
        CK(cuEventElapsedTime(&ms, e0, e1));
        cuEventDestroy(e0);
        cuEventDestroy(e1);
        *seconds = ms / 1e3;
        return true;
    }

    // Block 0 through the reference's kernels against the CPU oracle: every column chain.
    bool check(int threads, uint8_t* chains_out) {
        if (!init_chains() || !generate(0) || !encode() || !absorb()) return false;
        std::vector<uint64_t> hr(BLOCK * k), hm(std::max<uint64_t>(1, BLOCK * P_)), code(BLOCK * n);
        std::vector<uint8_t> got(n * 32), want(n * 32);
        CK(cuStreamSynchronize(s));
        // generate() again: encode_rows leaves intermediate values in `rows`
        if (!generate(0)) return false;
        CK(cuStreamSynchronize(s));
        CK(cuMemcpyDtoH(hr.data(), rows, hr.size() * 8));
        CK(cuMemcpyDtoH(hm.data(), masks, hm.size() * 8));
        CK(cuMemcpyDtoH(got.data(), chains, got.size()));
        uint8_t id[32];
        memset(id, 0x5A, 32);
        if (or_encode_rows(log_k, 1, P_, hr.data(), BLOCK, P_ ? hm.data() : nullptr, code.data(), threads) != 0) {
            g_err = "the oracle refused the check block";
            return false;
        }
        or_column_init(id, n, want.data(), threads);
        or_column_absorb(want.data(), n, code.data(), BLOCK, threads);
        if (chains_out) memcpy(chains_out, got.data(), got.size());
        if (got != want) {
            g_err = "the reference kernels' column chains differ from the CPU oracle's";
            return false;
        }
        return true;
    }

    void close() {
        for (CUdeviceptr p : {inverse, forward, scale, mask_pow, rows, masks, cw, chains, params})
            if (p) cuMemFree(p);
        if (s) cuStreamDestroy(s);
        if (mod) cuModuleUnload(mod);
        if (ctx) cuDevicePrimaryCtxRelease(dev);
    }
};

double median(std::vector<double> v) {
    std::sort(v.begin(), v.end());
    return v.size() % 2 ? v[v.size() / 2] : 0.5 * (v[v.size() / 2 - 1] + v[v.size() / 2]);
}

}  // namespace

extern "C" {

const char* refgpu_last_error(void) { return g_err.c_str(); }

// out[0..2]: medians in seconds of generate+encode+hash, generate, generate+encode over `rows`
// rows. With check_threads > 0, block 0's chains are first checked against the CPU oracle (on
// that many threads) and copied to chains_out (2k x 32 bytes) when it is not NULL.
// Returns 0, or −1 with refgpu_last_error().
int refgpu_cc(const char* fatbin, uint32_t log_k, uint32_t rows, uint32_t mask_coeffs, int warmup, int runs,
              int check_threads, double* out, uint8_t* chains_out) {
    Bench b;
    if (rows == 0 || rows % BLOCK || log_k < 1 || log_k > 26 || mask_coeffs > (1u << log_k) || runs < 1) {
        g_err = "rows must be a positive multiple of 32, 1 <= log_k <= 26, P <= k";
        return -1;
    }
    bool good = b.open(fatbin, log_k, mask_coeffs);
    if (good && check_threads > 0) good = b.check(check_threads, chains_out);
    const uint64_t blocks = rows / BLOCK;
    std::vector<double> full, gen, enc;
    for (int i = 0; good && i < warmup + runs; i++) {
        double t;
        good = b.run(blocks, 2, &t);
        if (good && i >= warmup) full.push_back(t);
    }
    for (int i = 0; good && i < runs; i++) {
        double t;
        good = b.run(blocks, 0, &t);
        if (good) gen.push_back(t);
    }
    for (int i = 0; good && i < runs; i++) {
        double t;
        good = b.run(blocks, 1, &t);
        if (good) enc.push_back(t);
    }
    b.close();
    if (!good) return -1;
    out[0] = median(full);
    out[1] = median(gen);
    out[2] = median(enc);
    return 0;
}

}  // extern "C"
