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
//
//   refgpu_pi: the product-forest leaf cost c_π with the reference's crates/tessera-gpu/kernels/
//   trees.cu (oracle/_ref/trees.fatbin): a forest of 2^s trees of 2^h prime-field leaves from the
//   counter generator at 2^61, proved level by level as Device::prove_forest_in does
//   (crates/tessera-gpu/src/trees.rs:176-318): the levels built bottom up (tree_level), then per
//   level the root challenges, γ, each round's split eq tables (eq_table), fused bind-and-sums
//   (level_sums_base, bind_sums_base, bind_sums_ext) and their block reduction (reduce_sums) read
//   back, the round message p(0), p(2), p(3) formed on the host, the last binding (bind_base,
//   bind_ext), the evaluations and ρ; the transcript is the CPU oracle's (the reference runs its
//   own on the host too). Timed on the host clock per proof with the workspace reused, as
//   gpu_unit_costs.rs `pi` (:175-205) times it; the final transcript state is returned so that the
//   caller can check that the library proves the same forest to the same bytes.
//
//   refgpu_fraction: one LogUp fraction tree of c_ℓ, as Device::prove_fraction_tree_in does
//   (crates/tessera-gpu/src/fraction.rs:208-634): leaves generated in the kernels from the counter
//   generator (LEAF_ARGS: key, value and multiplicity seeds, α, β, unit), levels h − 1 .. 1 built
//   (frac_level_leaves, frac_level), then per level γ, λ, the rounds (frac_sums_*, frac_bind_sums_*,
//   reduce_sums), the last binding (frac_last_*) or the one-entry level (frac_first_*), the four
//   evaluations and ρ. c_ℓ is the lookup tree's proof plus the table tree's, per lookup
//   (gpu_unit_costs.rs `l`, :212-296).
#include <cuda.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <chrono>
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

// ---- c_π ----------------------------------------------------------------------------------

struct F2 {
    uint64_t a, b;
};
uint64_t addm(uint64_t x, uint64_t y) { return (uint64_t)(((unsigned __int128)x + y) % P); }
uint64_t subm(uint64_t x, uint64_t y) { return x >= y ? x - y : (uint64_t)((unsigned __int128)x + P - y); }
F2 f2add(F2 x, F2 y) { return {addm(x.a, y.a), addm(x.b, y.b)}; }
F2 f2sub(F2 x, F2 y) { return {subm(x.a, y.a), subm(x.b, y.b)}; }
F2 f2mul(F2 x, F2 y) {
    return {addm(mulm(x.a, y.a), mulm(7, mulm(x.b, y.b))), addm(mulm(x.a, y.b), mulm(x.b, y.a))};
}
const F2 F2_ONE = {1, 0};

constexpr uint32_t SUM_THREADS = 256;  // trees.rs SUM_THREADS
constexpr uint64_t SUM_BLOCKS = 2048;  // trees.rs SUM_BLOCKS

struct Forest {
    CUcontext ctx = nullptr;
    CUmodule mod = nullptr, cmod = nullptr;
    CUstream s = nullptr;
    CUdevice dev = 0;
    CUfunction fill_counter, tree_level, level_sums_base, bind_sums_base, bind_sums_ext, eq_table, reduce_sums,
        bind_base, bind_ext;
    uint32_t height = 0, vars = 0;
    uint64_t leaves_n = 0;
    CUdeviceptr leaves = 0, cur0 = 0, cur1 = 0, sp0 = 0, sp1 = 0, partials = 0, sums = 0, eq_lo = 0, eq_hi = 0,
                points = 0;
    std::vector<CUdeviceptr> levels;  // level t at index t − 1, 1 <= t < h

    bool open(const char* trees_fatbin, const char* commit_fatbin, uint32_t s_log, uint32_t h) {
        height = h;
        vars = s_log + h;
        leaves_n = 1ull << vars;
        CK(cuInit(0));
        CK(cuDeviceGet(&dev, 0));
        CK(cuDevicePrimaryCtxRetain(&ctx, dev));
        CK(cuCtxSetCurrent(ctx));
        CK(cuModuleLoad(&mod, trees_fatbin));
        CK(cuModuleLoad(&cmod, commit_fatbin));
        CK(cuModuleGetFunction(&fill_counter, cmod, "fill_counter"));
        CK(cuModuleGetFunction(&tree_level, mod, "tree_level"));
        CK(cuModuleGetFunction(&level_sums_base, mod, "level_sums_base"));
        CK(cuModuleGetFunction(&bind_sums_base, mod, "bind_sums_base"));
        CK(cuModuleGetFunction(&bind_sums_ext, mod, "bind_sums_ext"));
        CK(cuModuleGetFunction(&eq_table, mod, "eq_table"));
        CK(cuModuleGetFunction(&reduce_sums, mod, "reduce_sums"));
        CK(cuModuleGetFunction(&bind_base, mod, "bind_base"));
        CK(cuModuleGetFunction(&bind_ext, mod, "bind_ext"));
        CK(cuStreamCreate(&s, CU_STREAM_NON_BLOCKING));
        // the workspace of Device::forest_workspace (trees.rs:128-160)
        CK(cuMemAlloc(&leaves, leaves_n * 8));
        for (uint32_t t = 1; t < h; t++) {
            CUdeviceptr p;
            CK(cuMemAlloc(&p, (leaves_n >> (h - t)) * 8));
            levels.push_back(p);
        }
        const uint64_t width = std::max<uint64_t>(leaves_n / 2, 2);
        for (CUdeviceptr* p : {&cur0, &cur1, &sp0, &sp1}) CK(cuMemAlloc(p, width * 8));
        CK(cuMemAlloc(&partials, 6 * SUM_BLOCKS * 8));
        CK(cuMemAlloc(&sums, 6 * SUM_THREADS * 8));
        const uint32_t half = vars >= 2 ? (vars - 2 + 1) / 2 : 0;
        const uint64_t eq_len = 2ull << half;
        CK(cuMemAlloc(&eq_lo, eq_len * 8));
        CK(cuMemAlloc(&eq_hi, eq_len * 8));
        CK(cuMemAlloc(&points, 2 * 8 * (vars + 1)));
        // the leaves: Device::fill_counter(leaves, 1 << 61) (gpu_unit_costs.rs:180)
        uint64_t len = leaves_n, base = 1ull << 61;
        void* args[] = {&leaves, &len, &base};
        CK(cuLaunchKernel(fill_counter, (uint32_t)((len + 1023) / 1024), 1, 1, 1024, 1, 1, 0, s, args, nullptr));
        CK(cuStreamSynchronize(s));
        return true;
    }

    bool launch1024(CUfunction f, uint64_t items, void** args) {
        CK(cuLaunchKernel(f, (uint32_t)std::max<uint64_t>(1, (items + 1023) / 1024), 1, 1, 1024, 1, 1, 0, s, args,
                          nullptr));
        return true;
    }

    bool eq(uint32_t first, uint32_t m, CUdeviceptr out) {
        void* args[] = {&points, &first, &m, &out};
        return launch1024(eq_table, 1ull << m, args);
    }

    // One round's three sums (trees.rs:342-452): the fused kernel, the reduction, the read-back.
    bool round_sums(int kind, CUdeviceptr v, CUdeviceptr e, CUdeviceptr o, F2 c, CUdeviceptr eo, CUdeviceptr oo,
                    uint64_t pairs, uint32_t lo_bits, F2 out[3]) {
        uint32_t blocks = (uint32_t)std::min<uint64_t>(std::max<uint64_t>((pairs + SUM_THREADS - 1) / SUM_THREADS, 1),
                                                       SUM_BLOCKS);
        uint64_t c0 = c.a, c1 = c.b;
        if (kind == 0) {
            void* args[] = {&v, &pairs, &eq_lo, &lo_bits, &eq_hi, &partials};
            CK(cuLaunchKernel(level_sums_base, blocks, 1, 1, SUM_THREADS, 1, 1, 0, s, args, nullptr));
        } else if (kind == 1) {
            void* args[] = {&v, &pairs, &c0, &c1, &eo, &oo, &eq_lo, &lo_bits, &eq_hi, &partials};
            CK(cuLaunchKernel(bind_sums_base, blocks, 1, 1, SUM_THREADS, 1, 1, 0, s, args, nullptr));
        } else {
            void* args[] = {&e, &o, &pairs, &c0, &c1, &eo, &oo, &eq_lo, &lo_bits, &eq_hi, &partials};
            CK(cuLaunchKernel(bind_sums_ext, blocks, 1, 1, SUM_THREADS, 1, 1, 0, s, args, nullptr));
        }
        void* rargs[] = {&partials, &blocks, &sums};
        CK(cuLaunchKernel(reduce_sums, 1, 1, 1, SUM_THREADS, 1, 1, 0, s, rargs, nullptr));
        uint64_t w[6];
        CK(cuMemcpyDtoHAsync(w, sums, 48, s));
        CK(cuStreamSynchronize(s));
        for (int k = 0; k < 3; k++) out[k] = {w[2 * k], w[2 * k + 1]};
        return true;
    }

    // Device::prove_forest_in (trees.rs:176-318) on transcript t.
    bool prove(or_transcript* t) {
        for (uint32_t lvl = height - 1; lvl >= 1; lvl--) {  // level lvl from level lvl + 1
            CUdeviceptr child = lvl + 1 < height ? levels[lvl] : leaves, parent = levels[lvl - 1];
            uint64_t n = leaves_n >> (height - lvl);
            void* args[] = {&child, &parent, &n};
            if (!launch1024(tree_level, n, args)) return false;
        }
        char label[96];
        std::vector<F2> point;
        for (uint32_t c = 0; c < vars - height; c++) {
            snprintf(label, sizeof label, "tree/0/root/%u", c);
            uint64_t r[2];
            or_transcript_challenge_fp2(t, label, r);
            point.push_back({r[0], r[1]});
        }
        for (uint32_t level = 0; level < height; level++) {
            uint64_t g[2];
            snprintf(label, sizeof label, "tree/%u/gamma", level);
            or_transcript_challenge_fp2(t, label, g);
            const CUdeviceptr table = level < levels.size() ? levels[level] : leaves;
            const uint32_t n = (uint32_t)point.size();
            std::vector<F2> chal;
            F2 u, w;
            if (n == 0) {
                uint64_t v[2];
                CK(cuMemcpyDtoHAsync(v, table, 16, s));
                CK(cuStreamSynchronize(s));
                u = {v[0], 0};
                w = {v[1], 0};
            } else {
                std::vector<uint64_t> pw;
                for (const F2& x : point) {
                    pw.push_back(x.a);
                    pw.push_back(x.b);
                }
                CK(cuMemcpyHtoDAsync(points, pw.data(), pw.size() * 8, s));
                F2 scale = F2_ONE;
                for (uint32_t j = 0; j < n; j++) {
                    const uint64_t pairs = 1ull << (n - 1 - j);
                    const uint32_t rest = n - 1 - j, lo_bits = (rest + 1) / 2;
                    if (!eq(j + 1, lo_bits, eq_lo) || !eq(j + 1 + lo_bits, rest - lo_bits, eq_hi)) return false;
                    F2 sm[3];
                    bool ok_;
                    if (j == 0) {
                        ok_ = round_sums(0, table, 0, 0, F2{0, 0}, 0, 0, pairs, lo_bits, sm);
                    } else if (j == 1) {
                        ok_ = round_sums(1, table, 0, 0, chal.back(), cur0, cur1, pairs, lo_bits, sm);
                    } else {
                        ok_ = round_sums(2, 0, cur0, cur1, chal.back(), sp0, sp1, pairs, lo_bits, sm);
                        std::swap(cur0, sp0);
                        std::swap(cur1, sp1);
                    }
                    if (!ok_) return false;
                    const F2 r = point[j];
                    auto eq_at = [&](F2 c) { return f2add(f2mul(f2sub(F2_ONE, r), f2sub(F2_ONE, c)), f2mul(r, c)); };
                    const F2 two = {2, 0}, three = {3, 0};
                    const F2 s3 = f2add(f2sub(sm[0], f2mul(three, sm[1])), f2mul(three, sm[2]));
                    uint64_t msg[6];
                    const F2 m0 = f2mul(f2mul(scale, eq_at(F2{0, 0})), sm[0]);
                    const F2 m2 = f2mul(f2mul(scale, eq_at(two)), sm[2]);
                    const F2 m3 = f2mul(f2mul(scale, eq_at(three)), s3);
                    msg[0] = m0.a, msg[1] = m0.b, msg[2] = m2.a, msg[3] = m2.b, msg[4] = m3.a, msg[5] = m3.b;
                    snprintf(label, sizeof label, "tree/%u/round/%u", level, j);
                    or_transcript_absorb_fp2s(t, label, msg, 3);
                    uint64_t c[2];
                    snprintf(label, sizeof label, "tree/%u/r/%u", level, j);
                    or_transcript_challenge_fp2(t, label, c);
                    scale = f2mul(scale, eq_at(F2{c[0], c[1]}));
                    chal.push_back({c[0], c[1]});
                }
                // the last round's binding, to one entry per table
                uint64_t c0 = chal.back().a, c1 = chal.back().b, one = 1;
                if (n == 1) {
                    CUdeviceptr tb = table;
                    void* args[] = {&tb, &one, &c0, &c1, &cur0, &cur1};
                    if (!launch1024(bind_base, 1, args)) return false;
                } else {
                    void* args[] = {&cur0, &cur1, &one, &c0, &c1, &sp0, &sp1};
                    if (!launch1024(bind_ext, 1, args)) return false;
                    std::swap(cur0, sp0);
                    std::swap(cur1, sp1);
                }
                uint64_t e[2], o[2];
                CK(cuMemcpyDtoHAsync(e, cur0, 16, s));
                CK(cuMemcpyDtoHAsync(o, cur1, 16, s));
                CK(cuStreamSynchronize(s));
                u = {e[0], e[1]};
                w = {o[0], o[1]};
            }
            uint64_t ev[4] = {u.a, u.b, w.a, w.b};
            snprintf(label, sizeof label, "tree/%u/evals", level);
            or_transcript_absorb_fp2s(t, label, ev, 2);
            uint64_t rho[2];
            snprintf(label, sizeof label, "tree/%u/line", level);
            or_transcript_challenge_fp2(t, label, rho);
            point.clear();
            point.push_back({rho[0], rho[1]});
            point.insert(point.end(), chal.begin(), chal.end());
        }
        return true;
    }

    void close() {
        for (CUdeviceptr p : levels) cuMemFree(p);
        for (CUdeviceptr p : {leaves, cur0, cur1, sp0, sp1, partials, sums, eq_lo, eq_hi, points})
            if (p) cuMemFree(p);
        if (s) cuStreamDestroy(s);
        if (mod) cuModuleUnload(mod);
        if (cmod) cuModuleUnload(cmod);
        if (ctx) cuDevicePrimaryCtxRelease(dev);
    }
};

// ---- c_ℓ: one fraction tree -----------------------------------------------------------------

struct Fraction {
    CUcontext ctx = nullptr;
    CUmodule mod = nullptr;
    CUstream s = nullptr;
    CUdevice dev = 0;
    CUfunction level_leaves, level, first_stored, first_leaves, sums_stored, sums_leaves, bind_sums_stored,
        bind_sums_leaves, bind_sums_bound, last_stored, last_leaves, last_bound, eq_table, reduce_sums;
    uint32_t height = 0, unit = 0;
    uint64_t leaf[7];  // key seed, value seed, multiplicity seed, α (two words), β (two words)
    std::vector<CUdeviceptr> num, den;  // level t at index t − 1, 1 <= t < h: 2^t Fp2 entries
    CUdeviceptr cur[4] = {0, 0, 0, 0}, spare[4] = {0, 0, 0, 0}, partials = 0, sums = 0, eq_lo = 0, eq_hi = 0,
                finals = 0, points = 0;

    bool open(const char* trees_fatbin, uint32_t h, const uint64_t seeds_ab[7], uint32_t unit_) {
        height = h;
        unit = unit_;
        memcpy(leaf, seeds_ab, sizeof leaf);
        CK(cuInit(0));
        CK(cuDeviceGet(&dev, 0));
        CK(cuDevicePrimaryCtxRetain(&ctx, dev));
        CK(cuCtxSetCurrent(ctx));
        CK(cuModuleLoad(&mod, trees_fatbin));
        const char* names[] = {"frac_level_leaves", "frac_level", "frac_first_stored", "frac_first_leaves",
                               "frac_sums_stored", "frac_sums_leaves", "frac_bind_sums_stored",
                               "frac_bind_sums_leaves", "frac_bind_sums_bound", "frac_last_stored",
                               "frac_last_leaves", "frac_last_bound", "eq_table", "reduce_sums"};
        CUfunction* fns[] = {&level_leaves, &level, &first_stored, &first_leaves, &sums_stored, &sums_leaves,
                             &bind_sums_stored, &bind_sums_leaves, &bind_sums_bound, &last_stored, &last_leaves,
                             &last_bound, &eq_table, &reduce_sums};
        for (int i = 0; i < 14; i++) CK(cuModuleGetFunction(fns[i], mod, names[i]));
        CK(cuStreamCreate(&s, CU_STREAM_NON_BLOCKING));
        // the workspace of Device::fraction_workspace (fraction.rs:160-206)
        const uint64_t d_len = 2 * std::max<uint64_t>(1ull << (h >= 2 ? h - 2 : 0), 2);
        const uint64_t n_len = unit ? 2 * std::max<uint64_t>(1ull << (h >= 3 ? h - 3 : 0), 2) : d_len;
        const uint32_t half = h >= 2 ? (h - 2 + 1) / 2 : 0;
        const uint64_t eq_len = 2ull << half;
        for (uint32_t t = 1; t < h; t++) {
            CUdeviceptr a, b;
            CK(cuMemAlloc(&a, (2ull << t) * 8));
            CK(cuMemAlloc(&b, (2ull << t) * 8));
            num.push_back(a);
            den.push_back(b);
        }
        const uint64_t lens[4] = {n_len, n_len, d_len, d_len};
        for (int i = 0; i < 4; i++) {
            CK(cuMemAlloc(&cur[i], lens[i] * 8));
            CK(cuMemAlloc(&spare[i], lens[i] * 8));
        }
        CK(cuMemAlloc(&partials, 6 * SUM_BLOCKS * 8));
        CK(cuMemAlloc(&sums, 6 * SUM_THREADS * 8));
        CK(cuMemAlloc(&eq_lo, eq_len * 8));
        CK(cuMemAlloc(&eq_hi, eq_len * 8));
        CK(cuMemAlloc(&finals, 64));
        CK(cuMemAlloc(&points, 2 * 8 * (h + 1)));
        return true;
    }

    // Pushes LEAF_ARGS (seven words and unit) then `rest` into one argument list.
    std::vector<void*> with_leaf(std::initializer_list<void*> rest) {
        std::vector<void*> a;
        for (int i = 0; i < 7; i++) a.push_back(&leaf[i]);
        a.push_back(&unit);
        a.insert(a.end(), rest.begin(), rest.end());
        return a;
    }

    bool launch(CUfunction f, uint32_t blocks, uint32_t threads, std::vector<void*> args) {
        CK(cuLaunchKernel(f, blocks, 1, 1, threads, 1, 1, 0, s, args.data(), nullptr));
        return true;
    }

    bool prove(or_transcript* t) {
        // levels h − 1 down to 1 (fraction.rs:327-375)
        for (uint32_t lv = height - 1; lv >= 1; lv--) {
            uint64_t parents = 1ull << lv;
            const uint32_t blocks = (uint32_t)((parents + 1023) / 1024);
            CUdeviceptr no = num[lv - 1], dout = den[lv - 1];
            if (lv + 1 < height) {
                CUdeviceptr ni = num[lv], di = den[lv];
                if (!launch(level, blocks, 1024, {&ni, &di, &no, &dout, &parents})) return false;
            } else if (!launch(level_leaves, blocks, 1024, with_leaf({&no, &dout, &parents}))) {
                return false;
            }
        }
        char label[96];
        std::vector<F2> point;
        for (uint32_t lvl = 0; lvl < height; lvl++) {
            uint64_t g[2], lam[2];
            snprintf(label, sizeof label, "tree/%u/gamma", lvl);
            or_transcript_challenge_fp2(t, label, g);
            snprintf(label, sizeof label, "tree/%u/lambda", lvl);
            or_transcript_challenge_fp2(t, label, lam);
            const bool stored = lvl + 1 < height;
            CUdeviceptr nt = stored ? num[lvl] : 0, dt = stored ? den[lvl] : 0;
            uint32_t level_unit = (!stored && unit == 1) ? 1 : 0;
            const uint32_t n = (uint32_t)point.size();
            std::vector<F2> chal;
            if (n == 0) {
                if (stored) {
                    if (!launch(first_stored, 1, 1, {&nt, &dt, &finals})) return false;
                } else if (!launch(first_leaves, 1, 1, with_leaf({&finals}))) {
                    return false;
                }
            } else {
                std::vector<uint64_t> pw;
                for (const F2& x : point) {
                    pw.push_back(x.a);
                    pw.push_back(x.b);
                }
                CK(cuMemcpyHtoDAsync(points, pw.data(), pw.size() * 8, s));
                F2 scale = F2_ONE;
                for (uint32_t j = 0; j < n; j++) {
                    uint64_t pairs = 1ull << (n - 1 - j);
                    uint32_t rest = n - 1 - j, lo_bits = (rest + 1) / 2, hi_bits = rest - lo_bits;
                    uint32_t first = j + 1, first_hi = j + 1 + lo_bits;
                    if (!launch(eq_table, (uint32_t)std::max<uint64_t>(1, ((1ull << lo_bits) + 1023) / 1024), 1024,
                                {&points, &first, &lo_bits, &eq_lo}) ||
                        !launch(eq_table, (uint32_t)std::max<uint64_t>(1, ((1ull << hi_bits) + 1023) / 1024), 1024,
                                {&points, &first_hi, &hi_bits, &eq_hi}))
                        return false;
                    uint32_t blocks = (uint32_t)std::min<uint64_t>(
                        std::max<uint64_t>((pairs + SUM_THREADS - 1) / SUM_THREADS, 1), SUM_BLOCKS);
                    uint64_t l0 = lam[0], l1 = lam[1];
                    uint64_t c0 = chal.empty() ? 0 : chal.back().a, c1 = chal.empty() ? 0 : chal.back().b;
                    bool good;
                    if (j == 0 && stored) {
                        good = launch(sums_stored, blocks, SUM_THREADS,
                                      {&nt, &dt, &pairs, &l0, &l1, &eq_lo, &lo_bits, &eq_hi, &partials});
                    } else if (j == 0) {
                        good = launch(sums_leaves, blocks, SUM_THREADS,
                                      with_leaf({&pairs, &l0, &l1, &eq_lo, &lo_bits, &eq_hi, &partials}));
                    } else if (j == 1 && stored) {
                        good = launch(bind_sums_stored, blocks, SUM_THREADS,
                                      {&nt, &dt, &c0, &c1, &cur[0], &cur[1], &cur[2], &cur[3], &pairs, &l0, &l1,
                                       &eq_lo, &lo_bits, &eq_hi, &partials});
                    } else if (j == 1) {
                        good = launch(bind_sums_leaves, blocks, SUM_THREADS,
                                      with_leaf({&c0, &c1, &cur[0], &cur[1], &cur[2], &cur[3], &pairs, &l0, &l1,
                                                 &eq_lo, &lo_bits, &eq_hi, &partials}));
                    } else {
                        good = launch(bind_sums_bound, blocks, SUM_THREADS,
                                      {&cur[0], &cur[1], &cur[2], &cur[3], &level_unit, &c0, &c1, &spare[0],
                                       &spare[1], &spare[2], &spare[3], &pairs, &l0, &l1, &eq_lo, &lo_bits, &eq_hi,
                                       &partials});
                        for (int i = 0; i < 4; i++) std::swap(cur[i], spare[i]);
                    }
                    if (!good) return false;
                    if (!launch(reduce_sums, 1, SUM_THREADS, {&partials, &blocks, &sums})) return false;
                    uint64_t w[6];
                    CK(cuMemcpyDtoHAsync(w, sums, 48, s));
                    CK(cuStreamSynchronize(s));
                    const F2 sm[3] = {{w[0], w[1]}, {w[2], w[3]}, {w[4], w[5]}};
                    const F2 r = point[j];
                    auto eq_at = [&](F2 c) { return f2add(f2mul(f2sub(F2_ONE, r), f2sub(F2_ONE, c)), f2mul(r, c)); };
                    const F2 two = {2, 0}, three = {3, 0};
                    const F2 s3 = f2add(f2sub(sm[0], f2mul(three, sm[1])), f2mul(three, sm[2]));
                    const F2 m0 = f2mul(f2mul(scale, eq_at(F2{0, 0})), sm[0]);
                    const F2 m2 = f2mul(f2mul(scale, eq_at(two)), sm[2]);
                    const F2 m3 = f2mul(f2mul(scale, eq_at(three)), s3);
                    uint64_t msg[6] = {m0.a, m0.b, m2.a, m2.b, m3.a, m3.b};
                    snprintf(label, sizeof label, "tree/%u/round/%u", lvl, j);
                    or_transcript_absorb_fp2s(t, label, msg, 3);
                    uint64_t c[2];
                    snprintf(label, sizeof label, "tree/%u/r/%u", lvl, j);
                    or_transcript_challenge_fp2(t, label, c);
                    scale = f2mul(scale, eq_at(F2{c[0], c[1]}));
                    chal.push_back({c[0], c[1]});
                }
                uint64_t c0 = chal.back().a, c1 = chal.back().b;
                bool good;
                if (n == 1 && stored)
                    good = launch(last_stored, 1, 1, {&nt, &dt, &c0, &c1, &finals});
                else if (n == 1)
                    good = launch(last_leaves, 1, 1, with_leaf({&c0, &c1, &finals}));
                else
                    good = launch(last_bound, 1, 1, {&cur[0], &cur[1], &cur[2], &cur[3], &level_unit, &c0, &c1, &finals});
                if (!good) return false;
            }
            uint64_t f[8];
            CK(cuMemcpyDtoHAsync(f, finals, 64, s));
            CK(cuStreamSynchronize(s));
            snprintf(label, sizeof label, "tree/%u/evals", lvl);
            or_transcript_absorb_fp2s(t, label, f, 4);
            uint64_t rho[2];
            snprintf(label, sizeof label, "tree/%u/line", lvl);
            or_transcript_challenge_fp2(t, label, rho);
            point.clear();
            point.push_back({rho[0], rho[1]});
            point.insert(point.end(), chal.begin(), chal.end());
        }
        return true;
    }

    void close() {
        for (CUdeviceptr p : num) cuMemFree(p);
        for (CUdeviceptr p : den) cuMemFree(p);
        for (int i = 0; i < 4; i++) {
            if (cur[i]) cuMemFree(cur[i]);
            if (spare[i]) cuMemFree(spare[i]);
        }
        for (CUdeviceptr p : {partials, sums, eq_lo, eq_hi, finals, points})
            if (p) cuMemFree(p);
        if (s) cuStreamDestroy(s);
        if (mod) cuModuleUnload(mod);
        if (ctx) cuDevicePrimaryCtxRelease(dev);
    }
};

// The transcript of the reference benchmark's proofs (gpu_unit_costs.rs transcript()): protocol
// "tessera-protocol/1", non-interactive, params "bench/1", statement [0x65; 32], session [0x13; 16].
void bench_transcript(or_transcript* t) {
    std::vector<uint8_t> tce;
    auto le = [&](uint64_t v, int bytes) {
        for (int i = 0; i < bytes; i++) tce.push_back((uint8_t)(v >> (8 * i)));
    };
    const char* proto = "tessera-protocol/1";
    const char* params = "bench/1";
    le(strlen(proto), 8);
    tce.insert(tce.end(), proto, proto + strlen(proto));
    le(1, 2);
    le(strlen(params), 8);
    tce.insert(tce.end(), params, params + strlen(params));
    tce.insert(tce.end(), 32, 0x65);
    tce.insert(tce.end(), 16, 0x13);
    or_transcript_init(t, tce.data(), tce.size());
}

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

// c_π: out[0] the median seconds of one forest proof (after `warmup` proofs, over `runs`);
// state (32 bytes) and *counter: the transcript after the first proof. Returns 0 or −1.
int refgpu_pi(const char* trees_fatbin, const char* commit_fatbin, uint32_t s_log, uint32_t h, int warmup, int runs,
              double* out, uint8_t* state, uint64_t* counter) {
    if (h < 1 || s_log + h > 34 || runs < 1) {
        g_err = "a forest of 2^s trees of height 1..34 - s";
        return -1;
    }
    Forest f;
    bool good = f.open(trees_fatbin, commit_fatbin, s_log, h);
    std::vector<double> ts;
    for (int i = 0; good && i < warmup + runs; i++) {
        or_transcript t;
        bench_transcript(&t);
        const auto t0 = std::chrono::steady_clock::now();
        good = f.prove(&t);
        if (good) good = ok(cuStreamSynchronize(f.s), "cuStreamSynchronize");
        const double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        if (good && i == 0) {
            memcpy(state, t.state, 32);
            *counter = t.counter;
        }
        if (good && i >= warmup) ts.push_back(dt);
    }
    f.close();
    if (!good) return -1;
    out[0] = median(ts);
    return 0;
}

// One fraction tree of height h: leaf j is (1, α − (k_j + β·v_j)) with unit, else (−m_j, α −
// (k_j + β·v_j)), k_j = counter(key_seed + j), v_j = counter(value_seed + j), m_j =
// counter(mult_seed + j) mod 2^16 (fraction.rs:61-105); seeds_ab = {key, value, mult, α0, α1, β0, β1}.
// out[0]: the median seconds of one proof; state and *counter: the transcript after the first.
int refgpu_fraction(const char* trees_fatbin, uint32_t h, const uint64_t seeds_ab[7], uint32_t unit, int warmup,
                    int runs, double* out, uint8_t* state, uint64_t* counter) {
    if (h < 1 || h > 34 || runs < 1) {
        g_err = "a fraction tree of height 1..34";
        return -1;
    }
    Fraction f;
    bool good = f.open(trees_fatbin, h, seeds_ab, unit);
    std::vector<double> ts;
    for (int i = 0; good && i < warmup + runs; i++) {
        or_transcript t;
        bench_transcript(&t);
        const auto t0 = std::chrono::steady_clock::now();
        good = f.prove(&t);
        if (good) good = ok(cuStreamSynchronize(f.s), "cuStreamSynchronize");
        const double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        if (good && i == 0) {
            memcpy(state, t.state, 32);
            *counter = t.counter;
        }
        if (good && i >= warmup) ts.push_back(dt);
    }
    f.close();
    if (!good) return -1;
    out[0] = median(ts);
    return 0;
}

}  // extern "C"
