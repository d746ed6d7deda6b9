// SPDX-License-Identifier: Apache-2.0 OR MIT
//
// Internal host-side declarations shared by the translation units of libtessera_gb300.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/tessera_gb300.h"
#include "gl.cuh"

namespace tg {

// Records the failure message for tg_last_error() (thread-local) and returns `code`.
int fail(int code, const char* fmt, ...);
int cuda_fail(cudaError_t e, const char* what);

#define TG_CUDA(call)                                      \
    do {                                                   \
        cudaError_t e_ = (call);                           \
        if (e_ != cudaSuccess) return tg::cuda_fail(e_, #call); \
    } while (0)

// A device buffer that grows on demand and is freed with its owner.
struct DevBuf {
    void* ptr = nullptr;
    size_t bytes = 0;
    bool owned = true;  // false: a caller's memory, read in place and never freed here
    int ensure(size_t want);
    void release();
    ~DevBuf() { release(); }
};

// Twiddle tables for one codeword length n = 2^lgn and message length k = 2^lgk:
// pw[m] = ω_n^m for m < n, and pow7k[i] = 7^i / k for i < k. Built once and kept on the device.
struct Tables {
    uint32_t lgn = 0, lgk = 0;
    uint64_t* pw = nullptr;
    uint64_t* pow7k = nullptr;
};

// Per-kernel timing on the launching stream: when enabled, each launch is bracketed by a pair of
// CUDA events; tg_profile_read sums their elapsed times by kernel name.
struct ProfRec {
    const char* name;
    cudaEvent_t begin, end;
    uint64_t units;  // work units of the launch (rows, columns, pairs), for per-unit rates
};

// A stream of the batched commitment path with its own encoder scratch.
struct Worker {
    cudaStream_t s = nullptr;
    cudaEvent_t done = nullptr;
    DevBuf y, z;
};

struct Device {
    int ordinal = 0;
    cudaStream_t stream = nullptr;
    int sm_count = 0;
    size_t smem_optin = 0;
    int coop = -1;  // cooperative launches supported (1) or not (0); −1 until asked
    std::mutex mu;  // guards the caches and the shared scratch below
    std::map<uint64_t, Tables> tables;
    DevBuf scratch_y, scratch_z, scratch_misc;
    DevBuf scratch_sc;  // the sumcheck's tables, transcript state and outputs
    // The host-buffer commitment's pipeline: row chunks are copied into one half of stage_rows on
    // copy_stream while the chunk in the other half is encoded on `stream`.
    DevBuf stage_rows, stage_cw, stage_nodes;
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t staged[2] = {nullptr, nullptr}, consumed[2] = {nullptr, nullptr};
    cudaEvent_t ramp[4] = {nullptr, nullptr, nullptr, nullptr};  // the first chunk's pieces landed
    DevBuf err;  // device error words for bounded waits
    DevBuf scratch_aux;  // the advice mask stream's per-CTA counts and offsets
    // Pinned host memory that small results (a tree level's or a sumcheck batch's transcript
    // states, messages, challenges, evaluations) come back through in one copy and one wait, not a
    // synchronous copy each (readback_ensure grows it; used under mu).
    uint8_t* readback = nullptr;
    size_t readback_bytes = 0;
    tg_config cfg;
    std::atomic<uint64_t> launches{0};  // kernels this handle has launched
    // While a CUDA graph is captured, Launch counts kernels into `captured` instead (a replay
    // adds them to `launches`) and records no profiling events.
    bool capturing = false;
    uint64_t captured = 0;
    std::vector<Worker*> workers;  // the batched commitment path's streams, created on demand
    cudaEvent_t fork = nullptr;
    DevBuf batch_roots;
    bool prof_on = false;
    std::mutex prof_mu;
    std::vector<ProfRec> prof;
    std::vector<cudaEvent_t> event_pool;
    // Workspace memory released by leaf stages (levels, bound tables), kept for later stages as a
    // prover pools its device memory: a stage takes the smallest spare buffer that fits before it
    // allocates. The cache goes back to the driver (zeroed) when it would pass spare_cap bytes
    // (half the device's memory), when an allocation fails, and on tg_device_trim.
    std::mutex spare_mu;
    std::multimap<size_t, void*> spare;
    size_t spare_bytes = 0, spare_cap = 0;
    // Returns the tables for (lgn, lgk), building them on first use.
    int get_tables(uint32_t lgn, uint32_t lgk, const Tables** out);
};

// Device::readback of at least `bytes` (caller holds d->mu).
int readback_ensure(Device* d, size_t bytes);

cudaStream_t pick_stream(Device* d, void* stream);

// Reads one byte of every page of a host buffer (tg_host_prefault).
void host_prefault(const void* p, size_t bytes);

// The workspace cache: b (empty) gets a spare buffer of at least `want` bytes (at most twice that)
// or a new one; spare_give returns b's memory to the cache (a borrowed buffer is only dropped);
// spare_trim zeroes and frees every spare buffer.
int spare_take(Device* d, DevBuf& b, size_t want);
void spare_give(Device* d, DevBuf& b);
void spare_trim(Device* d);

// Brackets the kernel launches of one logical kernel on stream s: counts them, and records
// events around them while profiling is on.
struct Launch {
    Device* d;
    cudaStream_t s;
    int idx = -1;
    Launch(Device* d, cudaStream_t s, const char* name, uint64_t nkernels, uint64_t units);
    ~Launch();
};

// ---- LDE (lde.cu) ---------------------------------------------------------------------------
// Encodes npolys rows of k = 2^lgk values (device, row-major) into codewords of n = 2^(lgk+lgr)
// symbols (device, row-major), with P mask coefficients per row (device, may be null for P = 0).
int lde_encode(Device* d, uint32_t lgk, uint32_t lgr, uint32_t P, const uint64_t* rows, size_t npolys,
               const uint64_t* masks, uint64_t* codewords, cudaStream_t s);

// The same encoder over caller-owned tables (pw: n words, pow7k: k words; rebuilt when
// build_tables) and scratch (y: group x k words, z: group x n words); allocates nothing. For
// 2^13 <= k <= 2^22, lgk1 picks the split of the row transform into 2^lgk1 by 2^(lgk − lgk1)
// (0: the default; encode_split_valid says which are built).
int lde_encode_into(Device* d, uint32_t lgk, uint32_t lgr, uint32_t P, const uint64_t* rows, size_t npolys,
                    const uint64_t* masks, uint64_t* codewords, cudaStream_t s, uint64_t* pw, uint64_t* pow7k,
                    bool build_tables, uint64_t* y, uint64_t* z, size_t group, int lgk1 = 0);
bool encode_split_valid(uint32_t lgk, int lgk1);

// Standalone transforms over nrows rows of n = 2^lgn values in place, natural order on both
// sides (NttPlan::{ntt, intt, coset_ntt, coset_intt}, crates/tessera-pcs/src/ntt.rs:461-516);
// shift is used by the coset kinds only. lgn <= 22.
enum { NTT_FORWARD = 0, NTT_INVERSE = 1, NTT_COSET_FORWARD = 2, NTT_COSET_INVERSE = 3 };
int ntt_rows(Device* d, int kind, uint32_t lgn, uint64_t shift, uint64_t* values, size_t nrows, cudaStream_t s);

// ---- hashing (hash.cu) ----------------------------------------------------------------------
// Context keys of the domains the hot path uses, derived on the host.
void context_key(const char* name, uint32_t key[8]);
int column_init(Device* d, const uint8_t id[32], uint64_t ncols, uint8_t* chains, cudaStream_t s);
// Absorbs `count` rows (row-major, count x ncols, row stride `ld` symbols) in blocks of
// `block` rows into the chains.
int column_absorb(Device* d, uint8_t* chains, uint64_t ncols, const uint64_t* rows, size_t ld, size_t count,
                  uint32_t block, cudaStream_t s);
int merkle_tree(Device* d, const uint8_t* leaves, size_t n, uint8_t* nodes, cudaStream_t s);
int column_merge(Device* d, const uint8_t* segs, size_t nseg, uint64_t n, uint8_t* leaves, cudaStream_t s);
// out[i] = the (first + i)-th word below p of the advice mask stream of `seed` (BLAKE3's extended
// output of H("advice-masks", seed), rejection-sampled), i < count; waits for the stream.
int advice_masks(Device* d, const uint8_t* seed, size_t seed_len, uint64_t first, uint64_t count, uint64_t* out,
                 cudaStream_t s);

// ---- openings (opening.cu) -------------------------------------------------------------------
// The answer to column queries on resident codewords (rows x n) and Merkle nodes (2n − 1
// digests, leaves first): cols[q·rows + r] = cw[r·n + idx[q]] for the m indices, and sib[t] the
// digest of node node[t], for ns nodes. All pointers on the device; enqueued on s.
int gather_answer(Device* d, const uint64_t* cw, uint64_t n, uint32_t rows, const uint64_t* idx, uint32_t m,
                  uint64_t* cols, const uint8_t* nodes, const uint64_t* node, uint32_t ns, uint8_t* sib,
                  cudaStream_t s);

// A bump allocator over one device buffer, 256-byte aligned pieces.
struct Arena {
    size_t used = 0;
    uint8_t* base = nullptr;
    size_t take(size_t bytes) {
        const size_t at = used;
        used += (bytes + 255) & ~(size_t)255;
        return at;
    }
    template <typename T>
    T* at(size_t off) const {
        return reinterpret_cast<T*>(base + off);
    }
};

// ---- sumcheck in phases (sumcheck.cu), for callers with their own streams and memory --------
// sc_prepare validates the jobs and draws each job's γ on its host transcript (NULL and *status
// on refusal, transcripts untouched); sc_enqueue launches everything on stream s over `arena`
// (sc_arena_bytes of device memory) and copies the results into `host_out` (sc_host_bytes; pinned
// memory for the copy to stay asynchronous); once the stream has run, sc_finish updates the
// transcripts and outputs. sc_restore puts the transcripts back as they were before sc_prepare.
// Options for callers that run their own protocol around a sumcheck (the tree levels): with
// `weights` (one job only) γ is not drawn and instance i weighs weights[i]; without
// `absorb_evals` the final evaluations are returned but not absorbed.
struct ScOptions {
    const std::vector<fp2>* weights = nullptr;
    bool absorb_evals = true;
};
struct ScRun;
ScRun* sc_prepare(Device* d, tg_sumcheck_job* jobs, int njobs, int tables_on_device, int* status,
                  const ScOptions& opts = ScOptions());
// The blocking form: prepare, enqueue on the device stream, wait, finish.
int prove_many_opts(Device* d, tg_sumcheck_job* jobs, int njobs, int tables_on_device, const ScOptions& opts);
size_t sc_arena_bytes(const ScRun* r);
size_t sc_host_bytes(const ScRun* r);
int sc_enqueue(Device* d, ScRun* r, cudaStream_t s, void* arena, void* host_out);
int sc_finish(ScRun* r);
int sc_restore(ScRun* r, int rc);
void sc_free(ScRun* r);

// ---- host BLAKE3 and transcript (host.cpp) --------------------------------------------------
void host_hash(const uint32_t key[8], const uint8_t* in, size_t len, uint8_t out[32]);

}  // namespace tg
