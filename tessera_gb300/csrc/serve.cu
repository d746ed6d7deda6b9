// SPDX-License-Identifier: Apache-2.0 OR MIT
//
// A proof server with continuous batching: requests are admitted as stream slots and HBM budget
// free up, each admitted request runs on its own stream with its own device memory (stream-ordered
// allocations, so admission never synchronises the device), and requests at different stages
// overlap on the GPU. A scheduler thread moves each request through its stages:
//
//   1. commit: rows host → device, encode, column chains, Merkle tree, root → pinned host memory
//   2. the host absorbs the root into the request's transcript (the sumcheck's challenges depend
//      on the commitment), draws γ, and enqueues the sumcheck with its transcript on the device
//   3. with queries: the host finishes the sumcheck's transcript, draws the query indices from it,
//      and the device gathers the answer (the queried columns of the resident codewords and the
//      canonical multiproof from the resident Merkle nodes) into pinned host memory
//   4. the host finishes the proof (transcript, round messages, evaluations, answer), frees the
//      request's device memory and hands the result to the waiting caller
//
// A stage's work ends with a host function on its stream that wakes the scheduler, so no thread
// polls while the GPU works. Each slot has a high- and a low-priority stream: the oldest request
// in flight enqueues its next stage on the high one, the others on the low one, so overlapping
// requests are served first come first served and the newer fill the gaps.
//
// A request's proof is a unit of the reference's prover shape: a resident unmasked commitment
// (crates/tessera-pcs/src/commitment.rs:343-458) whose root is absorbed under "<prefix>/root",
// then a one-instance prove_batch (crates/tessera-sumcheck/src/prover.rs:1122) of the product of
// its prime-field tables under <prefix>. The result is byte-identical however many requests share
// the GPU with it: each request has its own transcript, buffers and stream.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "internal.h"

namespace tg {

using Clock = std::chrono::steady_clock;

struct ServeReq {
    uint64_t ticket = 0;
    tg_proof_request req;
    std::vector<const uint64_t*> table_ptrs;
    std::string prefix;
    tg_proof_result* out = nullptr;
    // sizes and the request's device block: rows | codewords | nodes | encoder y | encoder z | sumcheck arena
    uint64_t k = 0, n = 0;
    size_t group = 0, off_cw = 0, off_nodes = 0, off_y = 0, off_z = 0, off_sc = 0, off_q = 0, footprint = 0;
    uint8_t* dmem = nullptr;
    cudaStream_t s = nullptr;  // the stream of the request's current stage
    int slot = -1, stage = 0, status = TG_OK;
    // the opening round: distinct indices and sibling nodes, uploaded from the slot's staging
    std::vector<uint64_t> distinct, sib_nodes;
    Clock::time_point t_submit, t_admit;
    // the sumcheck
    tg_transcript transcript;
    std::vector<tg_table> tabs;
    tg_instance inst;
    tg_sumcheck_job job;
    ScRun* run = nullptr;
    const Tables* tables = nullptr;
};

static size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

}  // namespace tg

struct tg_server {
    tg::Device* d = nullptr;
    size_t budget = 0;
    int max_inflight = 0;
    std::thread th;
    std::mutex mu;
    std::condition_variable wake, done_cv;
    bool stop = false;
    uint64_t next_ticket = 1;
    std::deque<tg::ServeReq*> queue;
    std::vector<tg::ServeReq*> active;
    std::map<uint64_t, tg::ServeReq*> finished;  // done, not yet collected
    std::vector<cudaStream_t> streams, streams_hi;  // per slot: low and high priority
    std::vector<cudaEvent_t> events;
    std::vector<int> slot_busy;
    uint8_t* pinned = nullptr;  // kSlotPinned bytes per slot
    size_t in_use = 0;
    uint64_t completions = 0;  // stage ends signalled by the streams' host functions
    tg_server_stats stats;
};

namespace tg {

constexpr size_t kSlotPinned = 1 << 20;
constexpr size_t kSumcheckPinned = 64 << 10;  // the sumcheck's outputs, after the 32-byte root

// A request's answer and its uploaded index lists: at most queries · (8·npolys + 40·log2 n + 8)
// bytes (distinct indices ≤ queries, multiproof siblings ≤ queries·log2 n).
static size_t answer_bytes(uint32_t queries, size_t npolys, uint32_t log_n) {
    return (size_t)queries * (8 * npolys + 40ull * log_n + 8);
}

// Runs on a CUDA host thread after a stage's work: wakes the scheduler (no CUDA calls here).
static void CUDART_CB stage_done(void* arg) {
    tg_server* sv = static_cast<tg_server*>(arg);
    {
        std::lock_guard<std::mutex> lock(sv->mu);
        sv->completions++;
    }
    sv->wake.notify_all();
}

// Records the slot's event and the wake-up after the work just enqueued on the stage's stream.
static int end_stage(tg_server* sv, ServeReq* r) {
    TG_CUDA(cudaEventRecord(sv->events[r->slot], r->s));
    TG_CUDA(cudaLaunchHostFunc(r->s, stage_done, sv));
    return TG_OK;
}

// The stream for a request's next stage: the slot's high-priority one for the oldest request in
// flight (the lowest ticket among the active), else its low one. The previous stage has ended.
static cudaStream_t stage_stream(tg_server* sv, ServeReq* r) {
    bool oldest = true;
    {
        std::lock_guard<std::mutex> lock(sv->mu);
        for (ServeReq* o : sv->active)
            if (o->ticket < r->ticket) oldest = false;
    }
    r->s = oldest ? sv->streams_hi[r->slot] : sv->streams[r->slot];
    return r->s;
}
constexpr size_t kServeGroupBytes = 256ull << 20;  // encoder scratch per request

// The request's sumcheck job over its (host) tables, on its own transcript copy.
static void build_job(ServeReq* r) {
    r->tabs.assign(r->req.ntables, tg_table());
    for (int k = 0; k < r->req.ntables; k++) {
        r->tabs[k].values = r->table_ptrs[k];
        r->tabs[k].is_ext = 0;
        r->tabs[k].is_public = 0;
    }
    r->inst.tables = r->tabs.data();
    r->inst.ntables = r->req.ntables;
    r->inst.vars = r->req.vars;
    memset(&r->job, 0, sizeof r->job);
    r->job.transcript = &r->transcript;
    r->job.prefix = r->prefix.c_str();
    r->job.degree = r->req.degree;
    r->job.instances = &r->inst;
    r->job.ninstances = 1;
    r->job.rounds = r->out->rounds;
    r->job.challenges = r->out->challenges;
    r->job.final_evals = r->out->final_evals;
}

// Stage 1: rows in, encode, chains, tree, root out.
static int start_commit(tg_server* sv, ServeReq* r) {
    Device* d = sv->d;
    cudaStream_t s = stage_stream(sv, r);
    TG_CUDA(cudaMallocAsync((void**)&r->dmem, r->footprint, s));
    uint64_t* rows = (uint64_t*)r->dmem;
    uint64_t* cw = (uint64_t*)(r->dmem + r->off_cw);
    uint8_t* nodes = r->dmem + r->off_nodes;
    const tg_proof_request& q = r->req;
    if (q.npolys) TG_CUDA(cudaMemcpyAsync(rows, q.rows, q.npolys * r->k * 8, cudaMemcpyHostToDevice, s));
    std::lock_guard<std::mutex> lock(d->mu);
    int rc = lde_encode_into(d, q.log_k, q.log_inv_rate, 0, rows, q.npolys, nullptr, cw, s, r->tables->pw,
                             r->tables->pow7k, false, (uint64_t*)(r->dmem + r->off_y), (uint64_t*)(r->dmem + r->off_z),
                             r->group);
    if (!rc) rc = column_init(d, q.commitment_id, r->n, nodes, s);
    if (!rc) rc = column_absorb(d, nodes, r->n, cw, r->n, q.npolys, q.row_block, s);
    if (!rc) rc = merkle_tree(d, nodes, r->n, nodes, s);
    if (rc) return rc;
    TG_CUDA(cudaMemcpyAsync(sv->pinned + kSlotPinned * r->slot, nodes + 32 * (2 * r->n - 2), 32, cudaMemcpyDeviceToHost, s));
    return end_stage(sv, r);
}

// Stage 2: the root into the transcript, γ, and the sumcheck on the device.
static int start_sumcheck(tg_server* sv, ServeReq* r) {
    Device* d = sv->d;
    cudaStream_t s = stage_stream(sv, r);
    uint8_t* pin = sv->pinned + kSlotPinned * r->slot;
    memcpy(r->out->root, pin, 32);
    int rc = tg_transcript_absorb(&r->transcript, (r->prefix + "/root").c_str(), r->out->root, 32);
    if (rc) return rc;
    build_job(r);
    r->run = sc_prepare(d, &r->job, 1, 0, &rc);
    if (!r->run) return rc;
    if (sc_host_bytes(r->run) + 32 > kSumcheckPinned) return fail(TG_ERR_INVALID, "sumcheck outputs exceed the slot's staging");
    {
        std::lock_guard<std::mutex> lock(d->mu);
        rc = sc_enqueue(d, r->run, s, r->dmem + r->off_sc, pin + 32);
    }
    if (rc) return rc;
    return end_stage(sv, r);
}

// Stage 3: the sumcheck's transcript finished on the host, the query indices drawn from it, and
// the answer gathered from the resident codewords and Merkle nodes into the slot's staging.
static int start_opening(tg_server* sv, ServeReq* r) {
    Device* d = sv->d;
    cudaStream_t s = stage_stream(sv, r);
    int rc = sc_finish(r->run);
    sc_free(r->run);
    r->run = nullptr;
    if (rc) return rc;
    const uint32_t lgn = r->req.log_k + r->req.log_inv_rate, tau = r->req.queries;
    rc = tg_transcript_challenge_indices(&r->transcript, (r->prefix + "/queries").c_str(), lgn, tau,
                                         r->out->query_indices);
    if (rc) return rc;
    r->distinct.assign(r->out->query_indices, r->out->query_indices + tau);
    std::sort(r->distinct.begin(), r->distinct.end());
    r->distinct.erase(std::unique(r->distinct.begin(), r->distinct.end()), r->distinct.end());
    // the canonical multiproof: per level from the leaves up, the sibling of every opened node
    // whose sibling is not opened, left to right; a level's nodes follow the level below's
    r->sib_nodes.clear();
    std::vector<uint64_t> cur = r->distinct, up;
    uint64_t base = 0, width = r->n;
    while (width > 1) {
        for (size_t i = 0; i < cur.size(); i++) {
            const uint64_t x = cur[i];
            const bool paired = (x & 1) ? (i > 0 && cur[i - 1] == (x ^ 1)) : (i + 1 < cur.size() && cur[i + 1] == (x ^ 1));
            if (!paired) r->sib_nodes.push_back(base + (x ^ 1));
        }
        up.clear();
        for (uint64_t x : cur)
            if (up.empty() || up.back() != (x >> 1)) up.push_back(x >> 1);
        cur.swap(up);
        base += width;
        width >>= 1;
    }
    const uint32_t m = (uint32_t)r->distinct.size(), ns = (uint32_t)r->sib_nodes.size();
    const size_t npolys = r->req.npolys;
    uint8_t* stage = sv->pinned + kSlotPinned * r->slot + kSumcheckPinned;
    uint64_t* lists = (uint64_t*)(r->dmem + r->off_q);
    memcpy(stage, r->distinct.data(), 8 * (size_t)m);
    memcpy(stage + 8 * (size_t)m, r->sib_nodes.data(), 8 * (size_t)ns);
    TG_CUDA(cudaMemcpyAsync(lists, stage, 8 * ((size_t)m + ns), cudaMemcpyHostToDevice, s));
    uint64_t* cols = lists + m + ns;
    uint8_t* sib = (uint8_t*)(cols + (size_t)m * npolys);
    {
        std::lock_guard<std::mutex> lock(d->mu);
        rc = gather_answer(d, (const uint64_t*)(r->dmem + r->off_cw), r->n, (uint32_t)npolys, lists, m, cols,
                           r->dmem + r->off_nodes, lists + m, ns, sib, s);
    }
    if (rc) return rc;
    // the answer lands after the index lists in the staging, which the copy above has read by then
    uint8_t* back = stage + 8 * ((size_t)m + ns);
    TG_CUDA(cudaMemcpyAsync(back, cols, 8 * (size_t)m * npolys + 32 * (size_t)ns, cudaMemcpyDeviceToHost, s));
    return end_stage(sv, r);
}

// Stage 3: the proof's outputs, memory back to the pool, the slot freed.
static void finish(tg_server* sv, ServeReq* r, int status) {
    cudaStream_t s = r->s ? r->s : sv->streams[r->slot];
    if (!status && r->run) status = sc_finish(r->run);
    if (!status && r->req.queries) {
        const size_t m = r->distinct.size(), ns = r->sib_nodes.size(), npolys = r->req.npolys;
        const uint8_t* back = sv->pinned + kSlotPinned * r->slot + kSumcheckPinned + 8 * (m + ns);
        memcpy(r->out->columns, back, 8 * m * npolys);
        memcpy(r->out->siblings, back + 8 * m * npolys, 32 * ns);
        r->out->n_distinct = (uint32_t)m;
        r->out->n_siblings = (uint32_t)ns;
    }
    if (r->run) {
        sc_free(r->run);
        r->run = nullptr;
    }
    if (r->dmem) {
        cudaFreeAsync(r->dmem, s);
        r->dmem = nullptr;
    }
    tg_proof_result* o = r->out;
    o->status = status;
    if (!status) {
        o->gamma[0] = r->job.gamma[0];
        o->gamma[1] = r->job.gamma[1];
        o->transcript = r->transcript;
    }
    const auto now = Clock::now();
    o->queued_ms = std::chrono::duration<double, std::milli>(r->t_admit - r->t_submit).count();
    o->latency_ms = std::chrono::duration<double, std::milli>(now - r->t_submit).count();
    std::lock_guard<std::mutex> lock(sv->mu);
    sv->slot_busy[r->slot] = 0;
    sv->in_use -= r->footprint;
    sv->active.erase(std::find(sv->active.begin(), sv->active.end(), r));
    sv->finished[r->ticket] = r;
    sv->stats.completed++;
    sv->done_cv.notify_all();
}

static void scheduler(tg_server* sv) {
    cudaSetDevice(sv->d->ordinal);
    for (;;) {
        bool progressed = false;
        std::vector<ServeReq*> admitted;
        uint64_t seen;
        {
            std::unique_lock<std::mutex> lock(sv->mu);
            seen = sv->completions;
            if (sv->stop && sv->queue.empty() && sv->active.empty()) return;
            // admission, first come first served: a free slot and room in the budget (a request
            // larger than the whole budget runs alone)
            while (!sv->queue.empty()) {
                ServeReq* r = sv->queue.front();
                int slot = -1;
                for (int i = 0; i < sv->max_inflight; i++)
                    if (!sv->slot_busy[i]) {
                        slot = i;
                        break;
                    }
                if (slot < 0) break;
                if (sv->in_use + r->footprint > sv->budget && !sv->active.empty()) break;
                sv->queue.pop_front();
                sv->slot_busy[slot] = 1;
                r->slot = slot;
                r->stage = 1;
                r->t_admit = Clock::now();
                sv->in_use += r->footprint;
                sv->active.push_back(r);
                sv->stats.peak_inflight = std::max<uint64_t>(sv->stats.peak_inflight, sv->active.size());
                sv->stats.peak_bytes = std::max(sv->stats.peak_bytes, sv->in_use);
                admitted.push_back(r);
            }
        }
        for (ServeReq* r : admitted) {
            const int rc = start_commit(sv, r);
            if (rc) finish(sv, r, rc);
            progressed = true;
        }
        std::vector<ServeReq*> snapshot;
        {
            std::lock_guard<std::mutex> lock(sv->mu);
            snapshot = sv->active;
        }
        for (ServeReq* r : snapshot) {
            if (r->stage == 0) continue;
            const cudaError_t e = cudaEventQuery(sv->events[r->slot]);
            if (e == cudaErrorNotReady) continue;
            progressed = true;
            if (e != cudaSuccess) {
                finish(sv, r, cuda_fail(e, "request stream"));
                continue;
            }
            if (r->stage >= 1 && r->stage <= 3)
                r->out->stage_ms[r->stage - 1] =
                    std::chrono::duration<double, std::milli>(Clock::now() - r->t_submit).count();
            if (r->stage == 1) {
                r->stage = 2;
                const int rc = start_sumcheck(sv, r);
                if (rc) finish(sv, r, rc);
            } else if (r->stage == 2 && r->req.queries) {
                r->stage = 3;
                const int rc = start_opening(sv, r);
                if (rc) finish(sv, r, rc);
            } else {
                finish(sv, r, TG_OK);
            }
        }
        if (!progressed) {
            // sleep until a stream signals the end of a stage or a request arrives (the bound is a
            // safety net only: every stage ends with a wake-up)
            std::unique_lock<std::mutex> lock(sv->mu);
            sv->wake.wait_for(lock, std::chrono::milliseconds(20), [&] {
                return sv->completions != seen || !sv->queue.empty() || sv->stop;
            });
        }
    }
}

static int check_request(const tg_proof_request& q) {
    if (q.log_inv_rate < 1 || q.log_inv_rate > 4 || q.log_k > 24)
        return fail(TG_ERR_INVALID, "unsupported shape 2^%u at rate 1/2^%u", q.log_k, q.log_inv_rate);
    if (q.row_block == 0 || q.row_block > 124) return fail(TG_ERR_INVALID, "row block %u outside 1..124", q.row_block);
    if (q.npolys && !q.rows) return fail(TG_ERR_INVALID, "null rows");
    if (q.degree < 1 || q.degree > 7) return fail(TG_ERR_INVALID, "degree %d outside 1..=7", q.degree);
    if (q.ntables < 1 || q.ntables > q.degree || !q.tables)
        return fail(TG_ERR_INVALID, "a product of %d tables at degree %d", q.ntables, q.degree);
    if (q.vars < 0 || q.vars > 30) return fail(TG_ERR_INVALID, "%d variables", q.vars);
    for (int k = 0; k < q.ntables; k++)
        if (!q.tables[k]) return fail(TG_ERR_INVALID, "table %d: null values", k);
    if (!q.prefix || strlen(q.prefix) > 150) return fail(TG_ERR_INVALID, "a prefix of at most 150 characters");
    if (q.queries && q.npolys == 0) return fail(TG_ERR_INVALID, "queries on a commitment of no rows");
    if (q.queries && answer_bytes(q.queries, q.npolys, q.log_k + q.log_inv_rate) > kSlotPinned - kSumcheckPinned)
        return fail(TG_ERR_INVALID, "an answer to %u queries over %zu rows exceeds the 1 MiB staging", q.queries,
                    q.npolys);
    return TG_OK;
}

}  // namespace tg

using namespace tg;

extern "C" int tg_server_open(tg_device* dev, size_t hbm_budget_bytes, int max_inflight, tg_server** out) {
    Device* d = reinterpret_cast<Device*>(dev);
    if (!d || !out) return fail(TG_ERR_INVALID, "tg_server_open: null argument");
    *out = nullptr;
    if (max_inflight < 1 || max_inflight > 64) return fail(TG_ERR_INVALID, "%d slots outside 1..64", max_inflight);
    if (hbm_budget_bytes == 0) return fail(TG_ERR_INVALID, "a zero HBM budget admits nothing");
    TG_CUDA(cudaSetDevice(d->ordinal));
    // Keep freed request memory in the stream-ordered pool instead of returning it to the driver.
    cudaMemPool_t pool;
    TG_CUDA(cudaDeviceGetDefaultMemPool(&pool, d->ordinal));
    uint64_t keep = UINT64_MAX;
    TG_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep));
    tg_server* sv = new tg_server();
    sv->d = d;
    sv->budget = hbm_budget_bytes;
    sv->max_inflight = max_inflight;
    memset(&sv->stats, 0, sizeof sv->stats);
    sv->streams.assign(max_inflight, nullptr);
    sv->streams_hi.assign(max_inflight, nullptr);
    sv->events.assign(max_inflight, nullptr);
    sv->slot_busy.assign(max_inflight, 0);
    int least = 0, greatest = 0;
    cudaError_t e = cudaDeviceGetStreamPriorityRange(&least, &greatest);
    if (e == cudaSuccess) e = cudaHostAlloc((void**)&sv->pinned, kSlotPinned * max_inflight, cudaHostAllocDefault);
    for (int i = 0; e == cudaSuccess && i < max_inflight; i++) {
        e = cudaStreamCreateWithPriority(&sv->streams[i], cudaStreamNonBlocking, least);
        if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&sv->streams_hi[i], cudaStreamNonBlocking, greatest);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&sv->events[i], cudaEventDisableTiming);
    }
    if (e != cudaSuccess) {
        for (int i = 0; i < max_inflight; i++) {
            if (sv->streams[i]) cudaStreamDestroy(sv->streams[i]);
            if (sv->streams_hi[i]) cudaStreamDestroy(sv->streams_hi[i]);
            if (sv->events[i]) cudaEventDestroy(sv->events[i]);
        }
        if (sv->pinned) cudaFreeHost(sv->pinned);
        delete sv;
        return cuda_fail(e, "server slots");
    }
    sv->th = std::thread(scheduler, sv);
    *out = sv;
    return TG_OK;
}

extern "C" int tg_server_submit(tg_server* sv, const tg_proof_request* req, tg_proof_result* out, uint64_t* ticket) {
    if (!sv || !req || !out || !ticket) return fail(TG_ERR_INVALID, "tg_server_submit: null argument");
    int rc = check_request(*req);
    if (rc) return rc;
    if (req->queries && (!out->query_indices || !out->columns || !out->siblings))
        return fail(TG_ERR_INVALID, "an opening round needs the result's index, column and sibling buffers");
    // the request's host buffers are read by copies soon: their pages, touched now, copy at full speed
    host_prefault(req->rows, req->npolys * ((size_t)8 << req->log_k));
    for (int k = 0; k < req->ntables; k++) host_prefault(req->tables[k], (size_t)8 << req->vars);
    ServeReq* r = new ServeReq();
    r->req = *req;
    r->table_ptrs.assign(req->tables, req->tables + req->ntables);
    r->prefix = req->prefix;
    r->req.tables = nullptr;
    r->req.prefix = nullptr;
    r->out = out;
    r->transcript = req->transcript;
    r->k = 1ull << req->log_k;
    r->n = r->k << req->log_inv_rate;
    r->group = std::max<size_t>(1, std::min<size_t>(std::max<size_t>(req->npolys, 1), kServeGroupBytes / ((r->k + r->n) * 8)));
    // the sumcheck's arena, sized by a dry run on a copy of the transcript (it also validates)
    {
        tg_transcript t = req->transcript;
        build_job(r);
        r->job.transcript = &t;
        ScRun* dry = sc_prepare(sv->d, &r->job, 1, 0, &rc);
        if (!dry) {
            delete r;
            return rc;
        }
        const size_t sc_bytes = sc_arena_bytes(dry);
        sc_free(dry);
        size_t off = align256(std::max<size_t>(req->npolys * r->k * 8, 8));
        r->off_cw = off;
        off += align256(std::max<size_t>(req->npolys * r->n * 8, 8));
        r->off_nodes = off;
        off += align256((2 * r->n - 1) * 32);
        r->off_y = off;
        off += align256(r->group * r->k * 8);
        r->off_z = off;
        off += align256(r->group * r->n * 8);
        r->off_sc = off;
        off += align256(sc_bytes);
        r->off_q = off;
        off += align256(answer_bytes(req->queries, req->npolys, req->log_k + req->log_inv_rate));
        r->footprint = off;
    }
    {
        std::lock_guard<std::mutex> lock(sv->d->mu);
        rc = sv->d->get_tables(req->log_k + req->log_inv_rate, req->log_k, &r->tables);
    }
    if (rc) {
        delete r;
        return rc;
    }
    r->t_submit = Clock::now();
    {
        std::lock_guard<std::mutex> lock(sv->mu);
        if (sv->stop) {
            delete r;
            return fail(TG_ERR_STATE, "the server is closing");
        }
        r->ticket = sv->next_ticket++;
        *ticket = r->ticket;
        sv->queue.push_back(r);
        sv->stats.submitted++;
    }
    sv->wake.notify_all();
    return TG_OK;
}

extern "C" int tg_server_wait(tg_server* sv, uint64_t ticket, int timeout_ms) {
    if (!sv) return fail(TG_ERR_INVALID, "tg_server_wait: null server");
    std::unique_lock<std::mutex> lock(sv->mu);
    auto ready = [&] { return sv->finished.count(ticket) > 0; };
    if (timeout_ms < 0)
        sv->done_cv.wait(lock, ready);
    else if (!sv->done_cv.wait_for(lock, std::chrono::milliseconds(timeout_ms), ready))
        return TG_DECLINED;
    ServeReq* r = sv->finished[ticket];
    sv->finished.erase(ticket);
    const int status = r->out->status;
    delete r;
    return status ? fail(status, "request %llu failed", (unsigned long long)ticket) : TG_OK;
}

extern "C" int tg_server_stats_read(tg_server* sv, tg_server_stats* out) {
    if (!sv || !out) return fail(TG_ERR_INVALID, "tg_server_stats_read: null argument");
    std::lock_guard<std::mutex> lock(sv->mu);
    *out = sv->stats;
    return TG_OK;
}

extern "C" int tg_server_close(tg_server* sv) {
    if (!sv) return TG_OK;
    {
        std::lock_guard<std::mutex> lock(sv->mu);
        sv->stop = true;
    }
    sv->wake.notify_all();
    sv->th.join();
    for (auto& kv : sv->finished) delete kv.second;
    for (int i = 0; i < sv->max_inflight; i++) {
        cudaStreamSynchronize(sv->streams[i]);
        cudaStreamSynchronize(sv->streams_hi[i]);
        cudaStreamDestroy(sv->streams[i]);
        cudaStreamDestroy(sv->streams_hi[i]);
        cudaEventDestroy(sv->events[i]);
    }
    cudaFreeHost(sv->pinned);
    delete sv;
    return TG_OK;
}
