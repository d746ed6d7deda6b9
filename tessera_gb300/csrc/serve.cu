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
//   3. the host finishes the proof (transcript, round messages, evaluations), frees the request's
//      device memory on its stream and hands the result to the waiting caller
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
    size_t group = 0, off_cw = 0, off_nodes = 0, off_y = 0, off_z = 0, off_sc = 0, footprint = 0;
    uint8_t* dmem = nullptr;
    int slot = -1, stage = 0, status = TG_OK;
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
    std::vector<cudaStream_t> streams;
    std::vector<cudaEvent_t> events;
    std::vector<int> slot_busy;
    uint8_t* pinned = nullptr;  // kSlotPinned bytes per slot
    size_t in_use = 0;
    tg_server_stats stats;
};

namespace tg {

constexpr size_t kSlotPinned = 64 << 10;
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

// Stage 1: rows in, encode, chains, tree, root out; on the slot's stream.
static int start_commit(tg_server* sv, ServeReq* r) {
    Device* d = sv->d;
    cudaStream_t s = sv->streams[r->slot];
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
    TG_CUDA(cudaEventRecord(sv->events[r->slot], s));
    return TG_OK;
}

// Stage 2: the root into the transcript, γ, and the sumcheck on the device.
static int start_sumcheck(tg_server* sv, ServeReq* r) {
    Device* d = sv->d;
    cudaStream_t s = sv->streams[r->slot];
    uint8_t* pin = sv->pinned + kSlotPinned * r->slot;
    memcpy(r->out->root, pin, 32);
    int rc = tg_transcript_absorb(&r->transcript, (r->prefix + "/root").c_str(), r->out->root, 32);
    if (rc) return rc;
    build_job(r);
    r->run = sc_prepare(d, &r->job, 1, 0, &rc);
    if (!r->run) return rc;
    if (sc_host_bytes(r->run) + 32 > kSlotPinned) return fail(TG_ERR_INVALID, "sumcheck outputs exceed the slot's staging");
    {
        std::lock_guard<std::mutex> lock(d->mu);
        rc = sc_enqueue(d, r->run, s, r->dmem + r->off_sc, pin + 32);
    }
    if (rc) return rc;
    TG_CUDA(cudaEventRecord(sv->events[r->slot], s));
    return TG_OK;
}

// Stage 3: the proof's outputs, memory back to the pool, the slot freed.
static void finish(tg_server* sv, ServeReq* r, int status) {
    cudaStream_t s = sv->streams[r->slot];
    if (!status && r->run) status = sc_finish(r->run);
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
        {
            std::unique_lock<std::mutex> lock(sv->mu);
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
            if (r->stage == 1) {
                r->stage = 2;
                const int rc = start_sumcheck(sv, r);
                if (rc) finish(sv, r, rc);
            } else {
                finish(sv, r, TG_OK);
            }
        }
        if (!progressed) {
            std::unique_lock<std::mutex> lock(sv->mu);
            sv->wake.wait_for(lock, std::chrono::microseconds(50));
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
    sv->events.assign(max_inflight, nullptr);
    sv->slot_busy.assign(max_inflight, 0);
    cudaError_t e = cudaHostAlloc((void**)&sv->pinned, kSlotPinned * max_inflight, cudaHostAllocDefault);
    for (int i = 0; e == cudaSuccess && i < max_inflight; i++) {
        e = cudaStreamCreateWithFlags(&sv->streams[i], cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&sv->events[i], cudaEventDisableTiming);
    }
    if (e != cudaSuccess) {
        for (int i = 0; i < max_inflight; i++) {
            if (sv->streams[i]) cudaStreamDestroy(sv->streams[i]);
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
        cudaStreamDestroy(sv->streams[i]);
        cudaEventDestroy(sv->events[i]);
    }
    cudaFreeHost(sv->pinned);
    delete sv;
    return TG_OK;
}
