// SPDX-License-Identifier: Apache-2.0 OR MIT
//
// Many unmasked commitments of uneven shapes at once (the batched pattern beside the plain
// per-commitment path, each commitment being the reference's commit_unmasked,
// crates/tessera-pcs/src/commitment.rs:343-458). The commitments are spread over W worker streams
// by longest-processing-time first (the biggest estimated cost goes to the least loaded stream),
// each worker with its own encoder scratch, so that small commitments — whose column chains and
// Merkle levels are too narrow to fill 152 SMs — run beside each other and beside the big ones.
//
// A plan captures the whole batch (fork from the device stream, the workers' encoders, chains,
// trees and root copies, join) into one CUDA graph and replays it: one graph launch instead of
// dozens of kernel launches per commitment. Creating a plan autotunes in two steps, on the batch
// itself:
//   1. per encoder shape (k, rate, rows) of the register-resident encoder: the split of the row
//      transform k = K1·K2 (which sets the tile shapes of the four passes: 2^13 / L columns of
//      length L = K1 or K2 per CTA) and the rows per group (the default, or few enough rows that
//      a group's scratch stays in L2 between passes), each candidate timed on the first job of
//      that shape; results can be kept in a cache file (TESSERA_GB300_TUNE_CACHE) and read back
//      by later plans on a GPU with the same SM count;
//   2. the worker count W over {1, 2, 4, 8}, by timing a replay of each candidate graph.
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <memory>
#include <vector>

#include "internal.h"

struct tg_commit_plan {
    tg::Device* d = nullptr;
    std::vector<tg_commit_job> jobs;
    std::vector<tg_encode_tuning> shapes;  // the encoder configuration chosen per shape
    cudaGraphExec_t exec = nullptr;
    int workers = 0;
    uint64_t kernels = 0;  // kernel launches one replay performs
    double tuned_ms[4] = {0, 0, 0, 0};  // a replay's time at W = 1, 2, 4, 8 (0: not tried)
    tg::DevBuf roots;
    std::vector<std::unique_ptr<tg::DevBuf>> scratch;  // the graph's encoder scratch, y and z per worker
};

namespace tg {

struct CommitWork {
    int index = 0;
    uint32_t lgk = 0, lgr = 0, block = 0;
    uint64_t n = 0;
    size_t npolys = 0, group = 0;
    int lgk1 = 0;  // the encoder's split (0: default)
    const Tables* t = nullptr;
    double cost = 0;
    int worker = 0;
};

static int check_commit_job(const tg_commit_job& j, int i) {
    if (j.log_inv_rate < 1 || j.log_inv_rate > 4 || j.log_k > 24)
        return fail(TG_ERR_INVALID, "job %d: unsupported shape 2^%u at rate 1/2^%u", i, j.log_k, j.log_inv_rate);
    if (j.row_block == 0 || j.row_block > 124) return fail(TG_ERR_INVALID, "job %d: row block %u outside 1..124", i, j.row_block);
    if (!j.nodes || (j.npolys && (!j.rows || !j.codewords))) return fail(TG_ERR_INVALID, "job %d: null buffer", i);
    return TG_OK;
}

static size_t default_group(Device* d, uint32_t lgk, uint32_t lgr, size_t npolys) {
    const size_t k = (size_t)1 << lgk, n = k << lgr;
    return std::min<size_t>(std::max<size_t>(1, d->cfg.lde_group_bytes / ((k + n) * 8)), std::max<size_t>(npolys, 1));
}

static const tg_encode_tuning* find_shape(const std::vector<tg_encode_tuning>& shapes, uint32_t lgk, uint32_t lgr,
                                          size_t npolys) {
    for (const auto& t : shapes)
        if (t.log_k == lgk && t.log_inv_rate == lgr && t.npolys == npolys) return &t;
    return nullptr;
}

// Resolves the jobs (tables built, group sizes and splits — tuned where `shapes` has the job's
// shape —, costs), assigns them to `nworkers` streams and returns each worker's encoder scratch
// in bytes (y, z).
static int plan_work(Device* d, const tg_commit_job* jobs, int njobs, int nworkers, std::vector<CommitWork>& work,
                     std::vector<size_t>& ybytes, std::vector<size_t>& zbytes,
                     const std::vector<tg_encode_tuning>* shapes = nullptr) {
    work.clear();
    for (int i = 0; i < njobs; i++) {
        const tg_commit_job& j = jobs[i];
        CommitWork w;
        w.index = i;
        w.lgk = j.log_k;
        w.lgr = j.log_inv_rate;
        w.block = j.row_block;
        w.n = 1ull << (j.log_k + j.log_inv_rate);
        w.npolys = j.npolys;
        w.group = default_group(d, w.lgk, w.lgr, j.npolys);
        if (shapes)
            if (const tg_encode_tuning* t = find_shape(*shapes, w.lgk, w.lgr, j.npolys)) {
                w.group = (size_t)t->group;
                w.lgk1 = t->split_log;
            }
        int rc = d->get_tables(w.lgk + w.lgr, w.lgk, &w.t);
        if (rc) return rc;
        // the encoder's butterflies per symbol grow with log n; one chain step per block per column
        w.cost = (double)j.npolys * (double)w.n * (w.lgk + w.lgr) + (double)w.n * 40.0 * ((j.npolys + w.block - 1) / w.block + 1);
        work.push_back(w);
    }
    std::vector<size_t> order(work.size());
    for (size_t i = 0; i < order.size(); i++) order[i] = i;
    std::sort(order.begin(), order.end(), [&](size_t a, size_t b) { return work[a].cost > work[b].cost; });
    std::vector<double> load(nworkers, 0.0);
    for (size_t i : order) {
        const int w = (int)(std::min_element(load.begin(), load.end()) - load.begin());
        work[i].worker = w;
        load[w] += work[i].cost;
    }
    // workers and their scratch
    while ((int)d->workers.size() < nworkers) {
        Worker* w = new Worker();
        cudaError_t e = cudaStreamCreateWithFlags(&w->s, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&w->done, cudaEventDisableTiming);
        if (e != cudaSuccess) {
            if (w->s) cudaStreamDestroy(w->s);
            delete w;
            return cuda_fail(e, "worker stream");
        }
        d->workers.push_back(w);
    }
    if (!d->fork) TG_CUDA(cudaEventCreateWithFlags(&d->fork, cudaEventDisableTiming));
    ybytes.assign(nworkers, 8);
    zbytes.assign(nworkers, 8);
    for (auto& w : work)
        if (w.npolys) {
            ybytes[w.worker] = std::max(ybytes[w.worker], w.group * ((size_t)1 << w.lgk) * 8);
            zbytes[w.worker] = std::max(zbytes[w.worker], w.group * w.n * 8);
        }
    return TG_OK;
}

// Enqueues the batch: fork from the device stream, each worker's commitments in turn (encode,
// chains, tree, root into roots[i]), join back into the device stream.
static int enqueue(Device* d, const tg_commit_job* jobs, const std::vector<CommitWork>& work, int nworkers,
                   uint8_t* roots, const std::vector<uint64_t*>& ys, const std::vector<uint64_t*>& zs) {
    cudaStream_t s = d->stream;
    TG_CUDA(cudaEventRecord(d->fork, s));
    for (int wi = 0; wi < nworkers; wi++) TG_CUDA(cudaStreamWaitEvent(d->workers[wi]->s, d->fork, 0));
    for (int wi = 0; wi < nworkers; wi++) {
        Worker* wk = d->workers[wi];
        for (const CommitWork& w : work) {
            if (w.worker != wi) continue;
            const tg_commit_job& j = jobs[w.index];
            int rc = lde_encode_into(d, w.lgk, w.lgr, 0, j.rows, w.npolys, nullptr, j.codewords, wk->s, w.t->pw,
                                     w.t->pow7k, false, ys[wi], zs[wi], w.group, w.lgk1);
            if (!rc) rc = column_init(d, j.commitment_id, w.n, j.nodes, wk->s);
            if (!rc) rc = column_absorb(d, j.nodes, w.n, j.codewords, w.n, w.npolys, w.block, wk->s);
            if (!rc) rc = merkle_tree(d, j.nodes, w.n, j.nodes, wk->s);
            if (rc) return rc;
            TG_CUDA(cudaMemcpyAsync(roots + 32 * (size_t)w.index, j.nodes + 32 * (2 * w.n - 2), 32,
                                    cudaMemcpyDeviceToDevice, wk->s));
        }
        TG_CUDA(cudaEventRecord(wk->done, wk->s));
        TG_CUDA(cudaStreamWaitEvent(s, wk->done, 0));
    }
    return TG_OK;
}

static int default_workers(int njobs) { return std::max(1, std::min(4, njobs)); }

// ---- the encoder autotuner -----------------------------------------------------------------------

static const char* cache_path() {
    const char* p = getenv("TESSERA_GB300_TUNE_CACHE");
    return p && *p ? p : nullptr;
}

// The cache file holds one line per shape (the last line of a shape wins):
//   encode <SM count> <log2 k> <log2 inverse rate> <rows> <log2 K1> <rows per group> <ms default> <ms tuned>
static void cache_read(Device* d, std::vector<tg_encode_tuning>& out) {
    const char* path = cache_path();
    if (!path) return;
    FILE* f = fopen(path, "r");
    if (!f) return;
    char line[256];
    while (fgets(line, sizeof line, f)) {
        int sm = 0, split = 0;
        unsigned lgk = 0, lgr = 0;
        unsigned long long np = 0, group = 0;
        double md = 0, mb = 0;
        if (sscanf(line, "encode %d %u %u %llu %d %llu %lf %lf", &sm, &lgk, &lgr, &np, &split, &group, &md, &mb) != 8)
            continue;
        if (sm != d->sm_count || lgr < 1 || lgr > 4 || np == 0 || group == 0 || group > np || group > 65535 ||
            !encode_split_valid(lgk, split))
            continue;
        tg_encode_tuning t;
        memset(&t, 0, sizeof t);
        t.log_k = lgk;
        t.log_inv_rate = lgr;
        t.npolys = np;
        t.split_log = split;
        t.group = group;
        t.ms_default = md;
        t.ms_tuned = mb;
        t.from_cache = 1;
        bool replaced = false;
        for (auto& o : out)
            if (o.log_k == lgk && o.log_inv_rate == lgr && o.npolys == np) {
                o = t;
                replaced = true;
            }
        if (!replaced) out.push_back(t);
    }
    fclose(f);
}

static void cache_append(Device* d, const std::vector<tg_encode_tuning>& fresh) {
    const char* path = cache_path();
    if (!path || fresh.empty()) return;
    FILE* f = fopen(path, "a");
    if (!f) return;
    for (const auto& t : fresh)
        fprintf(f, "encode %d %u %u %llu %d %llu %.4f %.4f\n", d->sm_count, t.log_k, t.log_inv_rate,
                (unsigned long long)t.npolys, t.split_log, (unsigned long long)t.group, t.ms_default, t.ms_tuned);
    fclose(f);
}

// One encode of job j with (split, group) on the device stream: a warm-up, then the faster of two
// timed runs.
static int time_encode(Device* d, const tg_commit_job& j, const Tables* t, int split, size_t group, uint64_t* y,
                       uint64_t* z, cudaEvent_t e0, cudaEvent_t e1, double* ms) {
    cudaStream_t s = d->stream;
    double best = -1;
    for (int rep = 0; rep < 3; rep++) {
        if (rep) TG_CUDA(cudaEventRecord(e0, s));
        int rc = lde_encode_into(d, j.log_k, j.log_inv_rate, 0, j.rows, j.npolys, nullptr, j.codewords, s, t->pw,
                                 t->pow7k, false, y, z, group, split);
        if (rc) return rc;
        if (!rep) continue;
        TG_CUDA(cudaEventRecord(e1, s));
        TG_CUDA(cudaEventSynchronize(e1));
        float m = 0;
        TG_CUDA(cudaEventElapsedTime(&m, e0, e1));
        if (best < 0 || m < best) best = m;
    }
    *ms = best;
    return TG_OK;
}

// Step 1 of plan creation: the encoder configuration of every shape of the register-resident
// encoder among the jobs, from the cache or by timing the candidates on the first job of the shape.
static int tune_shapes(Device* d, tg_commit_plan* p) {
    std::vector<tg_encode_tuning> cached, fresh;
    cache_read(d, cached);
    int l2 = 0;
    TG_CUDA(cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, d->ordinal));
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    TG_CUDA(cudaEventCreate(&e0));
    cudaError_t ce = cudaEventCreate(&e1);
    if (ce != cudaSuccess) {
        cudaEventDestroy(e0);
        return cuda_fail(ce, "cudaEventCreate");
    }
    DevBuf y, z;
    int rc = TG_OK;
    for (const tg_commit_job& j : p->jobs) {
        const int c0 = (int)(j.log_k + 1) / 2;
        if (j.npolys == 0 || !encode_split_valid(j.log_k, c0)) continue;
        if (find_shape(p->shapes, j.log_k, j.log_inv_rate, j.npolys)) continue;
        if (const tg_encode_tuning* c = find_shape(cached, j.log_k, j.log_inv_rate, j.npolys)) {
            p->shapes.push_back(*c);
            continue;
        }
        const size_t k = (size_t)1 << j.log_k, n = k << j.log_inv_rate;
        const size_t gd = default_group(d, j.log_k, j.log_inv_rate, j.npolys);
        // rows whose scratch (k + n words each) fits in three quarters of L2
        const size_t gl = std::max<size_t>(1, (size_t)l2 * 3 / 4 / ((k + n) * 8));
        std::vector<int> splits = {c0};
        for (int c : {c0 - 1, c0 + 1})
            if (encode_split_valid(j.log_k, c)) splits.push_back(c);
        std::vector<size_t> groups = {gd};
        if (gl < gd) groups.push_back(gl);
        rc = y.ensure(gd * k * 8);
        if (!rc) rc = z.ensure(gd * n * 8);
        if (rc) break;
        const Tables* t = nullptr;
        rc = d->get_tables(j.log_k + j.log_inv_rate, j.log_k, &t);
        if (rc) break;
        tg_encode_tuning best;
        memset(&best, 0, sizeof best);
        best.log_k = j.log_k;
        best.log_inv_rate = j.log_inv_rate;
        best.npolys = j.npolys;
        best.ms_tuned = -1;
        for (int c : splits) {
            for (size_t g : groups) {
                double ms = 0;
                rc = time_encode(d, j, t, c, g, (uint64_t*)y.ptr, (uint64_t*)z.ptr, e0, e1, &ms);
                if (rc) break;
                best.candidates++;
                if (c == c0 && g == gd) best.ms_default = ms;
                if (best.ms_tuned < 0 || ms < best.ms_tuned) {
                    best.ms_tuned = ms;
                    best.split_log = c;
                    best.group = g;
                }
            }
            if (rc) break;
        }
        if (rc) break;
        fresh.push_back(best);
        p->shapes.push_back(best);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (!rc) {
        TG_CUDA(cudaStreamSynchronize(d->stream));  // the scratch is freed on return
        cache_append(d, fresh);
    }
    return rc;
}

}  // namespace tg

using namespace tg;

extern "C" int tg_commit_many(tg_device* dev, tg_commit_job* jobs, int njobs, int workers) {
    Device* d = reinterpret_cast<Device*>(dev);
    if (!d || (njobs && !jobs)) return fail(TG_ERR_INVALID, "tg_commit_many: null argument");
    if (njobs <= 0) return TG_OK;
    if (workers < 0 || workers > 16) return fail(TG_ERR_INVALID, "%d workers outside 0..16", workers);
    for (int i = 0; i < njobs; i++) {
        int rc = check_commit_job(jobs[i], i);
        if (rc) return rc;
    }
    const int nw = workers ? std::min(workers, njobs) : default_workers(njobs);
    std::lock_guard<std::mutex> lock(d->mu);
    std::vector<CommitWork> work;
    std::vector<size_t> yb, zb;
    int rc = plan_work(d, jobs, njobs, nw, work, yb, zb);
    if (rc) return rc;
    std::vector<uint64_t*> ys(nw), zs(nw);
    for (int wi = 0; wi < nw; wi++) {
        rc = d->workers[wi]->y.ensure(yb[wi]);
        if (!rc) rc = d->workers[wi]->z.ensure(zb[wi]);
        if (rc) return rc;
        ys[wi] = (uint64_t*)d->workers[wi]->y.ptr;
        zs[wi] = (uint64_t*)d->workers[wi]->z.ptr;
    }
    rc = d->batch_roots.ensure((size_t)njobs * 32);
    if (rc) return rc;
    rc = enqueue(d, jobs, work, nw, (uint8_t*)d->batch_roots.ptr, ys, zs);
    if (rc) return rc;
    std::vector<uint8_t> roots((size_t)njobs * 32);
    TG_CUDA(cudaMemcpyAsync(roots.data(), d->batch_roots.ptr, roots.size(), cudaMemcpyDeviceToHost, d->stream));
    TG_CUDA(cudaStreamSynchronize(d->stream));
    for (int i = 0; i < njobs; i++) memcpy(jobs[i].root, roots.data() + 32 * (size_t)i, 32);
    return TG_OK;
}

// Captures the batch with `nw` workers into an executable graph over its own scratch.
static int capture(Device* d, tg_commit_plan* p, int nw, cudaGraphExec_t* exec, uint64_t* kernels,
                   std::vector<std::unique_ptr<DevBuf>>& scratch) {
    std::vector<CommitWork> work;
    std::vector<size_t> yb, zb;
    int rc = plan_work(d, p->jobs.data(), (int)p->jobs.size(), nw, work, yb, zb, &p->shapes);
    if (rc) return rc;
    scratch.clear();
    std::vector<uint64_t*> ys(nw), zs(nw);
    for (int wi = 0; wi < nw; wi++) {
        scratch.emplace_back(new DevBuf());
        scratch.emplace_back(new DevBuf());
        rc = scratch[2 * wi]->ensure(yb[wi]);
        if (!rc) rc = scratch[2 * wi + 1]->ensure(zb[wi]);
        if (rc) return rc;
        ys[wi] = (uint64_t*)scratch[2 * wi]->ptr;
        zs[wi] = (uint64_t*)scratch[2 * wi + 1]->ptr;
    }
    TG_CUDA(cudaStreamBeginCapture(d->stream, cudaStreamCaptureModeThreadLocal));
    d->capturing = true;
    d->captured = 0;
    rc = enqueue(d, p->jobs.data(), work, nw, (uint8_t*)p->roots.ptr, ys, zs);
    d->capturing = false;
    cudaGraph_t graph = nullptr;
    const cudaError_t e = cudaStreamEndCapture(d->stream, &graph);
    if (rc) {
        if (graph) cudaGraphDestroy(graph);
        return rc;
    }
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
    const cudaError_t e2 = cudaGraphInstantiate(exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e2 != cudaSuccess) return cuda_fail(e2, "cudaGraphInstantiate");
    *kernels = d->captured;
    return TG_OK;
}

extern "C" int tg_commit_plan_create(tg_device* dev, const tg_commit_job* jobs, int njobs, int workers,
                                     tg_commit_plan** out) {
    Device* d = reinterpret_cast<Device*>(dev);
    if (!d || !out || (njobs && !jobs)) return fail(TG_ERR_INVALID, "tg_commit_plan_create: null argument");
    *out = nullptr;
    if (njobs <= 0) return fail(TG_ERR_INVALID, "a plan needs at least one commitment");
    if (workers < 0 || workers > 16) return fail(TG_ERR_INVALID, "%d workers outside 0..16", workers);
    for (int i = 0; i < njobs; i++) {
        int rc = check_commit_job(jobs[i], i);
        if (rc) return rc;
    }
    std::lock_guard<std::mutex> lock(d->mu);
    tg_commit_plan* p = new tg_commit_plan();
    p->d = d;
    p->jobs.assign(jobs, jobs + njobs);
    int rc = p->roots.ensure((size_t)njobs * 32);
    if (rc) {
        delete p;
        return rc;
    }
    rc = tune_shapes(d, p);
    if (rc) {
        delete p;
        return rc;
    }
    std::vector<int> cands;
    if (workers)
        cands.push_back(std::min(workers, njobs));
    else
        for (int w : {1, 2, 4, 8})
            if (w <= njobs) cands.push_back(w);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    TG_CUDA(cudaEventCreate(&e0));
    TG_CUDA(cudaEventCreate(&e1));
    double best = -1;
    for (int w : cands) {
        cudaGraphExec_t exec = nullptr;
        uint64_t kernels = 0;
        std::vector<std::unique_ptr<DevBuf>> scratch;
        rc = capture(d, p, w, &exec, &kernels, scratch);
        if (rc) break;
        if (cands.size() > 1) {  // autotune: warm replay, then one timed replay
            cudaError_t e = cudaGraphLaunch(exec, d->stream);
            if (e == cudaSuccess) e = cudaEventRecord(e0, d->stream);
            if (e == cudaSuccess) e = cudaGraphLaunch(exec, d->stream);
            if (e == cudaSuccess) e = cudaEventRecord(e1, d->stream);
            if (e == cudaSuccess) e = cudaEventSynchronize(e1);
            float ms = 0;
            if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
            if (e != cudaSuccess) {
                cudaGraphExecDestroy(exec);
                rc = cuda_fail(e, "autotune replay");
                break;
            }
            d->launches += 2 * kernels;
            const int slot = w == 1 ? 0 : w == 2 ? 1 : w == 4 ? 2 : 3;
            p->tuned_ms[slot] = ms;
            if (best >= 0 && ms >= best) {
                cudaGraphExecDestroy(exec);
                continue;
            }
            best = ms;
        }
        if (p->exec) cudaGraphExecDestroy(p->exec);
        p->exec = exec;
        p->workers = w;
        p->kernels = kernels;
        p->scratch.swap(scratch);  // the replaced candidate's scratch is freed with `scratch`
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) {
        if (p->exec) cudaGraphExecDestroy(p->exec);
        delete p;
        return rc;
    }
    *out = p;
    return TG_OK;
}

extern "C" int tg_commit_plan_launch(tg_commit_plan* p, uint8_t* roots) {
    if (!p || !roots) return fail(TG_ERR_INVALID, "tg_commit_plan_launch: null argument");
    Device* d = p->d;
    std::lock_guard<std::mutex> lock(d->mu);
    TG_CUDA(cudaGraphLaunch(p->exec, d->stream));
    d->launches += p->kernels;
    TG_CUDA(cudaMemcpyAsync(roots, p->roots.ptr, p->jobs.size() * 32, cudaMemcpyDeviceToHost, d->stream));
    TG_CUDA(cudaStreamSynchronize(d->stream));
    return TG_OK;
}

extern "C" int tg_commit_plan_info(const tg_commit_plan* p, int* workers, uint64_t* kernels, double tuned_ms[4]) {
    if (!p) return fail(TG_ERR_INVALID, "tg_commit_plan_info: null plan");
    if (workers) *workers = p->workers;
    if (kernels) *kernels = p->kernels;
    if (tuned_ms) memcpy(tuned_ms, p->tuned_ms, sizeof p->tuned_ms);
    return TG_OK;
}

extern "C" int tg_commit_plan_tuning(const tg_commit_plan* p, tg_encode_tuning* out, int cap, int* count) {
    if (!p || !count || (cap > 0 && !out)) return fail(TG_ERR_INVALID, "tg_commit_plan_tuning: null argument");
    *count = (int)p->shapes.size();
    for (int i = 0; i < cap && i < (int)p->shapes.size(); i++) out[i] = p->shapes[i];
    return TG_OK;
}

extern "C" int tg_commit_plan_destroy(tg_commit_plan* p) {
    if (!p) return TG_OK;
    {
        std::lock_guard<std::mutex> lock(p->d->mu);
        cudaStreamSynchronize(p->d->stream);
        if (p->exec) cudaGraphExecDestroy(p->exec);
    }
    delete p;
    return TG_OK;
}
