// SPDX-License-Identifier: Apache-2.0 OR MIT
//
// Tree levels on the device: product forests and LogUp fraction trees, built bottom-up and proven
// level by level from the roots (RFC-0010 'Tree levels', as the reference proves them in
// crates/tessera-sumcheck/src/trees.rs: FractionTree :260-345, prove_trees :761; and LogUp's leaf
// stage, crates/tessera-logup/src/prover.rs:361).
//
// A forest of 2^s product trees of height h is stored as its stacked levels: level l holds 2^(s+l)
// entries, entry 2k and 2k + 1 of level l + 1 multiplying into entry k (a single tree is s = 0).
// A fraction tree of height h holds (n, d) per node, node x combining its children 2x (left) and
// 2x + 1 (right) into (n_L·d_R + n_R·d_L, d_L·d_R). Every level lives in HBM as Fp2 words.
//
// Level l of the schedule (H the tallest height; a tree of height h joins at level H − h):
//   - joining forests take their root points from the challenges tree/l/root/c (the last s of
//     s_max), entering with Σ_y root_y·eq(point, y); a fraction tree enters with its sent root;
//   - γ = tree/l/gamma, then λ = tree/l/lambda when a fraction tree is present;
//   - one batched degree-3 sumcheck over the present trees (tree i weighs γ^i): a forest proves
//     Σ_x eq(p, x)·L(x)·R(x), a fraction tree Σ_x eq(p, x)·(N0·D1 + N1·D0 + λ·D0·D1)(x), over the
//     halves of the level below, front-padded to the level's n_max;
//   - tree/l/evals absorbs (L, R) per forest and (N0, N1, D0, D1) per fraction tree at the end
//     point r', and with ρ = tree/l/line each tree's claim moves to the next level at ρ ‖ r'.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <memory>
#include <string>
#include <vector>

#include "internal.h"

namespace tg {

constexpr int EQ_LOW = 10;  // variables of an eq table kept in shared memory per block

__global__ void tr_product_level(const ulonglong2* below, ulonglong2* above, uint64_t m) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t x = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; x < m; x += stride) {
        const ulonglong2 a = below[2 * x], b = below[2 * x + 1];
        const fp2 p = e_mul(fp2{a.x, a.y}, fp2{b.x, b.y});
        above[x] = make_ulonglong2(p.c0, p.c1);
    }
}

__global__ void tr_fraction_level(const ulonglong2* n, const ulonglong2* d, ulonglong2* n_out, ulonglong2* d_out,
                                  uint64_t m) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t x = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; x < m; x += stride) {
        const ulonglong2 nl = n[2 * x], nr = n[2 * x + 1], dl = d[2 * x], dr = d[2 * x + 1];
        const fp2 a = {nl.x, nl.y}, b = {nr.x, nr.y}, c = {dl.x, dl.y}, e = {dr.x, dr.y};
        const fp2 nn = e_add(e_mul(a, e), e_mul(b, c)), dd = e_mul(c, e);
        n_out[x] = make_ulonglong2(nn.c0, nn.c1);
        d_out[x] = make_ulonglong2(dd.c0, dd.c1);
    }
}

// even[x] = level[2x], odd[x] = level[2x + 1] for x < m.
__global__ void tr_split(const ulonglong2* level, ulonglong2* even, ulonglong2* odd, uint64_t m) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t x = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; x < m; x += stride) {
        even[x] = level[2 * x];
        odd[x] = level[2 * x + 1];
    }
}

// The high part of an eq table: hi[y] = Π_i (bit_i(y) ? r_i : 1 − r_i) over the point's
// coordinates from EQ_LOW on (r holds those coordinates).
__global__ void tr_eq_high(const ulonglong2* r, int nh, ulonglong2* hi) {
    const uint64_t m = 1ull << nh;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t y = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; y < m; y += stride) {
        fp2 p = {1, 0};
        for (int i = 0; i < nh; i++) {
            const fp2 ri = {r[i].x, r[i].y};
            p = e_mul(p, (y >> i) & 1 ? ri : e_sub(fp2{1, 0}, ri));
        }
        hi[y] = make_ulonglong2(p.c0, p.c1);
    }
}

// eq(r, x) for x < 2^n, x_1 the lowest bit: the low EQ_LOW coordinates' table is built in shared
// memory by each block, and entry x is low[x mod 2^L]·hi[x >> L].
__global__ void tr_eq(const ulonglong2* r, int nl, const ulonglong2* hi, ulonglong2* out, uint64_t total) {
    __shared__ ulonglong2 low[1 << EQ_LOW];
    if (threadIdx.x == 0) low[0] = make_ulonglong2(1, 0);
    __syncthreads();
    for (int i = 0; i < nl; i++) {  // doubling: low[x + 2^i] = low[x]·r_i, low[x] ·= (1 − r_i)
        const fp2 ri = {r[i].x, r[i].y}, si = e_sub(fp2{1, 0}, ri);
        const int half = 1 << i;
        for (int x = threadIdx.x; x < half; x += blockDim.x) {
            const fp2 v = {low[x].x, low[x].y};
            const fp2 a = e_mul(v, si), b = e_mul(v, ri);
            low[x] = make_ulonglong2(a.c0, a.c1);
            low[x + half] = make_ulonglong2(b.c0, b.c1);
        }
        __syncthreads();
    }
    const uint64_t mask = (1ull << nl) - 1;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t x = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; x < total; x += stride) {
        const ulonglong2 a = low[x & mask];
        fp2 v = {a.x, a.y};
        if (hi) {
            const ulonglong2 h = hi[x >> nl];
            v = e_mul(v, fp2{h.x, h.y});
        }
        out[x] = make_ulonglong2(v.c0, v.c1);
    }
}

// SplitMix64 of a counter, reduced once below p: the reference benchmark's counter-based input
// generator (its counter_value, crates/tessera-gpu/src/fraction.rs:61-70).
__device__ __forceinline__ uint64_t counter_value(uint64_t c) {
    uint64_t z = c * 0x9E3779B97F4A7C15ull + 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return z >= P ? z - P : z;
}

// Generated LogUp leaves: leaf j is (n_j, α − (k_j + β·v_j)) with k_j = counter(key_seed + j),
// v_j = counter(value_seed + j), and n_j = 1 (a lookup tree) or −m_j, m_j = counter(mult_seed + j)
// mod 2^16 (a table tree).
__global__ void tr_logup_leaves(uint64_t key_seed, uint64_t value_seed, uint64_t mult_seed, int unit, fp2 alpha,
                                fp2 beta, ulonglong2* n_out, ulonglong2* d_out, uint64_t count) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; j < count; j += stride) {
        const uint64_t k = counter_value(key_seed + j), v = counter_value(value_seed + j);
        const fp2 d = {sub(sub(alpha.c0, k), mul(beta.c0, v)), sub(alpha.c1, mul(beta.c1, v))};
        d_out[j] = make_ulonglong2(d.c0, d.c1);
        uint64_t nn = 1;
        if (!unit) {
            const uint64_t m = counter_value(mult_seed + j) & 0xFFFF;
            nn = m == 0 ? 0 : P - m;
        }
        n_out[j] = make_ulonglong2(nn, 0);
    }
}

static unsigned grid_of(const Device* d, uint64_t items) {
    return (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((items + 255) / 256, (uint64_t)d->sm_count * 16));
}

struct TreeLevels {
    int kind = 0;  // 0 forest, 1 fraction
    uint32_t s = 0, h = 0;
    std::vector<std::unique_ptr<DevBuf>> n, d;  // level l, l = 0..h (fractions use both)
    fp2 sent_n = {0, 0}, sent_d = {0, 0};
    std::vector<fp2> root;  // forest: the root level; fraction: (n, d)
    int own = -1;           // the tree's level of its current claim; −1 before it joins
    std::vector<fp2> point;
    fp2 value = {0, 0}, p = {0, 0}, q = {0, 0};
};

static fp2 host_eq(const std::vector<fp2>& r, uint64_t y) {
    fp2 out = {1, 0};
    for (size_t i = 0; i < r.size(); i++) out = e_mul(out, (y >> i) & 1 ? r[i] : e_sub(fp2{1, 0}, r[i]));
    return out;
}

// p(r) for the polynomial through (k, v_k), k = 0..3 (Lagrange).
static fp2 lagrange4(const fp2 v[4], fp2 r) {
    fp2 out = {0, 0};
    for (int i = 0; i < 4; i++) {
        fp2 num = {1, 0};
        int64_t den = 1;
        for (int m = 0; m < 4; m++)
            if (m != i) {
                num = e_mul(num, e_sub(r, fp2{(uint64_t)m, 0}));
                den *= (i - m);
            }
        const uint64_t dd = den < 0 ? P - (uint64_t)(-den) : (uint64_t)den;
        out = e_add(out, e_mul(v[i], e_scale(num, inv(dd))));
    }
    return out;
}

static int challenge2(tg_transcript* t, const std::string& label, fp2* out) {
    uint64_t w[2];
    int rc = tg_transcript_challenge_fp2(t, label.c_str(), w);
    if (rc) return rc;
    *out = {w[0], w[1]};
    return TG_OK;
}

}  // namespace tg

using namespace tg;

struct tg_leaf_stage {
    Device* d = nullptr;
    std::vector<TreeLevels> trees;
    int H = 0, level = 0;
};

extern "C" int tg_leaf_stage_open(tg_device* dev, const tg_tree* specs, int ntrees, int on_device, tg_leaf_stage** out) {
    Device* d = reinterpret_cast<Device*>(dev);
    if (!d || !out || ntrees < 1 || !specs) return fail(TG_ERR_INVALID, "tg_leaf_stage_open: null argument or no tree");
    *out = nullptr;
    for (int k = 0; k < ntrees; k++) {
        const tg_tree& t = specs[k];
        if (t.kind != 0 && t.kind != 1) return fail(TG_ERR_INVALID, "tree %d: kind %d", k, t.kind);
        if (t.height > 40 || t.s > 40 || t.s + t.height > 40) return fail(TG_ERR_INVALID, "tree %d: too large", k);
        if (t.kind == 1 && t.s) return fail(TG_ERR_INVALID, "tree %d: a fraction tree stands alone (s = 0)", k);
        if (t.kind == 0 && !t.leaves) return fail(TG_ERR_INVALID, "tree %d: null leaves", k);
        if (t.kind == 1 && !t.denominators) return fail(TG_ERR_INVALID, "tree %d: null denominators", k);
    }
    tg_leaf_stage* st = new tg_leaf_stage();
    st->d = d;
    st->trees.resize(ntrees);
    cudaStream_t s = d->stream;
    auto bail = [&](int rc) {
        delete st;
        return rc;
    };
    std::lock_guard<std::mutex> lock(d->mu);
    for (int k = 0; k < ntrees; k++) {
        const tg_tree& spec = specs[k];
        TreeLevels& tr = st->trees[k];
        tr.kind = spec.kind;
        tr.s = spec.s;
        tr.h = spec.height;
        st->H = std::max<int>(st->H, (int)spec.height);
        const uint32_t lg = spec.s + spec.height;
        for (uint32_t l = 0; l <= spec.height; l++) {
            tr.n.emplace_back(new DevBuf());
            tr.d.emplace_back(new DevBuf());
        }
        const uint64_t leaves = 1ull << lg;
        const cudaMemcpyKind kind = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
        int rc = tr.n[spec.height]->ensure(leaves * 16);
        if (rc) return bail(rc);
        if (spec.kind == 0) {
            TG_CUDA(cudaMemcpyAsync(tr.n[spec.height]->ptr, spec.leaves, leaves * 16, kind, s));
        } else {
            rc = tr.d[spec.height]->ensure(leaves * 16);
            if (rc) return bail(rc);
            TG_CUDA(cudaMemcpyAsync(tr.d[spec.height]->ptr, spec.denominators, leaves * 16, kind, s));
            if (spec.leaves) {
                TG_CUDA(cudaMemcpyAsync(tr.n[spec.height]->ptr, spec.leaves, leaves * 16, kind, s));
            } else {  // numerators of 1
                std::vector<uint64_t> ones(2 * leaves, 0);
                for (uint64_t i = 0; i < leaves; i++) ones[2 * i] = 1;
                TG_CUDA(cudaMemcpyAsync(tr.n[spec.height]->ptr, ones.data(), leaves * 16, cudaMemcpyHostToDevice, s));
                TG_CUDA(cudaStreamSynchronize(s));
            }
        }
        for (int l = (int)spec.height - 1; l >= 0; l--) {
            const uint64_t m = 1ull << (spec.s + l);
            rc = tr.n[l]->ensure(m * 16);
            if (!rc && spec.kind == 1) rc = tr.d[l]->ensure(m * 16);
            if (rc) return bail(rc);
            Launch L(d, s, spec.kind ? "tree_fraction_level" : "tree_product_level", 1, m);
            if (spec.kind == 0)
                tr_product_level<<<grid_of(d, m), 256, 0, s>>>((const ulonglong2*)tr.n[l + 1]->ptr, (ulonglong2*)tr.n[l]->ptr, m);
            else
                tr_fraction_level<<<grid_of(d, m), 256, 0, s>>>((const ulonglong2*)tr.n[l + 1]->ptr,
                                                               (const ulonglong2*)tr.d[l + 1]->ptr,
                                                               (ulonglong2*)tr.n[l]->ptr, (ulonglong2*)tr.d[l]->ptr, m);
            TG_CUDA(cudaGetLastError());
        }
        // the root level on the host
        const uint64_t r = 1ull << spec.s;
        std::vector<uint64_t> w(2 * r);
        TG_CUDA(cudaMemcpyAsync(w.data(), tr.n[0]->ptr, r * 16, cudaMemcpyDeviceToHost, s));
        TG_CUDA(cudaStreamSynchronize(s));
        for (uint64_t i = 0; i < r; i++) tr.root.push_back({w[2 * i], w[2 * i + 1]});
        if (spec.kind == 1) {
            TG_CUDA(cudaMemcpy(w.data(), tr.d[0]->ptr, 16, cudaMemcpyDeviceToHost));
            tr.root.push_back({w[0], w[1]});
            tr.sent_n = tr.root[0];
            tr.sent_d = tr.root[1];
            if (spec.sent) {
                tr.sent_n = {spec.sent[0], spec.sent[1]};
                tr.sent_d = {spec.sent[2], spec.sent[3]};
            }
        }
    }
    *out = st;
    return TG_OK;
}

extern "C" int tg_leaf_stage_height(const tg_leaf_stage* st, int* height, int* level) {
    if (!st) return fail(TG_ERR_INVALID, "null leaf stage");
    if (height) *height = st->H;
    if (level) *level = st->level;
    return TG_OK;
}

extern "C" int tg_leaf_stage_root(const tg_leaf_stage* st, int tree, uint64_t* out) {
    if (!st || !out || tree < 0 || tree >= (int)st->trees.size()) return fail(TG_ERR_INVALID, "tg_leaf_stage_root: bad argument");
    const TreeLevels& tr = st->trees[tree];
    for (size_t i = 0; i < tr.root.size(); i++) {
        out[2 * i] = tr.root[i].c0;
        out[2 * i + 1] = tr.root[i].c1;
    }
    return TG_OK;
}

extern "C" int tg_leaf_stage_claim(const tg_leaf_stage* st, int tree, uint64_t* point, int* npoint, uint64_t* claim,
                                   int* own) {
    if (!st || tree < 0 || tree >= (int)st->trees.size()) return fail(TG_ERR_INVALID, "tg_leaf_stage_claim: bad argument");
    const TreeLevels& tr = st->trees[tree];
    // A tree of height 0 joins at level H, after the last level: its root, its one leaf, is its
    // leaf claim on no variable.
    const bool leaf_root = tr.own < 0 && tr.h == 0 && st->level >= st->H;
    if (leaf_root) {
        if (own) *own = 0;
        if (npoint) *npoint = 0;
        if (claim) {
            const fp2 a = tr.kind ? tr.sent_n : tr.root[0], b = tr.kind ? tr.sent_d : fp2{0, 0};
            claim[0] = a.c0, claim[1] = a.c1, claim[2] = b.c0, claim[3] = b.c1;
        }
        return TG_OK;
    }
    if (own) *own = tr.own;
    if (npoint) *npoint = (int)tr.point.size();
    if (point)
        for (size_t i = 0; i < tr.point.size(); i++) {
            point[2 * i] = tr.point[i].c0;
            point[2 * i + 1] = tr.point[i].c1;
        }
    if (claim) {
        const fp2 a = tr.kind ? tr.p : tr.value, b = tr.kind ? tr.q : fp2{0, 0};
        claim[0] = a.c0;
        claim[1] = a.c1;
        claim[2] = b.c0;
        claim[3] = b.c1;
    }
    return TG_OK;
}

extern "C" int tg_leaf_stage_prove_level(tg_leaf_stage* st, tg_transcript* t, tg_tree_level_proof* out) {
    if (!st || !t || !out) return fail(TG_ERR_INVALID, "tg_leaf_stage_prove_level: null argument");
    if (st->level >= st->H) return fail(TG_ERR_STATE, "every level is proven");
    Device* d = st->d;
    const int level = st->level;
    const std::string prefix = "tree/" + std::to_string(level);
    const int ntrees = (int)st->trees.size();
    const tg_transcript saved = *t;
    auto bail = [&](int rc) {
        *t = saved;
        return rc;
    };
    // joining trees: root challenges for the forests, then their root claims
    uint32_t s_max = 0;
    for (auto& tr : st->trees)
        if (st->H - (int)tr.h == level && tr.kind == 0) s_max = std::max(s_max, tr.s);
    std::vector<fp2> rootc(s_max);
    for (uint32_t c = 0; c < s_max; c++) {
        int rc = challenge2(t, prefix + "/root/" + std::to_string(c), &rootc[c]);
        if (rc) return bail(rc);
    }
    std::vector<TreeLevels*> joined;
    for (auto& tr : st->trees)
        if (st->H - (int)tr.h == level) joined.push_back(&tr);
    std::vector<int> present;
    for (int k = 0; k < ntrees; k++)
        if (st->trees[k].own >= 0 || st->H - (int)st->trees[k].h == level) present.push_back(k);
    // the claims the joining trees enter with (applied once the level is proven)
    std::vector<std::vector<fp2>> jpoint(ntrees);
    std::vector<fp2> jvalue(ntrees), jp(ntrees), jq(ntrees);
    for (int k : present) {
        TreeLevels& tr = st->trees[k];
        if (tr.own >= 0) {
            jpoint[k] = tr.point;
            jvalue[k] = tr.value;
            jp[k] = tr.p;
            jq[k] = tr.q;
        } else if (tr.kind == 0) {
            jpoint[k].assign(rootc.begin() + (s_max - tr.s), rootc.end());
            fp2 v = {0, 0};
            for (uint64_t y = 0; y < tr.root.size(); y++) v = e_add(v, e_mul(tr.root[y], host_eq(jpoint[k], y)));
            jvalue[k] = v;
        } else {
            jp[k] = tr.sent_n;
            jq[k] = tr.sent_d;
        }
    }
    fp2 gamma, lambda = {0, 0};
    int rc = challenge2(t, prefix + "/gamma", &gamma);
    if (rc) return bail(rc);
    bool fraction = false;
    for (int k : present) fraction |= st->trees[k].kind == 1;
    if (fraction) {
        rc = challenge2(t, prefix + "/lambda", &lambda);
        if (rc) return bail(rc);
    }

    // the level's tables on the device: an eq table and the halves of the level below per tree
    cudaStream_t s = d->stream;
    std::vector<std::unique_ptr<DevBuf>> bufs;
    auto buf = [&](size_t bytes) -> ulonglong2* {
        bufs.emplace_back(new DevBuf());
        return bufs.back()->ensure(std::max<size_t>(bytes, 16)) ? nullptr : (ulonglong2*)bufs.back()->ptr;
    };
    std::vector<tg_table> tabs;
    tabs.reserve(9 * present.size());
    std::vector<tg_instance> insts;
    std::vector<fp2> weights;
    std::vector<int> nvars;
    fp2 gi = {1, 0};
    int n_max = 0;
    {
        std::lock_guard<std::mutex> lock(d->mu);
        for (int k : present) {
            TreeLevels& tr = st->trees[k];
            const int own = tr.own >= 0 ? tr.own : 0;
            const int n = (int)jpoint[k].size();
            n_max = std::max(n_max, n);
            nvars.push_back(n);
            const uint64_t m = 1ull << n;
            // eq(point, ·)
            ulonglong2* eq = buf(m * 16);
            ulonglong2* r = buf(std::max<size_t>(n, 1) * 16);
            if (!eq || !r) return bail(fail(TG_ERR_NOMEM, "level tables"));
            std::vector<uint64_t> rw(2 * std::max(n, 1), 0);
            for (int i = 0; i < n; i++) {
                rw[2 * i] = jpoint[k][i].c0;
                rw[2 * i + 1] = jpoint[k][i].c1;
            }
            TG_CUDA(cudaMemcpyAsync(r, rw.data(), rw.size() * 8, cudaMemcpyHostToDevice, s));
            const int nl = std::min(n, EQ_LOW), nh = n - nl;
            ulonglong2* hi = nullptr;
            if (nh > 0) {
                hi = buf((1ull << nh) * 16);
                if (!hi) return bail(fail(TG_ERR_NOMEM, "level tables"));
                Launch L(d, s, "tree_eq", 1, 1ull << nh);
                tr_eq_high<<<grid_of(d, 1ull << nh), 256, 0, s>>>(r + nl, nh, hi);
            }
            {
                Launch L(d, s, "tree_eq", 1, m);
                tr_eq<<<grid_of(d, m), 256, 0, s>>>(r, nl, hi, eq, m);
            }
            TG_CUDA(cudaStreamSynchronize(s));  // rw is a host temporary
            // halves of the level below
            auto split = [&](DevBuf& lv, ulonglong2** e, ulonglong2** o) -> int {
                *e = buf(m * 16);
                *o = buf(m * 16);
                if (!*e || !*o) return fail(TG_ERR_NOMEM, "level tables");
                Launch L(d, s, "tree_split", 1, m);
                tr_split<<<grid_of(d, m), 256, 0, s>>>((const ulonglong2*)lv.ptr, *e, *o, m);
                TG_CUDA(cudaGetLastError());
                return TG_OK;
            };
            auto table = [&](const void* p, int pub) {
                tg_table tb;
                tb.values = (const uint64_t*)p;
                tb.is_ext = 1;
                tb.is_public = pub;
                tabs.push_back(tb);
            };
            auto instance = [&](fp2 w) {
                tg_instance in;
                in.tables = &tabs[tabs.size() - 3];
                in.ntables = 3;
                in.vars = n;
                insts.push_back(in);
                weights.push_back(w);
            };
            if (tr.kind == 0) {
                ulonglong2 *lt, *rt;
                rc = split(*tr.n[own + 1], &lt, &rt);
                if (rc) return bail(rc);
                table(eq, 1), table(lt, 0), table(rt, 0);
                instance(gi);
            } else {
                ulonglong2 *n0, *n1, *d0, *d1;
                rc = split(*tr.n[own + 1], &n0, &n1);
                if (!rc) rc = split(*tr.d[own + 1], &d0, &d1);
                if (rc) return bail(rc);
                table(eq, 1), table(n0, 0), table(d1, 0);
                instance(gi);
                table(eq, 1), table(n1, 0), table(d0, 0);
                instance(gi);
                table(eq, 1), table(d0, 0), table(d1, 0);
                instance(e_mul(gi, lambda));
            }
            gi = e_mul(gi, gamma);
        }
    }

    // the batched level sumcheck (γ and λ already drawn; the evaluations absorbed below)
    std::vector<uint64_t> rounds((size_t)std::max(n_max, 1) * 6), chal((size_t)std::max(n_max, 1) * 2),
        fevals(insts.size() * 4);
    tg_sumcheck_job jb;
    memset(&jb, 0, sizeof jb);
    jb.transcript = t;
    jb.prefix = prefix.c_str();
    jb.degree = 3;
    jb.instances = insts.data();
    jb.ninstances = (int)insts.size();
    jb.gamma[0] = gamma.c0;
    jb.gamma[1] = gamma.c1;
    jb.rounds = rounds.data();
    jb.challenges = chal.data();
    jb.final_evals = fevals.data();
    ScOptions opts;
    opts.weights = &weights;
    opts.absorb_evals = false;
    rc = prove_many_opts(d, &jb, 1, 1, opts);
    if (rc) return bail(rc);

    // the evaluations: (L, R) per forest, (N0, N1, D0, D1) per fraction tree
    std::vector<fp2> evals;
    auto fe = [&](size_t inst, int which) { return fp2{fevals[4 * inst + 2 * which], fevals[4 * inst + 2 * which + 1]}; };
    size_t ii = 0;
    for (int k : present) {
        if (st->trees[k].kind == 0) {
            evals.push_back(fe(ii, 0));
            evals.push_back(fe(ii, 1));
            ii += 1;
        } else {
            evals.push_back(fe(ii, 0));      // N0 (instance 0: eq, n0, d1)
            evals.push_back(fe(ii + 1, 0));  // N1 (instance 1: eq, n1, d0)
            evals.push_back(fe(ii + 1, 1));  // D0
            evals.push_back(fe(ii, 1));      // D1
            ii += 3;
        }
    }
    std::vector<uint64_t> ew(2 * evals.size());
    for (size_t i = 0; i < evals.size(); i++) {
        ew[2 * i] = evals[i].c0;
        ew[2 * i + 1] = evals[i].c1;
    }
    rc = tg_transcript_absorb_fp2s(t, (prefix + "/evals").c_str(), ew.data(), evals.size());
    if (rc) return bail(rc);
    fp2 rho;
    rc = challenge2(t, prefix + "/line", &rho);
    if (rc) return bail(rc);

    // the claims as the verifier derives them: claim_0 = Σ γ^i 2^(n_max − n_i) held_i, then
    // claim_{j+1} = p_j(r_j) with p_j(1) = claim_j − p_j(0)
    std::vector<fp2> claims;
    {
        fp2 c = {0, 0}, g = {1, 0};
        size_t i = 0;
        for (int k : present) {
            const TreeLevels& tr = st->trees[k];
            const fp2 held = tr.kind == 0 ? jvalue[k] : e_add(jp[k], e_mul(lambda, jq[k]));
            c = e_add(c, e_mul(g, e_scale(held, (1ull << (n_max - nvars[i])) % P)));
            g = e_mul(g, gamma);
            i++;
        }
        claims.push_back(c);
        for (int j = 0; j < n_max; j++) {
            const fp2 m0 = {rounds[6 * j], rounds[6 * j + 1]};
            const fp2 v[4] = {m0, e_sub(claims.back(), m0), {rounds[6 * j + 2], rounds[6 * j + 3]},
                              {rounds[6 * j + 4], rounds[6 * j + 5]}};
            claims.push_back(lagrange4(v, {chal[2 * j], chal[2 * j + 1]}));
        }
    }

    // the next claims: ρ ‖ r' on the level below
    size_t cur = 0, pi = 0;
    for (int k : present) {
        TreeLevels& tr = st->trees[k];
        const int n = nvars[pi++];
        std::vector<fp2> pt;
        pt.push_back(rho);
        for (int j = n_max - n; j < n_max; j++) pt.push_back({chal[2 * j], chal[2 * j + 1]});
        const int own = tr.own >= 0 ? tr.own : 0;
        if (tr.kind == 0) {
            const fp2 u = evals[cur], w = evals[cur + 1];
            cur += 2;
            tr.value = e_add(u, e_mul(rho, e_sub(w, u)));
        } else {
            const fp2 N0 = evals[cur], N1 = evals[cur + 1], D0 = evals[cur + 2], D1 = evals[cur + 3];
            cur += 4;
            tr.p = e_add(N0, e_mul(rho, e_sub(N1, N0)));
            tr.q = e_add(D0, e_mul(rho, e_sub(D1, D0)));
        }
        tr.point = pt;
        tr.own = own + 1;
        tr.n[own]->release();  // the level above is no longer needed
        tr.d[own]->release();
    }
    st->level++;

    // the record
    out->level = level;
    out->n_root_challenges = (int)s_max;
    if (out->root_challenges)
        for (uint32_t c = 0; c < s_max; c++) {
            out->root_challenges[2 * c] = rootc[c].c0;
            out->root_challenges[2 * c + 1] = rootc[c].c1;
        }
    out->gamma[0] = gamma.c0;
    out->gamma[1] = gamma.c1;
    out->has_lambda = fraction;
    out->lambda[0] = lambda.c0;
    out->lambda[1] = lambda.c1;
    out->n_max = n_max;
    if (out->rounds) memcpy(out->rounds, rounds.data(), (size_t)n_max * 48);
    if (out->challenges) memcpy(out->challenges, chal.data(), (size_t)n_max * 16);
    if (out->claims)
        for (size_t i = 0; i < claims.size(); i++) {
            out->claims[2 * i] = claims[i].c0;
            out->claims[2 * i + 1] = claims[i].c1;
        }
    out->n_evals = (int)evals.size();
    if (out->evals) memcpy(out->evals, ew.data(), ew.size() * 8);
    out->rho[0] = rho.c0;
    out->rho[1] = rho.c1;
    out->n_present = (int)present.size();
    if (out->present)
        for (size_t i = 0; i < present.size(); i++) out->present[i] = present[i];
    return TG_OK;
}

extern "C" int tg_leaf_stage_close(tg_leaf_stage* st) {
    if (!st) return TG_OK;
    cudaStream_t s = st->d->stream;
    for (auto& tr : st->trees)  // secret-class levels are zeroed before release
        for (auto* v : {&tr.n, &tr.d})
            for (auto& b : *v)
                if (b->ptr) cudaMemsetAsync(b->ptr, 0, b->bytes, s);
    cudaStreamSynchronize(s);
    delete st;
    return TG_OK;
}

extern "C" int tg_logup_leaves(tg_device* dev, uint64_t key_seed, uint64_t value_seed, int unit, uint64_t mult_seed,
                               const uint64_t alpha[2], const uint64_t beta[2], size_t count, uint64_t* numerators,
                               uint64_t* denominators) {
    Device* d = reinterpret_cast<Device*>(dev);
    if (!d || !alpha || !beta || (count && (!numerators || !denominators)))
        return fail(TG_ERR_INVALID, "tg_logup_leaves: null argument");
    if (count == 0) return TG_OK;
    cudaStream_t s = d->stream;
    {
        Launch L(d, s, "logup_leaves", 1, count);
        tr_logup_leaves<<<grid_of(d, count), 256, 0, s>>>(key_seed, value_seed, mult_seed, unit, fp2{alpha[0], alpha[1]},
                                                          fp2{beta[0], beta[1]}, (ulonglong2*)numerators,
                                                          (ulonglong2*)denominators, count);
    }
    TG_CUDA(cudaGetLastError());
    TG_CUDA(cudaStreamSynchronize(s));
    return TG_OK;
}
