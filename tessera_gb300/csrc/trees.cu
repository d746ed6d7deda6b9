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

#include "fs.cuh"
#include "internal.h"

namespace tg {

// Level l from level l + 1: entry x is the product of entries 2x and 2x + 1, in Fp2.
__global__ void tr_product_level(const ulonglong2* below, ulonglong2* above, uint64_t m) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t x = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; x < m; x += stride) {
        const ulonglong2 a = below[2 * x], b = below[2 * x + 1];
        const fp2 p = e_mul(fp2{a.x, a.y}, fp2{b.x, b.y});
        above[x] = make_ulonglong2(p.c0, p.c1);
    }
}

// The same in the prime field: a forest of prime-field leaves keeps every level there, one word
// an entry (the pair is one 16-byte load).
__global__ void tr_product_level_base(const ulonglong2* below, uint64_t* above, uint64_t m) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t x = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; x < m; x += stride) {
        const ulonglong2 v = below[x];
        above[x] = mul(v.x, v.y);
    }
}

// Two levels in one pass: level l (m2 = 2m entries) and level l − 1 (m entries) from level l + 1,
// so that level l is written but not read back. Thread x reads entries 4x … 4x + 3 below.
__global__ void tr_product_level2(const ulonglong2* below, ulonglong2* mid, ulonglong2* above, uint64_t m) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t x = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; x < m; x += stride) {
        const ulonglong2 a = below[4 * x], b = below[4 * x + 1], c = below[4 * x + 2], d = below[4 * x + 3];
        const fp2 p = l2_canon(l2_muls(fp2{a.x, a.y}, fp2{b.x, b.y})), q = l2_canon(l2_muls(fp2{c.x, c.y}, fp2{d.x, d.y}));
        const fp2 r = l2_canon(l2_muls(p, q));
        mid[2 * x] = make_ulonglong2(p.c0, p.c1);
        mid[2 * x + 1] = make_ulonglong2(q.c0, q.c1);
        above[x] = make_ulonglong2(r.c0, r.c1);
    }
}

__global__ void tr_product_level2_base(const ulonglong2* below, ulonglong2* mid, uint64_t* above, uint64_t m) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t x = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; x < m; x += stride) {
        const ulonglong2 a = below[2 * x], b = below[2 * x + 1];
        const uint64_t p = lz::canon(lz::mul(a.x, a.y)), q = lz::canon(lz::mul(b.x, b.y));
        mid[x] = make_ulonglong2(p, q);
        above[x] = lz::canon(lz::mul(p, q));
    }
}

// (n, d) of level l from level l + 1; n null: every numerator below is 1, so n_out = d_L + d_R.
__global__ void tr_fraction_level(const ulonglong2* n, const ulonglong2* d, ulonglong2* n_out, ulonglong2* d_out,
                                  uint64_t m) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t x = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; x < m; x += stride) {
        const ulonglong2 dl = d[2 * x], dr = d[2 * x + 1];
        const fp2 c = {dl.x, dl.y}, e = {dr.x, dr.y};
        fp2 nn;
        if (n) {
            const ulonglong2 nl = n[2 * x], nr = n[2 * x + 1];
            nn = e_add(e_mul(fp2{nl.x, nl.y}, e), e_mul(fp2{nr.x, nr.y}, c));
        } else {
            nn = e_add(c, e);
        }
        const fp2 dd = e_mul(c, e);
        n_out[x] = make_ulonglong2(nn.c0, nn.c1);
        d_out[x] = make_ulonglong2(dd.c0, dd.c1);
    }
}

// Two fraction levels in one pass, as tr_product_level2 (n null: numerators of 1 below).
__global__ void tr_fraction_level2(const ulonglong2* n, const ulonglong2* d, ulonglong2* n_mid, ulonglong2* d_mid,
                                   ulonglong2* n_out, ulonglong2* d_out, uint64_t m) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t x = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; x < m; x += stride) {
        fp2 nn[2], dd[2];
        for (int h = 0; h < 2; h++) {
            const ulonglong2 dl = d[4 * x + 2 * h], dr = d[4 * x + 2 * h + 1];
            const fp2 c = {dl.x, dl.y}, e = {dr.x, dr.y};
            if (n) {
                const ulonglong2 nl = n[4 * x + 2 * h], nr = n[4 * x + 2 * h + 1];
                nn[h] = l2_canon(l2_dot(fp2{nl.x, nl.y}, e, fp2{nr.x, nr.y}, c));
            } else {
                nn[h] = l2_canon(l2_add(c, e));
            }
            dd[h] = l2_canon(l2_muls(c, e));
            n_mid[2 * x + h] = make_ulonglong2(nn[h].c0, nn[h].c1);
            d_mid[2 * x + h] = make_ulonglong2(dd[h].c0, dd[h].c1);
        }
        // (products as unreduced sums, every stored entry canonical)
        const fp2 no = l2_canon(l2_dot(nn[0], dd[1], nn[1], dd[0])), dn = l2_canon(l2_muls(dd[0], dd[1]));
        n_out[x] = make_ulonglong2(no.c0, no.c1);
        d_out[x] = make_ulonglong2(dn.c0, dn.c1);
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

// Generated LogUp leaf j: (n_j, α − (k_j + β·v_j)) with k_j = counter(key_seed + j),
// v_j = counter(value_seed + j), and n_j = 1 (a lookup tree) or −m_j, m_j = counter(mult_seed + j)
// mod 2^16 (a table tree); canonical.
struct LeafGen {
    uint64_t key_seed, value_seed, mult_seed;
    int unit, pad_;
    fp2 alpha, beta;
};
__device__ __forceinline__ void logup_leaf(const LeafGen& g, uint64_t j, fp2& n, fp2& d) {
    const uint64_t k = counter_value(g.key_seed + j), v = counter_value(g.value_seed + j);
    d = {sub(sub(g.alpha.c0, k), mul(g.beta.c0, v)), sub(g.alpha.c1, mul(g.beta.c1, v))};
    n = {1, 0};
    if (!g.unit) {
        const uint64_t m = counter_value(g.mult_seed + j) & 0xFFFF;
        n.c0 = m == 0 ? 0 : P - m;
    }
}

__global__ void tr_logup_leaves(LeafGen g, ulonglong2* n_out, ulonglong2* d_out, uint64_t count) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; j < count; j += stride) {
        fp2 n, d;
        logup_leaf(g, j, n, d);
        d_out[j] = make_ulonglong2(d.c0, d.c1);
        if (n_out) n_out[j] = make_ulonglong2(n.c0, n.c1);  // numerators of 1 are not stored
    }
}

// Generated leaves and the two levels above them in one pass (tr_fraction_level2 without reading
// the leaves back): thread x generates leaves 4x … 4x + 3 and stores them for the leaf level's
// rounds (numerators only when not all 1), then their two parents and their grandparent.
__global__ void tr_logup_level2(LeafGen g, ulonglong2* n_leaf, ulonglong2* d_leaf, ulonglong2* n_mid,
                                ulonglong2* d_mid, ulonglong2* n_out, ulonglong2* d_out, uint64_t m) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t x = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; x < m; x += stride) {
        fp2 n4[4], d4[4];
#pragma unroll
        for (int i = 0; i < 4; i++) {
            logup_leaf(g, 4 * x + i, n4[i], d4[i]);
            d_leaf[4 * x + i] = make_ulonglong2(d4[i].c0, d4[i].c1);
            if (!g.unit) n_leaf[4 * x + i] = make_ulonglong2(n4[i].c0, n4[i].c1);
        }
        fp2 nn[2], dd[2];
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const fp2 c = d4[2 * h], e = d4[2 * h + 1];
            nn[h] = g.unit ? l2_canon(l2_add(c, e)) : l2_canon(l2_dot(n4[2 * h], e, n4[2 * h + 1], c));
            dd[h] = l2_canon(l2_muls(c, e));
            n_mid[2 * x + h] = make_ulonglong2(nn[h].c0, nn[h].c1);
            d_mid[2 * x + h] = make_ulonglong2(dd[h].c0, dd[h].c1);
        }
        const fp2 no = l2_canon(l2_dot(nn[0], dd[1], nn[1], dd[0])), dn = l2_canon(l2_muls(dd[0], dd[1]));
        n_out[x] = make_ulonglong2(no.c0, no.c1);
        d_out[x] = make_ulonglong2(dn.c0, dn.c1);
    }
}

static LeafGen leaf_gen(const tg_leaf_gen& g) {
    LeafGen o;
    memset(&o, 0, sizeof o);
    o.key_seed = g.key_seed, o.value_seed = g.value_seed, o.mult_seed = g.mult_seed, o.unit = g.unit ? 1 : 0;
    o.alpha = {g.alpha[0], g.alpha[1]}, o.beta = {g.beta[0], g.beta[1]};
    return o;
}

static unsigned grid_of(const Device* d, uint64_t items) {
    return (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((items + 255) / 256, (uint64_t)d->sm_count * 16));
}

struct TreeLevels {
    int kind = 0;  // 0 forest, 1 fraction
    uint32_t s = 0, h = 0;
    bool base = false;  // a forest of prime-field leaves: every level one word an entry
    std::vector<std::unique_ptr<DevBuf>> n, d;  // level l, l = 0..h (fractions use both)
    fp2 sent_n = {0, 0}, sent_d = {0, 0};
    bool unit = false;      // a fraction tree whose leaf numerators are all 1
    std::vector<fp2> root;  // forest: the root level; fraction: (n, d)
    int own = -1;           // the tree's level of its current claim; −1 before it joins
    std::vector<fp2> point;
    fp2 value = {0, 0}, p = {0, 0}, q = {0, 0};
};

// Σ_y v[y]·eq(r, y) (y_1 the lowest bit) by binding one coordinate at a time: 2^n products for
// 2^n values, where a fresh eq product per y would cost n·2^n.
static fp2 host_mle(std::vector<fp2> v, const std::vector<fp2>& r) {
    for (size_t i = 0; i < r.size(); i++) {
        const size_t half = v.size() / 2;
        for (size_t k = 0; k < half; k++) v[k] = e_add(v[2 * k], e_mul(r[i], e_sub(v[2 * k + 1], v[2 * k])));
        v.resize(half);
    }
    return v.empty() ? fp2{0, 0} : v[0];
}

// p(r) for the polynomial through (k, v_k), k = 0..3 (Lagrange; the denominators' inverses are
// those of −6, 2, −2 and 6, computed once).
static fp2 lagrange4(const fp2 v[4], fp2 r) {
    static const uint64_t dinv[4] = {inv(P - 6), inv(2), inv(P - 2), inv(6)};
    fp2 out = {0, 0};
    for (int i = 0; i < 4; i++) {
        fp2 num = {1, 0};
        for (int m = 0; m < 4; m++)
            if (m != i) num = e_mul(num, e_sub(r, fp2{(uint64_t)m, 0}));
        out = e_add(out, e_mul(v[i], e_scale(num, dinv[i])));
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

// 1/a in Fp2 as conj(a)/N(a), N(a) = a0^2 − 7·a1^2 (nonzero for a ≠ 0: 7 is no square mod p);
// 0 for a = 0.
static fp2 host_inv2(fp2 a) {
    const uint64_t nrm = sub(mul(a.c0, a.c0), mul7(mul(a.c1, a.c1)));
    if (nrm == 0) return {0, 0};
    const uint64_t ni = inv(nrm);
    return {mul(a.c0, ni), mul(sub(0, a.c1), ni)};
}

// ---- the level sumcheck, specialised for tree levels ----------------------------------------------
//
// A present tree on n variables proves Σ_x eq(p, x)·g(x) with g = L·R (forest) or
// N0·D1 + N1·D0 + λ·D0·D1 (fraction tree) over the halves of the level below. eq is never
// tabulated or bound: at the tree's own round j the message is
//   p_j(X) = C_j · eq1(p_j, X) · q_j(X),   q_j(X) = Σ_{x'} eq(p_{>j}, x')·g(X, x')
// with C_j = Π_{i<j} eq1(p_i, r_i) a running scalar and eq1(t, X) = (1 − t)(1 − X) + t·X, and the
// weights eq(p_{>j}, x') = lo_j[x' mod 2^L]·hi_j[x' >> L] come from small per-round tables built
// once per level from the point. Round 0 reads the level below directly (the halves are its even
// and odd entries); each later round binds the previous challenge into the tables as it sums.
//
// q_j has degree 2, and the device sums only q_j(0) and its leading coefficient q_j(∞): the round's
// claim gives q_j(1) = (Q_j − (1 − p_j)·q_j(0))/p_j with Q_j = claim_j/C_j, which is the tree's
// claim in its first round and q_{j−1}(r_{j−1}) after, as the reference's CPU prover derives v(1)
// from its claim (crates/tessera-sumcheck/src/level.rs:317-347). Where p_j = 0 nothing divides, and
// that round's launch sums q_j(1) as well.

constexpr int TL_THREADS = 256;
constexpr int TL_LOW = 11;  // the low eq table's variables: the pairs of one chunk share a high weight
constexpr uint64_t TL_TAIL_PAIRS = 512;
constexpr uint32_t TL_ROOT_DEVICE_LOG = 12;  // a joining forest of 2^s ≥ 2^12 roots folds its claim on the device  // rounds of at most this many pairs a segment run in one block

struct TlSeg {
    const void* src[4];  // table T's entry x is src[T][x·stride]: Fp2, or prime-field words when base
    ulonglong2* dst[4];  // bound tables (when bind)
    const ulonglong2* lo;  // this round's eq weights over the remaining variables
    const ulonglong2* hi;
    const uint64_t* r;     // the challenge to bind
    ulonglong2* out;       // the round's sums: q(0), q(1) (launches that form it), q(∞)
    uint64_t n;            // pairs: 2^lbits a chunk
    uint64_t lam[2];
    uint64_t mu[2];        // 1/λ, for the shifted form of numerators of 1 (shift)
    int kind, stride, bind, lbits;
    int block0, nblocks, part0, mode;
    int shift, pad_;       // kind 2 with λ ≠ 0: g summed as (D0 + μ)(D1 + μ)
};
static_assert(sizeof(TlSeg) % 8 == 0, "TlSeg copies as words");

struct TlTree {  // one present tree, as the transcript kernel sees it
    uint64_t w[2];  // γ^i
    uint64_t C[2];  // the running eq scalar
    uint64_t Q[2];  // the sum its current own round proves, over C
    uint64_t S[2];  // its claim, which its padding rounds carry
    const uint64_t* point;  // n Fp2
    const uint64_t* tinv;   // n Fp2: 1/point[j], or 0 where point[j] = 0
    int n, pad;
};

__device__ __forceinline__ fp2 ld2(const ulonglong2* p) {
    const ulonglong2 v = *p;
    return {v.x, v.y};
}


// g at X = 0, at X = 1 (ONE) and its leading coefficient in X, over one pair whose tables take the
// values u at X = 0 and slopes d: KIND 0 L·R; 1 N0·D1 + N1·D0 + λ·D0·D1 = N0·D1 + D0·(N1 + λ·D1);
// 2 D0 + D1 + λ·D0·D1, whose leading coefficient λ·dD0·dD1 is returned without the λ (the kernel
// applies it once to the sum). With shift (λ ≠ 0, μ = 1/λ), kind 2 is λ·(D0 + μ)(D1 + μ) − μ: the
// pair gives (D0 + μ)(D1 + μ) at the nodes, and since the eq weights sum to 1 the kernel turns the
// segment's sums into λ·S − μ at 0 and 1 and λ·S at ∞ once — one Fp2 product fewer per node.
template <int KIND, bool ONE>
__device__ __forceinline__ void tl_nodes(const fp2* u, const fp2* d, fp2 lam, uint64_t lam7, fp2 mu, bool shift, fp2& g0,
                                         fp2& g1, fp2& gi) {
    if constexpr (KIND == 0) {
        g0 = l2_muls(u[0], u[1]);
        gi = l2_muls(d[0], d[1]);
        if constexpr (ONE) g1 = l2_muls(l2_add(u[0], d[0]), l2_add(u[1], d[1]));
    } else if constexpr (KIND == 1) {
        auto f = [&](fp2 n0, fp2 n1, fp2 d0, fp2 d1) { return l2_dot(n0, d1, d0, l2_fma(n1, lam, lam7, d1)); };
        g0 = f(u[0], u[1], u[2], u[3]);
        gi = f(d[0], d[1], d[2], d[3]);
        if constexpr (ONE)
            g1 = f(l2_add(u[0], d[0]), l2_add(u[1], d[1]), l2_add(u[2], d[2]), l2_add(u[3], d[3]));
    } else if (shift) {
        const fp2 a = l2_add(u[0], mu), b = l2_add(u[1], mu);
        g0 = l2_muls(a, b);
        gi = l2_muls(d[0], d[1]);
        if constexpr (ONE) g1 = l2_muls(l2_add(a, d[0]), l2_add(b, d[1]));
    } else {
        g0 = l2_fma(l2_add(u[0], u[1]), lam, lam7, l2_muls(u[0], u[1]));
        gi = l2_muls(d[0], d[1]);
        if constexpr (ONE) {
            const fp2 a = l2_add(u[0], d[0]), b = l2_add(u[1], d[1]);
            g1 = l2_fma(l2_add(a, b), lam, lam7, l2_muls(a, b));
        }
    }
}

// A kind-2 segment's per-thread sums under λ: all three with shift, else the leading coefficient.
__device__ __forceinline__ void tl_unit_scale(const TlSeg& g, fp2 (&acc)[3]) {
    const fp2 lam = {g.lam[0], g.lam[1]};
    acc[2] = l2_mul(lam, acc[2]);
    if (g.shift) acc[0] = l2_mul(lam, acc[0]), acc[1] = l2_mul(lam, acc[1]);
}

// A shifted kind-2 segment's reduced sums (canonical words) less μ at the nodes 0 and 1.
__device__ __forceinline__ void tl_unit_finish(const TlSeg& g, uint64_t (&words)[6]) {
    if (g.kind != 2 || !g.shift) return;
    for (int n = 0; n < 2; n++) words[2 * n] = sub(words[2 * n], g.mu[0]), words[2 * n + 1] = sub(words[2 * n + 1], g.mu[1]);
}

// The modes of a segment's tables in a round: Fp2 tables summed as they are (a tree's round 0),
// prime-field tables bound into Fp2 (a prime-field forest's round 1), prime-field tables summed (its
// round 0), and Fp2 tables bound by the previous challenge as they are summed (every later round).
enum : int { TL_SUM = 0, TL_BIND_BASE = 1, TL_SUM_BASE = 2, TL_BIND = 3 };

// Pairs a thread loads before it computes any: enough bytes in flight per thread to cover the
// latency of HBM at two or three resident blocks per SM, within the register budget.
template <int KIND, int MODE>
__host__ __device__ constexpr int tl_batch() {
    return MODE == TL_SUM_BASE ? 2 : (KIND == 1 || MODE == TL_BIND) ? 1 : 2;
}

// One pair's values as loaded: E entries of each of NT tables (E = 4 when binding, else 2),
// prime-field words in .x for the base modes.
template <int NT, int MODE>
struct TlRaw {
    static constexpr int E = (MODE == TL_BIND || MODE == TL_BIND_BASE) ? 4 : 2;
    ulonglong2 v[NT][E];
};

// The loads of pair p. Prime-field levels hold L and R interleaved (L[x], R[x]) as one 16-byte
// word pair, so a pair's 2E words come in E vector loads.
template <int NT, int MODE>
__device__ __forceinline__ void tl_load(const TlSeg& g, uint64_t p, TlRaw<NT, MODE>& raw) {
    constexpr int E = TlRaw<NT, MODE>::E;
    if constexpr (MODE == TL_SUM_BASE || MODE == TL_BIND_BASE) {
        const ulonglong2* lv = static_cast<const ulonglong2*>(g.src[0]) + E * p;
#pragma unroll
        for (int e = 0; e < E; e++) raw.v[0][e] = lv[e];
    } else {
        const uint64_t st = (uint64_t)g.stride;
#pragma unroll
        for (int k = 0; k < NT; k++) {
            const ulonglong2* src = static_cast<const ulonglong2*>(g.src[k]);
#pragma unroll
            for (int e = 0; e < E; e++) raw.v[k][e] = src[(E * p + e) * st];
        }
    }
}

// A pair's contribution: binds (writing the bound entries), forms g at the nodes and adds w·g to
// the chunk's unreduced part sums. k7 holds 7·c1 of the constants: r (the challenge), λ, w.
struct TlK7 {
    uint64_t r, lam;
};
template <int NT, int KIND, int MODE, bool ONE>
__device__ __forceinline__ void tl_pair(const TlSeg& g, uint64_t p, const TlRaw<NT, MODE>& raw, fp2 w, fp2 r, fp2 lam,
                                        TlK7 k7, Acc2 (&part)[3]) {
    if constexpr (MODE == TL_SUM_BASE) {
        const uint64_t l0 = raw.v[0][0].x, r0 = raw.v[0][0].y, l1 = raw.v[0][1].x, r1 = raw.v[0][1].y;
        const uint64_t v0 = lz::mul(l0, r0), vi = lz::mul(lz::sub(l1, l0), lz::sub(r1, r0));
        l2_mad_base(part[0], w, v0);
        l2_mad_base(part[2], w, vi);
        if constexpr (ONE) l2_mad_base(part[1], w, lz::mul(l1, r1));
    } else {
        fp2 u[NT], d[NT];
        if constexpr (MODE == TL_BIND_BASE) {
#pragma unroll
            for (int k = 0; k < 2; k++) {  // table k's entries 4p..4p+3 are raw.v[0][e] .x (L) or .y (R)
                const uint64_t a0 = k ? raw.v[0][0].y : raw.v[0][0].x, a1 = k ? raw.v[0][1].y : raw.v[0][1].x;
                const uint64_t b0 = k ? raw.v[0][2].y : raw.v[0][2].x, b1 = k ? raw.v[0][3].y : raw.v[0][3].x;
                const uint64_t da = lz::sub(a1, a0), db = lz::sub(b1, b0);
                const fp2 uu = {lz::add(a0, lz::mul(r.c0, da)), lz::mul(r.c1, da)};
                const fp2 vv = {lz::add(b0, lz::mul(r.c0, db)), lz::mul(r.c1, db)};
                g.dst[k][2 * p] = make_ulonglong2(uu.c0, uu.c1);
                g.dst[k][2 * p + 1] = make_ulonglong2(vv.c0, vv.c1);
                u[k] = uu;
                d[k] = l2_sub(vv, uu);
            }
        } else if constexpr (MODE == TL_BIND) {
#pragma unroll
            for (int k = 0; k < NT; k++) {
                const fp2 a0 = {raw.v[k][0].x, raw.v[k][0].y}, a1 = {raw.v[k][1].x, raw.v[k][1].y};
                const fp2 b0 = {raw.v[k][2].x, raw.v[k][2].y}, b1 = {raw.v[k][3].x, raw.v[k][3].y};
                const fp2 uu = l2_fma(a0, r, k7.r, l2_sub(a1, a0));
                const fp2 vv = l2_fma(b0, r, k7.r, l2_sub(b1, b0));
                g.dst[k][2 * p] = make_ulonglong2(uu.c0, uu.c1);
                g.dst[k][2 * p + 1] = make_ulonglong2(vv.c0, vv.c1);
                u[k] = uu;
                d[k] = l2_sub(vv, uu);
            }
        } else {
#pragma unroll
            for (int k = 0; k < NT; k++) {
                u[k] = {raw.v[k][0].x, raw.v[k][0].y};
                d[k] = l2_sub(fp2{raw.v[k][1].x, raw.v[k][1].y}, u[k]);
            }
        }
        fp2 g0, g1, gi;
        tl_nodes<KIND, ONE>(u, d, lam, k7.lam, fp2{g.mu[0], g.mu[1]}, g.shift, g0, g1, gi);
        const uint64_t w7 = lz::mul7(w.c1);
        l2_mad(part[0], w, w7, g0);
        l2_mad(part[2], w, w7, gi);
        if constexpr (ONE) l2_mad(part[1], w, w7, g1);
    }
}

// This block's share of a segment: chunks c = b, b + nblocks, … of 2^lbits pairs, each summed with
// its low weights and then scaled once by its high weight, into acc = (q(0), q(1), q(∞)). A thread
// loads tl_batch pairs (TL_THREADS apart) before it computes them.
template <int NT, int KIND, int MODE, bool ONE>
__device__ __forceinline__ void tl_sum(const TlSeg& g, uint64_t b, fp2 (&acc)[3]) {
    constexpr int U = tl_batch<KIND, MODE>();
    const int lb = g.lbits;
    const uint64_t span = 1ull << lb, chunks = g.n >> lb;
    const fp2 r = (MODE == TL_BIND || MODE == TL_BIND_BASE) ? fp2{g.r[0], g.r[1]} : fp2{0, 0};
    const fp2 lam = {g.lam[0], g.lam[1]};
    const TlK7 k7 = {lz::mul7(r.c1), lz::mul7(lam.c1)};
    for (uint64_t c = b; c < chunks; c += (uint64_t)g.nblocks) {
        Acc2 part[3] = {acc2_zero(), acc2_zero(), acc2_zero()};
        for (uint64_t e0 = threadIdx.x; e0 < span; e0 += (uint64_t)U * TL_THREADS) {
            TlRaw<NT, MODE> raw[U];
#pragma unroll
            for (int u = 0; u < U; u++) {
                const uint64_t e = e0 + (uint64_t)u * TL_THREADS;
                if (U == 1 || e < span) tl_load<NT, MODE>(g, (c << lb) + e, raw[u]);
            }
#pragma unroll
            for (int u = 0; u < U; u++) {
                const uint64_t e = e0 + (uint64_t)u * TL_THREADS;
                if (U == 1 || e < span) tl_pair<NT, KIND, MODE, ONE>(g, (c << lb) + e, raw[u], ld2(g.lo + e), r, lam, k7, part);
            }
        }
        const fp2 h = ld2(g.hi + c);
        acc[0] = l2_add(acc[0], l2_mul(h, l2_reduce(part[0])));
        acc[2] = l2_add(acc[2], l2_mul(h, l2_reduce(part[2])));
        if constexpr (ONE) acc[1] = l2_add(acc[1], l2_mul(h, l2_reduce(part[1])));
    }
}

// The block's six-word sum, into thread 0's words (red: a row per warp; the call ends with every
// thread past a barrier after the last use of red but thread 0's reads).
__device__ __forceinline__ void tl_block_sum(uint64_t (&words)[6], uint64_t (*red)[6]) {
#pragma unroll
    for (int w = 0; w < 6; w++)
        for (int o = 16; o > 0; o >>= 1) words[w] = add(words[w], __shfl_down_sync(0xFFFFFFFFu, words[w], o));
    if ((threadIdx.x & 31) == 0)
        for (int w = 0; w < 6; w++) red[threadIdx.x >> 5][w] = words[w];
    __syncthreads();
    if (threadIdx.x == 0)
        for (int k = 1; k < (int)(blockDim.x >> 5); k++)
            for (int w = 0; w < 6; w++) words[w] = add(words[w], red[k][w]);
}

// One round's segments of one kind and mode: each block sums its share of its segment, and the
// segment's last block adds the blocks' rows into the segment's q.
// Resident blocks per SM a variant's registers allow: three for the prime-field sums, two else.
template <int KIND, int MODE>
__host__ __device__ constexpr int tl_min_blocks() {
    return MODE == TL_SUM_BASE || (KIND != 1 && MODE == TL_BIND) ? 3 : 2;
}

template <int NT, int KIND, int MODE, bool ONE>
__global__ void __launch_bounds__(TL_THREADS, tl_min_blocks<KIND, MODE>()) tl_rounds(const TlSeg* segs, int nseg,
                                                                              uint64_t* partials, unsigned* counters) {
    __shared__ TlSeg g;
    __shared__ int si;
    __shared__ uint64_t red[TL_THREADS / 32][6];
    __shared__ bool last;
    if (threadIdx.x == 0) {
        int lo = 0, hi = nseg - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) / 2;
            if (segs[mid].block0 <= (int)blockIdx.x)
                lo = mid;
            else
                hi = mid - 1;
        }
        si = lo;
    }
    __syncthreads();
    {
        const uint64_t* from = reinterpret_cast<const uint64_t*>(segs + si);
        uint64_t* to = reinterpret_cast<uint64_t*>(&g);
        for (int w = threadIdx.x; w < (int)(sizeof(TlSeg) / 8); w += blockDim.x) to[w] = from[w];
    }
    __syncthreads();
    fp2 acc[3] = {{0, 0}, {0, 0}, {0, 0}};
    const uint64_t b = (uint64_t)(blockIdx.x - g.block0);
    tl_sum<NT, KIND, MODE, ONE>(g, b, acc);
    if constexpr (KIND == 2) tl_unit_scale(g, acc);
    // block sums, then the segment's last block reduces the partial rows (every thread a share)
    uint64_t words[6];
    for (int i = 0; i < 3; i++) {
        const fp2 c = l2_canon(acc[i]);
        words[2 * i] = c.c0, words[2 * i + 1] = c.c1;
    }
    auto block_sum = [&]() { tl_block_sum(words, red); };
    block_sum();
    if (threadIdx.x == 0) {
        for (int w = 0; w < 6; w++) partials[(size_t)(g.part0 + b) * 8 + w] = words[w];
        __threadfence();
        last = atomicAdd(&counters[si], 1u) == (unsigned)g.nblocks - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    for (int w = 0; w < 6; w++) words[w] = 0;
    for (int k = threadIdx.x; k < g.nblocks; k += blockDim.x)
        for (int w = 0; w < 6; w++) words[w] = add(words[w], __ldcg(&partials[(size_t)(g.part0 + k) * 8 + w]));
    __syncthreads();  // red is reused
    block_sum();
    if (threadIdx.x == 0) {
        tl_unit_finish(g, words);
        for (int w = 0; w < 6; w++) reinterpret_cast<uint64_t*>(g.out)[w] = words[w];
        counters[si] = 0;
    }
}

// A segment's kernel key: its kind and mode (the launches of a round go one per key).
__host__ __device__ constexpr int tl_key(int kind, int mode) { return kind * 4 + mode; }

template <bool ONE>
static void tl_launch(int key, int blocks, cudaStream_t s, const TlSeg* segs, int nseg, uint64_t* partials,
                      unsigned* counters) {
    switch (key) {
#define TL_CASE(NT, KIND, MODE)                                                                          \
    case KIND * 4 + MODE:                                                                                \
        tl_rounds<NT, KIND, MODE, ONE><<<blocks, TL_THREADS, 0, s>>>(segs, nseg, partials, counters); \
        break;
        TL_CASE(2, 0, TL_SUM)
        TL_CASE(2, 0, TL_BIND_BASE)
        TL_CASE(2, 0, TL_SUM_BASE)
        TL_CASE(2, 0, TL_BIND)
        TL_CASE(4, 1, TL_SUM)
        TL_CASE(4, 1, TL_BIND)
        TL_CASE(2, 2, TL_SUM)
        TL_CASE(2, 2, TL_BIND)
#undef TL_CASE
        default:
            break;
    }
}

// The low eq table's variables for a round over 2^rem pairs: TL_LOW for large rounds (one high
// weight per chunk of 2^TL_LOW pairs), fewer where that would leave too few chunks to fill the GPU,
// but at least a block's worth of pairs a chunk.
inline int tl_low_bits(int rem) { return std::min(rem, std::max(8, std::min(TL_LOW, rem - 10))); }

// The eq weight tables of every round of every present tree: entry e of table t is
// Π_i eq1(c_i, bit_i(e)) over the table's coordinates c (lo: the first L of the round's remaining
// coordinates, hi: the rest).
struct TlEqJob {
    const uint64_t* coords;  // Fp2 coordinates
    int ncoords;
    ulonglong2* out;
    uint64_t entries;
};
__global__ void tl_eq_tables(const TlEqJob* jobs, int njobs, uint64_t total) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += stride) {
        uint64_t at = i;
        int jb = 0;
        while (jb < njobs && at >= jobs[jb].entries) at -= jobs[jb++].entries;
        if (jb >= njobs) return;
        const TlEqJob& J = jobs[jb];
        fp2 pr = {1, 0};
        for (int c = 0; c < J.ncoords; c++) {
            const fp2 t = {J.coords[2 * c], J.coords[2 * c + 1]};
            pr = e_mul(pr, (at >> c) & 1 ? t : e_sub(fp2{1, 0}, t));
        }
        J.out[at] = make_ulonglong2(pr.c0, pr.c1);
    }
}

// eq1(t, X) = (1 − t)(1 − X) + t·X
__device__ __forceinline__ fp2 eq1(fp2 t, fp2 x) {
    const fp2 one = {1, 0};
    return e_add(e_mul(e_sub(one, t), e_sub(one, x)), e_mul(t, x));
}

// Own round jj's q(X) = a + b·X + c·X², from its sums q(0), q(∞) and q(1) = (Q − (1 − t)·q(0))/t
// (t = point[jj]), or the summed q(1) where t = 0.
__device__ void tl_quad(const TlTree& T, int jj, const ulonglong2* q, fp2& a, fp2& b, fp2& c) {
    a = ld2(q);
    c = ld2(q + 2);
    const fp2 t = {T.point[2 * jj], T.point[2 * jj + 1]}, ti = {T.tinv[2 * jj], T.tinv[2 * jj + 1]};
    fp2 q1;
    if (ti.c0 == 0 && ti.c1 == 0)
        q1 = ld2(q + 1);
    else
        q1 = l2_mul(l2_sub(fp2{T.Q[0], T.Q[1]}, l2_mul(l2_sub(fp2{1, 0}, t), a)), ti);
    b = l2_sub(l2_sub(q1, a), c);  // lazy words, as Q and C are kept
}

// Round j of a level: the message Σ_i γ^i·(2^{pad_i − j − 1}·S_i while padded, else
// C_i·eq1(p_i[j'], X)·q_i(X)) at X = 0, 2, 3, absorbed under <prefix>/round/j; r_j drawn under
// <prefix>/r/j; then each tree in its own rounds takes Q_i ← q_i(r_j) and C_i ← C_i·eq1(p_i[j'], r_j).
// One warp runs it (sbuf: FS_BUF_WORDS of shared memory).
__device__ void tl_fs_round(FsState* st, const FsJob& jb, int j, const FsKeys& keys, TlTree* trees, int ntrees,
                            ulonglong2* q, uint64_t* rounds_out, uint64_t* chal_out, uint32_t* sbuf) {
    const int lane = threadIdx.x & 31;
    // lane x (< 3) forms node x of the message (X = 0, 2, 3), lazy words; the others follow along
    const int x = lane < 3 ? lane : 0;
    fp2 mine = {0, 0};
    for (int i = 0; i < ntrees; i++) {
        const TlTree& T = trees[i];
        const fp2 w = {T.w[0], T.w[1]};
        const int jj = j - T.pad;
        if (jj < 0) {
            const fp2 ws = l2_mul(w, fp2{T.S[0], T.S[1]});
            mine = l2_add(mine, fp2{mul_pow2_lt64(ws.c0, T.pad - j - 1), mul_pow2_lt64(ws.c1, T.pad - j - 1)});
        } else {
            // γ^i·C·eq1(t, X) at this lane's node (1 − t, 3t − 1, 5t − 2), independent of the sums
            const fp2 t = {T.point[2 * jj], T.point[2 * jj + 1]};
            const fp2 t2 = l2_add(t, t), t3 = l2_add(t2, t);
            const fp2 e = x == 0 ? l2_sub(fp2{1, 0}, t) : x == 1 ? l2_sub(t3, fp2{1, 0}) : l2_sub(l2_add(t3, t2), fp2{2, 0});
            const fp2 wce = l2_mul(l2_mul(w, fp2{T.C[0], T.C[1]}), e);
            fp2 a, b, c;
            tl_quad(T, jj, q + 4 * i, a, b, c);
            if (lane == 0) q[4 * i + 3] = make_ulonglong2(b.c0, b.c1);  // for the update after the challenge
            // q(0) = a, q(2) = a + 2b + 4c, q(3) = a + 3b + 9c
            const fp2 b2 = l2_add(b, b), c2 = l2_add(c, c), c4 = l2_add(c2, c2);
            const fp2 qx = x == 0 ? a
                         : x == 1 ? l2_add(a, l2_add(b2, c4))
                                  : l2_add(l2_add(a, l2_add(b2, b)), l2_add(l2_add(c4, c4), c));
            mine = l2_add(mine, l2_mul(wce, qx));
        }
    }
    mine = l2_canon(mine);
    fp2 msg[3];
    for (int k = 0; k < 3; k++) msg[k] = {__shfl_sync(0xFFFFFFFFu, mine.c0, k), __shfl_sync(0xFFFFFFFFu, mine.c1, k)};
    uint32_t state[8];
    for (int i = 0; i < 8; i++) state[i] = reinterpret_cast<const uint32_t*>(st->state)[i];
    uint64_t counter = st->counter;
    if (lane == 0)
        for (int x = 0; x < 3; x++) rounds_out[6 * j + 2 * x] = msg[x].c0, rounds_out[6 * j + 2 * x + 1] = msg[x].c1;
    // the message as TCE Vec<Fp2>: its length, then the values
    const uint64_t pay[7] = {3, msg[0].c0, msg[0].c1, msg[1].c0, msg[1].c1, msg[2].c0, msg[2].c1};
    const uint32_t len = fs_msg_warp<7>(state, jb, fs_pack("/round/"), fs_len("/round/"), j, pay, 7, sbuf);
    uint64_t c0, c1;
    const bool ok = fs_round_warp(keys, jb, j, sbuf, len, state, &counter, &c0, &c1);  // ends with a warp barrier
    if (lane == 0) {
        if (!ok) {
            st->err = 1;
        } else {
            for (int i = 0; i < 8; i++) reinterpret_cast<uint32_t*>(st->state)[i] = state[i];
            st->counter = counter;
            st->r[0] = c0, st->r[1] = c1;
            chal_out[2 * j] = c0, chal_out[2 * j + 1] = c1;
        }
    }
    if (!ok || lane < 1 || lane > 2) return;
    // each tree in its own rounds: lane 1 takes Q ← q(r), lane 2 C ← C·eq1(t, r)
    const fp2 r = {c0, c1};
    for (int i = 0; i < ntrees; i++) {
        TlTree& T = trees[i];
        const int jj = j - T.pad;
        if (jj < 0) continue;
        if (lane == 1) {
            const fp2 a = ld2(q + 4 * i), b = ld2(q + 4 * i + 3), c = ld2(q + 4 * i + 2);  // b as the message pass left it
            const fp2 Q = l2_add(a, l2_mul(r, l2_add(b, l2_mul(r, c))));
            T.Q[0] = Q.c0, T.Q[1] = Q.c1;
        } else {
            const fp2 t = {T.point[2 * jj], T.point[2 * jj + 1]};
            const fp2 tr = l2_mul(t, r);  // eq1(t, r) = 1 − t − r + 2·t·r
            const fp2 C = l2_mul(fp2{T.C[0], T.C[1]}, l2_add(l2_sub(l2_sub(fp2{1, 0}, t), r), l2_add(tr, tr)));
            T.C[0] = C.c0, T.C[1] = C.c1;
        }
    }
}

__global__ void tl_fs(FsState* st, FsJob jb, int j, FsKeys keys, TlTree* trees, int ntrees, ulonglong2* q,
                      uint64_t* rounds_out, uint64_t* chal_out) {
    __shared__ uint32_t sbuf[FS_BUF_WORDS];
    tl_fs_round(st, jb, j, keys, trees, ntrees, q, rounds_out, chal_out, sbuf);
}

// A joining forest's claim Σ_y root[y]·eq(point, y) (y_1 the lowest bit) by binding one point
// coordinate at a time, in one block: the root level (2^s prime-field words or Fp2 entries) folds
// into the ping-pong scratch (2^(s−1) + 2^(s−2) entries). The claim becomes the tree's Q and S for
// the rounds, and goes to out (canonical) for the host's record of the level.
constexpr int TL_ROOT_THREADS = 1024;
__global__ void __launch_bounds__(TL_ROOT_THREADS, 1) tl_root_claim(const void* level, int base, int s,
                                                                  const uint64_t* point, ulonglong2* scratch,
                                                                  TlTree* T, uint64_t* out) {
    ulonglong2* buf[2] = {scratch, scratch + (1ull << (s - 1))};
    for (int c = 0; c < s; c++) {
        const uint64_t m = 1ull << (s - c - 1);  // entries after this fold
        const fp2 t = {point[2 * c], point[2 * c + 1]};
        const uint64_t t7 = lz::mul7(t.c1);
        const ulonglong2* src = c ? buf[(c - 1) & 1] : static_cast<const ulonglong2*>(level);
        ulonglong2* dst = buf[c & 1];
        for (uint64_t k = threadIdx.x; k < m; k += blockDim.x) {
            fp2 a, b;
            if (c == 0 && base) {
                const ulonglong2 w = src[k];  // prime-field words 2k, 2k + 1
                a = {w.x, 0}, b = {w.y, 0};
            } else {
                a = ld2(src + 2 * k), b = ld2(src + 2 * k + 1);
            }
            const fp2 v = l2_fma(a, t, t7, l2_sub(b, a));
            dst[k] = make_ulonglong2(v.c0, v.c1);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const fp2 v = l2_canon(ld2(buf[(s - 1) & 1]));
        T->Q[0] = v.c0, T->Q[1] = v.c1;
        T->S[0] = v.c0, T->S[1] = v.c1;
        out[0] = v.c0, out[1] = v.c1;
    }
}

// A segment's whole sum by one block (its chunks one after another); each variant is its own
// function, so that the tail kernel's registers are those of the variant it calls.
template <int NT, int KIND, int MODE, bool ONE>
__device__ __noinline__ void tl_sum_block(const TlSeg& g, fp2 (&acc)[3]) {
    tl_sum<NT, KIND, MODE, ONE>(g, 0, acc);
}

template <bool ONE>
__device__ void tl_sum_any(const TlSeg& g, fp2 (&acc)[3]) {
    switch (tl_key(g.kind, g.mode)) {
        case tl_key(0, TL_SUM): tl_sum_block<2, 0, TL_SUM, ONE>(g, acc); break;
        case tl_key(0, TL_BIND_BASE): tl_sum_block<2, 0, TL_BIND_BASE, ONE>(g, acc); break;
        case tl_key(0, TL_SUM_BASE): tl_sum_block<2, 0, TL_SUM_BASE, ONE>(g, acc); break;
        case tl_key(0, TL_BIND): tl_sum_block<2, 0, TL_BIND, ONE>(g, acc); break;
        case tl_key(1, TL_SUM): tl_sum_block<4, 1, TL_SUM, ONE>(g, acc); break;
        case tl_key(1, TL_BIND): tl_sum_block<4, 1, TL_BIND, ONE>(g, acc); break;
        case tl_key(2, TL_SUM): tl_sum_block<2, 2, TL_SUM, ONE>(g, acc); break;
        case tl_key(2, TL_BIND): tl_sum_block<2, 2, TL_BIND, ONE>(g, acc); break;
        default: break;
    }
}

// A level's small rounds, j0 to the last, run by one block with no launch between them.
struct TlTail {
    FsJob jb;
    FsKeys keys;
    FsState* st;
    TlTree* trees;
    ulonglong2* q;
    uint64_t* rounds_out;
    uint64_t* chal_out;
    const TlSeg* segs;     // the tail rounds' segments, in round order (one block each: nblocks = 1)
    const int* first;      // round j0 + t's segments are segs[first[t] .. first[t + 1])
    const uint8_t* one;    // round j0 + t sums q(1)
    int ntrees, j0, rounds, pad_;
};

// Each round sums its segments with the whole block, then warp 0 runs the round's transcript,
// whose challenge the next round binds (the barrier between them orders the block's memory).
__global__ void __launch_bounds__(TL_THREADS, 1) tl_tail(const TlTail* A) {
    __shared__ TlSeg g;
    __shared__ uint64_t red[TL_THREADS / 32][6];
    __shared__ uint32_t sbuf[FS_BUF_WORDS];
    const int rounds = A->rounds;
    for (int t = 0; t < rounds; t++) {
        const bool one = A->one[t];
        for (int si = A->first[t]; si < A->first[t + 1]; si++) {
            if (threadIdx.x < (int)(sizeof(TlSeg) / 8))
                reinterpret_cast<uint64_t*>(&g)[threadIdx.x] = reinterpret_cast<const uint64_t*>(A->segs + si)[threadIdx.x];
            __syncthreads();
            fp2 acc[3] = {{0, 0}, {0, 0}, {0, 0}};
            if (one)
                tl_sum_any<true>(g, acc);
            else
                tl_sum_any<false>(g, acc);
            if (g.kind == 2) tl_unit_scale(g, acc);
            uint64_t words[6];
            for (int i = 0; i < 3; i++) {
                const fp2 c = l2_canon(acc[i]);
                words[2 * i] = c.c0, words[2 * i + 1] = c.c1;
            }
            tl_block_sum(words, red);
            if (threadIdx.x == 0) {
                tl_unit_finish(g, words);
                for (int w = 0; w < 6; w++) reinterpret_cast<uint64_t*>(g.out)[w] = words[w];
            }
            __syncthreads();
        }
        if (threadIdx.x < 32)
            tl_fs_round(A->st, A->jb, A->j0 + t, A->keys, A->trees, A->ntrees, A->q, A->rounds_out, A->chal_out,
                                    sbuf);
        __syncthreads();
    }
}

// The last bind: each table of two entries (2·stride apart) into one, by r, as the evaluations
// (src null: the constant 1 of numerators of 1).
struct TlFinal {
    const void* src;
    int stride, base;
    ulonglong2* out;
};
__global__ void tl_bind_last(const TlFinal* f, int n, const uint64_t* r) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const fp2 rr = {r[0], r[1]};
    fp2 a = {1, 0}, b = {1, 0};
    if (f[i].src && f[i].base) {
        const uint64_t* w = static_cast<const uint64_t*>(f[i].src);
        a = {lz::canon(w[0]), 0};
        b = {lz::canon(w[f[i].stride]), 0};
    } else if (f[i].src) {
        const ulonglong2* v = static_cast<const ulonglong2*>(f[i].src);
        a = l2_canon(ld2(v));
        b = l2_canon(ld2(v + f[i].stride));
    }
    const fp2 v = e_add(a, e_mul(rr, e_sub(b, a)));
    *f[i].out = make_ulonglong2(v.c0, v.c1);
}

}  // namespace tg

using namespace tg;

struct tg_leaf_stage {
    Device* d = nullptr;
    std::vector<TreeLevels> trees;
    int H = 0, level = 0;
    // per tree: the eq table, its point and high part, and the halves of the level below, sized
    // once for the tree's deepest level so that no level allocates
    std::vector<std::vector<std::unique_ptr<DevBuf>>> pool;
    DevBuf misc;  // a level's points, eq tables, segments, transcript and outputs
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
        if (t.kind == 1 && t.base_leaves) return fail(TG_ERR_INVALID, "tree %d: prime-field leaves are a forest's", k);
        if (t.kind == 0 && !t.leaves) return fail(TG_ERR_INVALID, "tree %d: null leaves", k);
        if (t.kind == 1 && !t.denominators) return fail(TG_ERR_INVALID, "tree %d: null denominators", k);
        if (t.gen) {
            if (t.kind != 1) return fail(TG_ERR_INVALID, "tree %d: generated leaves are a fraction tree's", k);
            if (!on_device) return fail(TG_ERR_INVALID, "tree %d: generated leaves go to device buffers", k);
            if (((uintptr_t)t.denominators & 15) || ((uintptr_t)t.leaves & 15))
                return fail(TG_ERR_INVALID, "tree %d: generated leaves need 16-byte aligned buffers", k);
            if ((t.leaves == nullptr) != (t.gen->unit != 0))
                return fail(TG_ERR_INVALID, "tree %d: numerators buffer %s for %s numerators", k, t.leaves ? "given" : "missing",
                            t.gen->unit ? "unit" : "generated");
            if (t.gen->alpha[0] >= P || t.gen->alpha[1] >= P || t.gen->beta[0] >= P || t.gen->beta[1] >= P)
                return fail(TG_ERR_INVALID, "tree %d: alpha and beta must be canonical", k);
        }
    }
    tg_leaf_stage* st = new tg_leaf_stage();
    st->d = d;
    st->trees.resize(ntrees);
    cudaStream_t s = d->stream;
    auto bail = [&](int rc) {
        tg_leaf_stage_close(st);
        return rc;
    };
    std::lock_guard<std::mutex> lock(d->mu);
    for (int k = 0; k < ntrees; k++) {
        const tg_tree& spec = specs[k];
        TreeLevels& tr = st->trees[k];
        tr.kind = spec.kind;
        tr.s = spec.s;
        tr.h = spec.height;
        tr.base = spec.kind == 0 && spec.base_leaves;
        st->H = std::max<int>(st->H, (int)spec.height);
        const uint32_t lg = spec.s + spec.height;
        const size_t es = tr.base ? 8 : 16;  // bytes an entry
        for (uint32_t l = 0; l <= spec.height; l++) {
            tr.n.emplace_back(new DevBuf());
            tr.d.emplace_back(new DevBuf());
        }
        const uint64_t leaves = 1ull << lg;
        // the leaf level: device leaves in place (when 16-byte aligned), else a copy
        auto place = [&](DevBuf& b, const uint64_t* src) -> int {
            if (on_device && ((uintptr_t)src & 15) == 0) {
                b.ptr = (void*)src;
                b.bytes = leaves * es;
                b.owned = false;
                return TG_OK;
            }
            const int rc = spare_take(d, b, leaves * es);
            if (rc) return rc;
            if (!on_device) host_prefault(src, leaves * es);
            TG_CUDA(cudaMemcpyAsync(b.ptr, src, leaves * es, on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s));
            return TG_OK;
        };
        int rc = TG_OK;
        if (spec.kind == 0) {
            rc = place(*tr.n[spec.height], spec.leaves);
        } else {
            rc = place(*tr.d[spec.height], spec.denominators);
            tr.unit = !spec.leaves;
            if (!rc && spec.leaves) rc = place(*tr.n[spec.height], spec.leaves);
        }
        if (rc) return bail(rc);
        // generated leaves: in the same pass as the two levels above them, or alone for a tree of
        // height below 2
        const bool gen_fused = spec.gen && spec.height >= 2;
        const LeafGen lg_spec = spec.gen ? leaf_gen(*spec.gen) : LeafGen{};
        if (spec.gen && !gen_fused) {
            Launch L(d, s, "logup_leaves", 1, leaves);
            tr_logup_leaves<<<grid_of(d, leaves), 256, 0, s>>>(lg_spec, spec.leaves ? (ulonglong2*)tr.n[spec.height]->ptr : nullptr,
                                                              (ulonglong2*)tr.d[spec.height]->ptr, leaves);
            TG_CUDA(cudaGetLastError());
        }
        // levels two at a time (l and l − 1 from l + 1), the last one alone when the count is odd
        for (int l = (int)spec.height - 1; l >= 0;) {
            const bool two = l >= 1;
            const uint64_t m = 1ull << (spec.s + l);  // entries of level l
            for (int t = 0; t < (two ? 2 : 1); t++) {
                const uint64_t mt = m >> t;
                rc = spare_take(d, *tr.n[l - t], mt * es);
                if (!rc && spec.kind == 1) rc = spare_take(d, *tr.d[l - t], mt * es);
                if (rc) return bail(rc);
            }
            const ulonglong2* nb = tr.unit && l + 1 == (int)spec.height ? nullptr : (const ulonglong2*)tr.n[l + 1]->ptr;
            Launch L(d, s, spec.kind ? "tree_fraction_level" : "tree_product_level", 1, m);
            if (two) {
                const uint64_t mo = m / 2;  // entries of level l − 1, one per thread
                if (spec.kind == 0 && tr.base)
                    tr_product_level2_base<<<grid_of(d, mo), 256, 0, s>>>(
                        (const ulonglong2*)tr.n[l + 1]->ptr, (ulonglong2*)tr.n[l]->ptr, (uint64_t*)tr.n[l - 1]->ptr, mo);
                else if (spec.kind == 0)
                    tr_product_level2<<<grid_of(d, mo), 256, 0, s>>>((const ulonglong2*)tr.n[l + 1]->ptr,
                                                                    (ulonglong2*)tr.n[l]->ptr, (ulonglong2*)tr.n[l - 1]->ptr, mo);
                else if (gen_fused && l + 1 == (int)spec.height)
                    tr_logup_level2<<<grid_of(d, mo), 256, 0, s>>>(
                        lg_spec, spec.leaves ? (ulonglong2*)tr.n[l + 1]->ptr : nullptr, (ulonglong2*)tr.d[l + 1]->ptr,
                        (ulonglong2*)tr.n[l]->ptr, (ulonglong2*)tr.d[l]->ptr, (ulonglong2*)tr.n[l - 1]->ptr,
                        (ulonglong2*)tr.d[l - 1]->ptr, mo);
                else
                    tr_fraction_level2<<<grid_of(d, mo), 256, 0, s>>>(
                        nb, (const ulonglong2*)tr.d[l + 1]->ptr, (ulonglong2*)tr.n[l]->ptr, (ulonglong2*)tr.d[l]->ptr,
                        (ulonglong2*)tr.n[l - 1]->ptr, (ulonglong2*)tr.d[l - 1]->ptr, mo);
            } else if (spec.kind == 0 && tr.base) {
                tr_product_level_base<<<grid_of(d, m), 256, 0, s>>>((const ulonglong2*)tr.n[l + 1]->ptr,
                                                                   (uint64_t*)tr.n[l]->ptr, m);
            } else if (spec.kind == 0) {
                tr_product_level<<<grid_of(d, m), 256, 0, s>>>((const ulonglong2*)tr.n[l + 1]->ptr, (ulonglong2*)tr.n[l]->ptr, m);
            } else {
                tr_fraction_level<<<grid_of(d, m), 256, 0, s>>>(nb, (const ulonglong2*)tr.d[l + 1]->ptr,
                                                               (ulonglong2*)tr.n[l]->ptr, (ulonglong2*)tr.d[l]->ptr, m);
            }
            TG_CUDA(cudaGetLastError());
            l -= two ? 2 : 1;
        }
        // the root level on the host
        const uint64_t r = 1ull << spec.s;
        std::vector<uint64_t> w(2 * r);
        if (spec.kind == 1 && spec.height == 0 && tr.unit) {  // a single leaf of numerator 1
            w[0] = 1, w[1] = 0;
        } else {
            TG_CUDA(cudaMemcpyAsync(w.data(), tr.n[0]->ptr, r * es, cudaMemcpyDeviceToHost, s));
            TG_CUDA(cudaStreamSynchronize(s));
        }
        for (uint64_t i = 0; i < r; i++) tr.root.push_back(tr.base ? fp2{w[i], 0} : fp2{w[2 * i], w[2 * i + 1]});
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
    // per tree and table, the bound tables of its deepest level (n = s + h − 1 variables): A holds
    // 2^(n−1) entries (own rounds 1, 3, …), B 2^(n−2) (own rounds 2, 4, …)
    st->pool.resize(ntrees);
    for (int k = 0; k < ntrees; k++) {
        const TreeLevels& tr = st->trees[k];
        const int n = (int)(tr.s + tr.h) - 1;
        const int nt = tr.kind ? 4 : 2;
        for (int t2 = 0; t2 < nt; t2++)
            for (int ab = 0; ab < 2; ab++) {
                st->pool[k].emplace_back(new DevBuf());
                const size_t entries = n - 1 - ab >= 0 ? (1ull << (n - 1 - ab)) : 1;
                const int rc = spare_take(d, *st->pool[k].back(), entries * 16);
                if (rc) return bail(rc);
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
    std::vector<char> root_on_device(ntrees, 0);
    for (int k : present) {
        TreeLevels& tr = st->trees[k];
        if (tr.own >= 0) {
            jpoint[k] = tr.point;
            jvalue[k] = tr.value;
            jp[k] = tr.p;
            jq[k] = tr.q;
        } else if (tr.kind == 0) {
            jpoint[k].assign(rootc.begin() + (s_max - tr.s), rootc.end());
            if (tr.s >= TL_ROOT_DEVICE_LOG)
                root_on_device[k] = 1;  // folded on the device before the rounds (tl_root_claim)
            else
                jvalue[k] = host_mle(tr.root, jpoint[k]);
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

    // each present tree's claim on the level: a forest's value, a fraction tree's p + λ·q, as the
    // verifier holds it (held: a joining fraction tree's from its sent root) and as the prover
    // sums it (own: from the tree's own root, which the rounds' q(1) and padding derive from)
    const int np = (int)present.size();
    std::vector<fp2> held(np), own_claim(np);
    for (int i = 0; i < np; i++) {
        const int k = present[i];
        const TreeLevels& tr = st->trees[k];
        held[i] = tr.kind == 0 ? jvalue[k] : e_add(jp[k], e_mul(lambda, jq[k]));
        own_claim[i] = tr.kind == 1 && tr.own < 0 ? e_add(tr.root[0], e_mul(lambda, tr.root[1])) : held[i];
    }

    // ---- the level's sumcheck on the device (TlSeg rounds, tl_fs transcript, tl_bind_last)
    cudaStream_t s = d->stream;
    std::vector<int> nvars(np), pads(np);
    int n_max = 0;
    for (int i = 0; i < np; i++) n_max = std::max(n_max, nvars[i] = (int)jpoint[present[i]].size());
    for (int i = 0; i < np; i++) pads[i] = n_max - nvars[i];
    const int seg_cap = std::min(1024, 4 * d->sm_count);
    auto blocks_for = [&](uint64_t n) {
        return (int)std::max<uint64_t>(1, std::min<uint64_t>((n + TL_THREADS - 1) / TL_THREADS, seg_cap));
    };
    // the level block: points | eq tables | eq jobs | trees | q | segments | finals | partials |
    // counters | FsState | rounds | challenges | evaluations
    Arena ar;
    std::vector<size_t> off_point(np), off_tinv(np), off_eq(np);
    std::vector<std::vector<std::pair<uint64_t, uint64_t>>> eqtab(np);  // per own round: (lo offset, hi offset) in entries
    std::vector<TlEqJob> eqjobs;
    uint64_t eq_total = 0;
    for (int i = 0; i < np; i++) {
        const int n = nvars[i];
        off_point[i] = ar.take((size_t)std::max(n, 1) * 16);
        off_tinv[i] = ar.take((size_t)std::max(n, 1) * 16);
        uint64_t entries = 0;
        for (int jj = 0; jj < n; jj++) {
            const int rem = n - jj - 1, nl = tl_low_bits(rem), nh = rem - nl;
            eqtab[i].push_back({entries, entries + (1ull << nl)});
            entries += (1ull << nl) + (1ull << nh);
        }
        off_eq[i] = entries;  // the entry count for now; the tables go after everything uploaded
        eq_total += entries;
    }
    const size_t off_jobs = ar.take(sizeof(TlEqJob) * std::max<size_t>(2 * np * 64, 1));
    const size_t off_trees = ar.take(sizeof(TlTree) * np);
    const size_t off_q = ar.take((size_t)64 * np);
    // segments: launch 0 is every tree's own round 0, launch j (1 ≤ j < n_max) the trees in own rounds ≥ 1
    std::vector<std::vector<TlSeg>> launches(std::max(n_max, 1));
    std::vector<std::vector<std::pair<int, int>>> owners(std::max(n_max, 1));  // (tree i, own round jj)
    std::vector<TlFinal> finals;
    auto table_src = [&](int i, int jj, int k, int* stride, int* base) -> const void* {
        // the tables own round jj reads: the level below (jj ≤ 1; prime-field words for a
        // prime-field forest), else round jj − 1's bound output
        TreeLevels& tr = st->trees[present[i]];
        const int own = tr.own >= 0 ? tr.own : 0;
        if (jj <= 1) {
            *stride = 2;
            *base = tr.base;
            const DevBuf& lv = (tr.kind == 1 && k >= 2) ? *tr.d[own + 1] : *tr.n[own + 1];
            if (tr.base) return (const uint64_t*)lv.ptr + (k & 1);
            return (const ulonglong2*)lv.ptr + (k & 1);
        }
        *stride = 1;
        *base = 0;
        return st->pool[present[i]][2 * k + ((jj - 2) & 1)]->ptr;
    };
    // where a point coordinate is 0, q(1) has no derivation from the claim: that round's launch sums
    // it (every round's does under TG_TREE_SUM_Q1, which takes the summed q(1) throughout)
    const bool sum_q1 = (d->cfg.tree_flags & TG_TREE_SUM_Q1) != 0;
    std::vector<char> one(std::max(n_max, 1), sum_q1 ? 1 : 0);
    for (int i = 0; i < np; i++)
        for (int jj = 0; jj < nvars[i]; jj++) {
            const fp2 c = jpoint[present[i]][jj];
            if (c.c0 == 0 && c.c1 == 0) one[jj == 0 ? 0 : jj + pads[i]] = 1;
        }
    // a fraction tree whose leaves have numerators of 1, at the level right above its leaves:
    // N0 and N1 stay 1 through every bind, so only D0 and D1 are tables
    auto unit_level = [&](int i) {
        const TreeLevels& tr = st->trees[present[i]];
        const int own = tr.own >= 0 ? tr.own : 0;
        return tr.kind == 1 && tr.unit && own + 1 == (int)tr.h;
    };
    size_t total_segs = 0, max_blocks = 1, max_segs = 1;
    for (int j = 0; j < std::max(n_max, 1); j++) {
        int block0 = 0;
        for (int i = 0; i < np; i++) {
            const int jj = j == 0 ? 0 : j - pads[i];
            if (j > 0 && jj < 1) continue;
            if (nvars[i] == 0 || jj >= nvars[i]) continue;
            TreeLevels& tr = st->trees[present[i]];
            const bool unit = unit_level(i);
            const int nt = unit ? 2 : tr.kind ? 4 : 2;
            TlSeg g;
            memset(&g, 0, sizeof g);
            g.kind = unit ? 2 : tr.kind;
            g.bind = jj >= 1;
            int base = 0;
            for (int k = 0; k < nt; k++) {
                const int tk = unit ? k + 2 : k;  // the unit kind's tables are D0 and D1
                g.src[k] = table_src(i, jj, tk, &g.stride, &base);
                if (g.bind) g.dst[k] = (ulonglong2*)st->pool[present[i]][2 * tk + ((jj - 1) & 1)]->ptr;
            }
            g.mode = base ? (g.bind ? TL_BIND_BASE : TL_SUM_BASE) : (g.bind ? TL_BIND : TL_SUM);
            g.n = 1ull << (nvars[i] - jj - 1);
            g.lam[0] = lambda.c0, g.lam[1] = lambda.c1;
            if (g.kind == 2 && !(lambda.c0 == 0 && lambda.c1 == 0)) {
                const fp2 mu = host_inv2(lambda);
                g.mu[0] = mu.c0, g.mu[1] = mu.c1;
                g.shift = 1;
            }
            g.lbits = tl_low_bits(nvars[i] - jj - 1);
            g.nblocks = (int)std::min<uint64_t>(blocks_for(g.n), g.n >> g.lbits);
            launches[j].push_back(g);
            owners[j].push_back({i, jj});
        }
        // one kernel per kind and mode: the round's segments grouped by key, blocks numbered
        // within each group (the groups run one after another and share partials and counters)
        {
            std::vector<size_t> order(launches[j].size());
            for (size_t q = 0; q < order.size(); q++) order[q] = q;
            std::stable_sort(order.begin(), order.end(), [&](size_t x, size_t y) {
                return tl_key(launches[j][x].kind, launches[j][x].mode) < tl_key(launches[j][y].kind, launches[j][y].mode);
            });
            std::vector<TlSeg> segs2;
            std::vector<std::pair<int, int>> own2;
            for (size_t q : order) segs2.push_back(launches[j][q]), own2.push_back(owners[j][q]);
            launches[j].swap(segs2);
            owners[j].swap(own2);
            for (size_t q = 0; q < launches[j].size(); q++) {
                TlSeg& g = launches[j][q];
                if (q == 0 || tl_key(g.kind, g.mode) != tl_key(launches[j][q - 1].kind, launches[j][q - 1].mode))
                    block0 = 0;
                g.block0 = g.part0 = block0;
                block0 += g.nblocks;
                max_blocks = std::max(max_blocks, (size_t)block0);
            }
        }
        total_segs += launches[j].size();
        max_segs = std::max(max_segs, launches[j].size());
    }
    // the tail: the last rounds, from the first whose segments all have at most TL_TAIL_PAIRS pairs,
    // run in one block (each segment one block's work)
    int j0 = std::max(n_max, 1);
    for (int j = (int)launches.size() - 1; j >= 0; j--) {
        uint64_t most = 0;
        for (const TlSeg& g : launches[j]) most = std::max(most, g.n);
        if (most > TL_TAIL_PAIRS) break;
        j0 = j;
    }
    size_t tail_seg0 = 0;
    for (int j = 0; j < j0 && j < (int)launches.size(); j++) tail_seg0 += launches[j].size();
    for (int j = j0; j < (int)launches.size(); j++)
        for (TlSeg& g : launches[j]) g.nblocks = 1, g.block0 = g.part0 = 0;
    const int tail_rounds = n_max > 0 ? n_max - j0 : 0;
    const size_t off_tail = ar.take(sizeof(TlTail));
    const size_t off_tail_first = ar.take(4 * ((size_t)tail_rounds + 1));
    const size_t off_tail_one = ar.take((size_t)tail_rounds + 1);
    const size_t off_segs = ar.take(sizeof(TlSeg) * std::max<size_t>(total_segs, 1));
    const size_t off_finals = ar.take(sizeof(TlFinal) * 4 * np);
    const size_t off_partials = ar.take(max_blocks * 64);
    const size_t off_counters = ar.take(4 * max_segs);
    const size_t off_fs = ar.take(sizeof(FsState));
    const size_t off_rounds = ar.take((size_t)std::max(n_max, 1) * 48);
    const size_t off_chal = ar.take((size_t)std::max(n_max, 1) * 16);
    const size_t off_evals = ar.take((size_t)64 * np);
    // the device root claims: one output pair per present tree, and the fold's scratch
    const size_t off_rootc = ar.take((size_t)16 * np);
    uint64_t root_scratch = 1;
    for (int i = 0; i < np; i++)
        if (root_on_device[present[i]]) root_scratch = std::max<uint64_t>(root_scratch, (3ull << st->trees[present[i]].s) / 4);
    const size_t off_rscratch = ar.take(root_scratch * 16);
    const size_t upload_bytes = ar.used;  // the eq tables, built on the device, follow
    for (int i = 0; i < np; i++) off_eq[i] = ar.take(std::max<uint64_t>(off_eq[i], 1) * 16);
    if (ar.used > st->misc.bytes) {  // grows geometrically, through the workspace cache: the levels
        // grow one after another, and a repeated proof of the same shape finds every size cached
        const size_t want = std::max(ar.used, 2 * st->misc.bytes);
        spare_give(d, st->misc);
        const int rc2 = spare_take(d, st->misc, want);
        if (rc2) return bail(rc2);
    }
    ar.base = (uint8_t*)st->misc.ptr;

    // host staging of everything the level uploads
    std::vector<uint8_t> up(upload_bytes, 0);
    auto host_at = [&](size_t off) { return up.data() + off; };
    std::vector<TlTree> ttrees(np);
    fp2 gi = {1, 0};
    for (int i = 0; i < np; i++) {
        const std::vector<fp2>& pt = jpoint[present[i]];
        uint64_t* pw = (uint64_t*)host_at(off_point[i]);
        uint64_t* iw = (uint64_t*)host_at(off_tinv[i]);
        for (size_t c = 0; c < pt.size(); c++) {
            pw[2 * c] = pt[c].c0, pw[2 * c + 1] = pt[c].c1;
            const fp2 ti = sum_q1 ? fp2{0, 0} : host_inv2(pt[c]);  // 0: tl_quad reads the summed q(1)
            iw[2 * c] = ti.c0, iw[2 * c + 1] = ti.c1;
        }
        const uint64_t* dpt = ar.at<uint64_t>(off_point[i]);
        for (int jj = 0; jj < nvars[i]; jj++) {  // round jj's weights over p[jj+1 ..]
            const int rem = nvars[i] - jj - 1, nl = tl_low_bits(rem), nh = rem - nl;
            ulonglong2* base = ar.at<ulonglong2>(off_eq[i]);
            eqjobs.push_back({dpt + 2 * (jj + 1), nl, base + eqtab[i][jj].first, 1ull << nl});
            eqjobs.push_back({dpt + 2 * (jj + 1 + nl), nh, base + eqtab[i][jj].second, 1ull << nh});
        }
        TlTree& T = ttrees[i];
        memset(&T, 0, sizeof T);
        T.w[0] = gi.c0, T.w[1] = gi.c1;
        T.C[0] = 1;
        T.Q[0] = own_claim[i].c0, T.Q[1] = own_claim[i].c1;
        T.S[0] = own_claim[i].c0, T.S[1] = own_claim[i].c1;
        T.point = dpt;
        T.tinv = ar.at<uint64_t>(off_tinv[i]);
        T.n = nvars[i];
        T.pad = pads[i];
        gi = e_mul(gi, gamma);
        // the final evaluations of its tables
        TreeLevels& tr = st->trees[present[i]];
        const int nt = tr.kind ? 4 : 2;
        for (int k = 0; k < nt; k++) {
            TlFinal f;
            memset(&f, 0, sizeof f);
            const int n = nvars[i];
            if (unit_level(i) && k < 2) {  // numerators of 1 stay 1
                f.src = nullptr;
            } else if (n == 0) {  // the entry itself
                f.src = table_src(i, 0, k, &f.stride, &f.base);
                f.stride = 0;
            } else {
                f.src = table_src(i, n - 1 >= 1 ? n : 1, k, &f.stride, &f.base);
            }
            f.out = ar.at<ulonglong2>(off_evals) + finals.size();
            finals.push_back(f);
        }
    }
    // segments' eq tables, outputs and challenge pointers, now that the block's addresses are known
    {
        size_t at = 0;
        FsState* dfs = ar.at<FsState>(off_fs);
        for (int j = 0; j < (int)launches.size(); j++)
            for (size_t q = 0; q < launches[j].size(); q++) {
                TlSeg& g = launches[j][q];
                const int i = owners[j][q].first, jj = owners[j][q].second;
                ulonglong2* base = ar.at<ulonglong2>(off_eq[i]);
                g.lo = base + eqtab[i][jj].first;
                g.hi = base + eqtab[i][jj].second;
                g.out = ar.at<ulonglong2>(off_q) + 4 * i;
                g.r = dfs->r;
                memcpy(host_at(off_segs) + sizeof(TlSeg) * at++, &g, sizeof g);
            }
    }
    if (!eqjobs.empty()) memcpy(host_at(off_jobs), eqjobs.data(), sizeof(TlEqJob) * eqjobs.size());
    memcpy(host_at(off_trees), ttrees.data(), sizeof(TlTree) * np);
    if (!finals.empty()) memcpy(host_at(off_finals), finals.data(), sizeof(TlFinal) * finals.size());
    {
        FsState fs0;
        memset(&fs0, 0, sizeof fs0);
        memcpy(fs0.state, t->state, 32);
        fs0.counter = t->counter;
        memcpy(host_at(off_fs), &fs0, sizeof fs0);
    }
    FsJob jb;
    memset(&jb, 0, sizeof jb);
    jb.label_len = (int)prefix.size();
    memcpy(jb.label, prefix.data(), prefix.size());
    FsKeys keys;
    context_key("transcript-absorb", keys.absorb);
    context_key("transcript-squeeze", keys.squeeze);
    context_key("transcript-ratchet", keys.ratchet);
    if (tail_rounds > 0) {
        TlTail tl;
        memset(&tl, 0, sizeof tl);
        tl.jb = jb;
        tl.keys = keys;
        tl.st = ar.at<FsState>(off_fs);
        tl.trees = ar.at<TlTree>(off_trees);
        tl.q = ar.at<ulonglong2>(off_q);
        tl.rounds_out = ar.at<uint64_t>(off_rounds);
        tl.chal_out = ar.at<uint64_t>(off_chal);
        tl.segs = ar.at<TlSeg>(off_segs) + tail_seg0;
        tl.first = ar.at<int>(off_tail_first);
        tl.one = ar.at<uint8_t>(off_tail_one);
        tl.ntrees = np;
        tl.j0 = j0;
        tl.rounds = tail_rounds;
        memcpy(host_at(off_tail), &tl, sizeof tl);
        int* first = (int*)host_at(off_tail_first);
        uint8_t* onef = host_at(off_tail_one);
        first[0] = 0;
        for (int t2 = 0; t2 < tail_rounds; t2++) {
            first[t2 + 1] = first[t2] + (int)launches[j0 + t2].size();
            onef[t2] = (uint8_t)one[j0 + t2];
        }
    }

    std::vector<uint64_t> rounds((size_t)std::max(n_max, 1) * 6), chal((size_t)std::max(n_max, 1) * 2),
        fevals(8 * (size_t)np), rootc_host(2 * (size_t)np);
    FsState fs1;
    {
        std::lock_guard<std::mutex> lock(d->mu);
        TG_CUDA(cudaMemcpyAsync(ar.base, up.data(), up.size(), cudaMemcpyHostToDevice, s));
        for (int i = 0; i < np; i++) {
            if (!root_on_device[present[i]]) continue;
            const TreeLevels& tr = st->trees[present[i]];
            Launch L(d, s, "tree_root_claim", 1, 1ull << tr.s);
            tl_root_claim<<<1, TL_ROOT_THREADS, 0, s>>>(tr.n[0]->ptr, tr.base, (int)tr.s, ar.at<uint64_t>(off_point[i]),
                                                        ar.at<ulonglong2>(off_rscratch), ar.at<TlTree>(off_trees) + i,
                                                        ar.at<uint64_t>(off_rootc) + 2 * i);
            TG_CUDA(cudaGetLastError());
        }
        if (eq_total) {
            Launch L(d, s, "tree_eq", 1, eq_total);
            tl_eq_tables<<<grid_of(d, eq_total), 256, 0, s>>>(ar.at<TlEqJob>(off_jobs), (int)eqjobs.size(), eq_total);
            TG_CUDA(cudaGetLastError());
        }
        size_t seg0 = 0;
        auto run = [&](int j) -> int {
            const auto& L0 = launches[j];
            size_t q0 = 0;
            while (q0 < L0.size()) {  // one launch per group of one key
                const int key = tl_key(L0[q0].kind, L0[q0].mode);
                size_t q1 = q0;
                int blocks = 0;
                uint64_t units = 0;
                while (q1 < L0.size() && tl_key(L0[q1].kind, L0[q1].mode) == key) blocks += L0[q1].nblocks, units += L0[q1].n, q1++;
                Launch L(d, s, "tree_level_round", 1, units);
                const TlSeg* segs = ar.at<TlSeg>(off_segs) + seg0 + q0;
                if (one[j])
                    tl_launch<true>(key, blocks, s, segs, (int)(q1 - q0), ar.at<uint64_t>(off_partials),
                                    ar.at<unsigned>(off_counters));
                else
                    tl_launch<false>(key, blocks, s, segs, (int)(q1 - q0), ar.at<uint64_t>(off_partials),
                                     ar.at<unsigned>(off_counters));
                TG_CUDA(cudaGetLastError());
                q0 = q1;
            }
            seg0 += L0.size();
            return TG_OK;
        };
        TG_CUDA(cudaMemsetAsync(ar.at<unsigned>(off_counters), 0, 4 * max_segs, s));
        for (int j = 0; j < std::min(n_max, j0); j++) {
            rc = run(j);
            if (rc) return bail(rc);
            Launch L(d, s, "tree_level_transcript", 1, 1);
            tl_fs<<<1, 32, 0, s>>>(ar.at<FsState>(off_fs), jb, j, keys, ar.at<TlTree>(off_trees), np,
                                   ar.at<ulonglong2>(off_q), ar.at<uint64_t>(off_rounds), ar.at<uint64_t>(off_chal));
            TG_CUDA(cudaGetLastError());
        }
        if (tail_rounds > 0) {
            uint64_t units = 0;
            for (int j = j0; j < n_max; j++)
                for (const TlSeg& g : launches[j]) units += g.n;
            Launch L(d, s, "tree_level_tail", 1, units);
            tl_tail<<<1, TL_THREADS, 0, s>>>(ar.at<TlTail>(off_tail));
            TG_CUDA(cudaGetLastError());
        }
        if (!finals.empty()) {
            Launch L(d, s, "tree_level_evals", 1, finals.size());
            tl_bind_last<<<1, 128, 0, s>>>(ar.at<TlFinal>(off_finals), (int)finals.size(), ar.at<FsState>(off_fs)->r);
            TG_CUDA(cudaGetLastError());
        }
        // the outputs lie back to back in the block (state, messages, challenges, evaluations, root
        // claims): one copy into pinned memory and one wait, not a round trip each
        const size_t out_lo = off_fs, out_bytes = off_rootc + 16 * (size_t)np - off_fs;
        rc = readback_ensure(d, out_bytes);
        if (rc) return bail(rc);
        TG_CUDA(cudaMemcpyAsync(d->readback, ar.base + out_lo, out_bytes, cudaMemcpyDeviceToHost, s));
        TG_CUDA(cudaStreamSynchronize(s));
        auto from = [&](size_t off) { return d->readback + (off - out_lo); };
        memcpy(&fs1, from(off_fs), sizeof fs1);
        memcpy(rounds.data(), from(off_rounds), rounds.size() * 8);
        memcpy(chal.data(), from(off_chal), chal.size() * 8);
        memcpy(fevals.data(), from(off_evals), finals.size() * 16);
        memcpy(rootc_host.data(), from(off_rootc), 16 * (size_t)np);
    }
    for (int i = 0; i < np; i++)  // the device root claims, for the record
        if (root_on_device[present[i]]) held[i] = jvalue[present[i]] = {rootc_host[2 * i], rootc_host[2 * i + 1]};
    if (fs1.err) return bail(fail(TG_ERR_STATE, "a level challenge found no canonical Fp2 in %d squeezes", FS_MAX_TRIES));
    memcpy(t->state, fs1.state, 32);
    t->counter = fs1.counter;
    std::vector<fp2> evals;
    for (size_t i = 0; i < finals.size(); i++) evals.push_back({fevals[2 * i], fevals[2 * i + 1]});
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
        for (int i = 0; i < np; i++) {
            c = e_add(c, e_mul(g, e_scale(held[i], (1ull << (n_max - nvars[i])) % P)));
            g = e_mul(g, gamma);
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
        spare_give(d, *tr.n[own]);  // the level above is no longer needed
        spare_give(d, *tr.d[own]);
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
    Device* d = st->d;
    cudaStreamSynchronize(d->stream);  // nothing of the stage in flight
    // the workspace goes back to the device's cache (zeroed when the cache returns it to the driver)
    for (auto& tr : st->trees)
        for (auto* v : {&tr.n, &tr.d})
            for (auto& b : *v) spare_give(d, *b);
    for (auto& tables : st->pool)
        for (auto& b : tables) spare_give(d, *b);
    spare_give(d, st->misc);
    delete st;
    return TG_OK;
}

extern "C" int tg_logup_leaves(tg_device* dev, uint64_t key_seed, uint64_t value_seed, int unit, uint64_t mult_seed,
                               const uint64_t alpha[2], const uint64_t beta[2], size_t count, uint64_t* numerators,
                               uint64_t* denominators) {
    Device* d = reinterpret_cast<Device*>(dev);
    if (!d || !alpha || !beta || (count && (!denominators || (!numerators && !unit))))
        return fail(TG_ERR_INVALID, "tg_logup_leaves: null argument");
    if (count == 0) return TG_OK;
    cudaStream_t s = d->stream;
    {
        Launch L(d, s, "logup_leaves", 1, count);
        tg_leaf_gen g;
        memset(&g, 0, sizeof g);
        g.key_seed = key_seed, g.value_seed = value_seed, g.mult_seed = mult_seed, g.unit = unit;
        g.alpha[0] = alpha[0], g.alpha[1] = alpha[1], g.beta[0] = beta[0], g.beta[1] = beta[1];
        tr_logup_leaves<<<grid_of(d, count), 256, 0, s>>>(leaf_gen(g), (ulonglong2*)numerators, (ulonglong2*)denominators,
                                                          count);
    }
    TG_CUDA(cudaGetLastError());
    TG_CUDA(cudaStreamSynchronize(s));
    return TG_OK;
}
