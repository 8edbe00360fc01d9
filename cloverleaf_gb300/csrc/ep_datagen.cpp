// ep_datagen.cpp -- the seeded synthetic workload generators of
// include/ep_datagen.h (SBM and Chung-Lu graphs, token and Zipf features).
//
// Built into its own library, libep_datagen.so, apart from the trainer
// (libep_gb300.so): the benchmark's CPU reference arm generates its workload
// here without loading any of the trainer's code.
//
// Plain C++17 + OpenMP; no CUDA.  Identical results on x86_64 and aarch64:
// no intrinsics, no floating-point contraction (built with
// -ffp-contract=off), and parallel loops draw from per-block RNG streams whose
// blocking does not depend on the thread count.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <memory>
#include <mutex>
#include <numeric>
#include <unordered_map>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../../include/ep_datagen.h"

// status codes of include/ep_datagen.h
#define EP_OK 0
#define EP_ERR_INVALID_ARG (-1)

namespace {

// ---------------------------------------------------------------------------
// RNG: splitmix64-seeded xoshiro256** (Blackman & Vigna), one stream per block.
// ---------------------------------------------------------------------------
inline uint64_t splitmix(uint64_t& x) {
    uint64_t z = (x += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}
inline uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

struct Rng {
    uint64_t s[4];
    Rng(uint64_t seed, uint64_t stream, uint64_t block) {
        uint64_t x = seed ^ (stream * 0xd1b54a32d192ed03ull) ^ (block * 0x8cb92ba72f3d8dd7ull);
        for (auto& v : s) v = splitmix(x);
    }
    uint64_t next() {
        const uint64_t r = rotl(s[1] * 5, 7) * 9, t = s[1] << 17;
        s[2] ^= s[0]; s[3] ^= s[1]; s[1] ^= s[2]; s[0] ^= s[3]; s[2] ^= t; s[3] = rotl(s[3], 45);
        return r;
    }
    double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
    uint64_t below(uint64_t n) {   // unbiased, Lemire-style rejection
        if (n <= 1) return 0;
        const uint64_t lim = (~0ull) - ((~0ull) % n);
        uint64_t x;
        do { x = next(); } while (x >= lim);
        return x % n;
    }
    uint32_t poisson(double lambda) {   // Knuth, fine for lambda <= ~30
        const double L = std::exp(-lambda);
        uint32_t k = 0;
        double p = 1.0;
        do { ++k; p *= uniform(); } while (p > L);
        return k - 1;
    }
};

inline uint64_t fmix64(uint64_t k) {
    k ^= k >> 33; k *= 0xff51afd7ed558ccdull; k ^= k >> 33; k *= 0xc4ceb9fe1a85ec53ull; k ^= k >> 33;
    return k;
}

// Walker/Vose alias table over non-negative weights.
struct Alias {
    std::vector<double> prob;
    std::vector<uint32_t> alias;
    explicit Alias(const std::vector<double>& w) {
        const size_t n = w.size();
        prob.resize(n);
        alias.resize(n);
        const double sum = std::accumulate(w.begin(), w.end(), 0.0);
        std::vector<uint32_t> small, large;
        std::vector<double> q(n);
        for (size_t i = 0; i < n; ++i) {
            q[i] = w[i] * (double)n / sum;
            (q[i] < 1.0 ? small : large).push_back((uint32_t)i);
        }
        while (!small.empty() && !large.empty()) {
            const uint32_t s = small.back(); small.pop_back();
            const uint32_t l = large.back(); large.pop_back();
            prob[s] = q[s];
            alias[s] = l;
            q[l] = (q[l] + q[s]) - 1.0;
            (q[l] < 1.0 ? small : large).push_back(l);
        }
        for (uint32_t i : large) { prob[i] = 1.0; alias[i] = i; }
        for (uint32_t i : small) { prob[i] = 1.0; alias[i] = i; }
    }
    uint32_t draw(Rng& r) const {
        const uint64_t i = r.below(prob.size());
        return r.uniform() < prob[i] ? (uint32_t)i : alias[i];
    }
};

// Builds a symmetric CSR from undirected pairs; rows sorted, duplicates and
// self loops dropped.  Weight per undirected edge from wfun(min, max).
template <typename WF>
void build_sym_csr(uint64_t n, const std::vector<uint32_t>& a, const std::vector<uint32_t>& b, WF wfun,
                   std::vector<uint64_t>& rows, std::vector<uint32_t>& cols, std::vector<float>& w) {
    const uint64_t m = a.size();
    std::vector<std::atomic<uint32_t>> deg(n);
    for (auto& d : deg) d.store(0, std::memory_order_relaxed);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)m; ++i) {
        if (a[i] == b[i]) continue;
        deg[a[i]].fetch_add(1, std::memory_order_relaxed);
        deg[b[i]].fetch_add(1, std::memory_order_relaxed);
    }
    std::vector<uint64_t> off(n + 1, 0);
    for (uint64_t v = 0; v < n; ++v) off[v + 1] = off[v] + deg[v].load(std::memory_order_relaxed);
    std::vector<uint32_t> tmp(off[n]);
    std::vector<std::atomic<uint64_t>> cur(n);
    for (uint64_t v = 0; v < n; ++v) cur[v].store(off[v], std::memory_order_relaxed);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)m; ++i) {
        if (a[i] == b[i]) continue;
        tmp[cur[a[i]].fetch_add(1, std::memory_order_relaxed)] = b[i];
        tmp[cur[b[i]].fetch_add(1, std::memory_order_relaxed)] = a[i];
    }
    // sort + unique per row (row contents are a deterministic multiset)
    std::vector<uint64_t> uniq(n + 1, 0);
#pragma omp parallel for schedule(dynamic, 4096)
    for (int64_t v = 0; v < (int64_t)n; ++v) {
        auto bgn = tmp.begin() + off[v], end = tmp.begin() + off[v + 1];
        std::sort(bgn, end);
        uniq[v + 1] = (uint64_t)(std::unique(bgn, end) - bgn);
    }
    rows.assign(n + 1, 0);
    for (uint64_t v = 0; v < n; ++v) rows[v + 1] = rows[v] + uniq[v + 1];
    cols.resize(rows[n]);
    w.resize(rows[n]);
#pragma omp parallel for schedule(dynamic, 4096)
    for (int64_t v = 0; v < (int64_t)n; ++v) {
        const uint64_t k = rows[v + 1] - rows[v];
        for (uint64_t j = 0; j < k; ++j) {
            const uint32_t u = tmp[off[v] + j];
            cols[rows[v] + j] = u;
            w[rows[v] + j] = wfun(std::min<uint32_t>((uint32_t)v, u), std::max<uint32_t>((uint32_t)v, u));
        }
    }
}

// One cached result per generator so that the sizing call and the copy call
// generate once.
struct GraphCache {
    std::mutex mu;
    uint64_t key = 0;
    bool valid = false;
    std::vector<uint64_t> rows;
    std::vector<uint32_t> cols, extra;
    std::vector<float> w;
};

uint64_t hash_params(std::initializer_list<double> xs) {
    uint64_t h = 0x12345678;
    for (double x : xs) {
        uint64_t b;
        memcpy(&b, &x, 8);
        h = fmix64(h ^ b) + 0x9e37;
    }
    return h;
}

int copy_out(GraphCache& gc, uint64_t* row_ptr, uint32_t* cols, float* w, uint64_t* n_edges_out) {
    *n_edges_out = gc.rows.back();
    if (!row_ptr) return 0;
    memcpy(row_ptr, gc.rows.data(), gc.rows.size() * 8);
    if (cols) memcpy(cols, gc.cols.data(), gc.cols.size() * 4);
    if (w) memcpy(w, gc.w.data(), gc.w.size() * 4);
    return 0;
}

GraphCache g_sbm, g_cl;

}  // namespace

// ---------------------------------------------------------------------------
// Generators
// ---------------------------------------------------------------------------
extern "C" int epg_sbm(uint64_t n, uint32_t blocks, double k_in, double k_out, uint64_t seed, uint64_t* row_ptr,
                       uint32_t* cols, float* w, uint32_t* community_out, uint64_t* n_edges_out) {
    if (n < 2 || blocks == 0 || blocks > n || !n_edges_out) return EP_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(g_sbm.mu);
    const uint64_t key = hash_params({(double)n, (double)blocks, k_in, k_out, (double)seed});
    auto comm = [&](uint64_t i) { return (uint32_t)(i * blocks / n); };
    if (!(g_sbm.valid && g_sbm.key == key)) {
        std::vector<uint64_t> start(blocks + 1);
        for (uint32_t c = 0; c <= blocks; ++c) start[c] = (c * n + blocks - 1) / blocks;
        // pair sampling by geometric skipping over each block pair (Batagelj & Brandes 2005)
        std::vector<uint32_t> a, b;
        for (uint32_t c1 = 0; c1 < blocks; ++c1) {
            for (uint32_t c2 = c1; c2 < blocks; ++c2) {
                const uint64_t n1 = start[c1 + 1] - start[c1], n2 = start[c2 + 1] - start[c2];
                const uint64_t pairs = c1 == c2 ? n1 * (n1 - 1) / 2 : n1 * n2;
                if (!pairs) continue;
                const double p = c1 == c2 ? (n1 > 1 ? k_in / (double)(n1 - 1) : 0.0)
                                          : k_out / (double)(n - n1) * 1.0;
                if (p <= 0) continue;
                Rng r(seed, 1, (uint64_t)c1 * blocks + c2);
                const double lq = std::log(1.0 - std::min(p, 0.999999));
                int64_t idx = -1;
                for (;;) {
                    const double u = r.uniform();
                    idx += 1 + (int64_t)std::floor(std::log(1.0 - u) / lq);
                    if ((uint64_t)idx >= pairs) break;
                    uint64_t x, y;
                    if (c1 == c2) {   // idx -> (i < j) within the block
                        uint64_t i = (uint64_t)((std::sqrt(8.0 * (double)idx + 1.0) + 1.0) / 2.0);
                        while (i * (i - 1) / 2 > (uint64_t)idx) --i;
                        while ((i + 1) * i / 2 <= (uint64_t)idx) ++i;
                        const uint64_t j = (uint64_t)idx - i * (i - 1) / 2;
                        x = start[c1] + i;
                        y = start[c1] + j;
                    } else {
                        x = start[c1] + (uint64_t)idx / n2;
                        y = start[c2] + (uint64_t)idx % n2;
                    }
                    a.push_back((uint32_t)x);
                    b.push_back((uint32_t)y);
                }
            }
        }
        // give isolated nodes one edge inside their community
        std::vector<uint8_t> has(n, 0);
        for (size_t i = 0; i < a.size(); ++i) { has[a[i]] = 1; has[b[i]] = 1; }
        Rng r(seed, 2, 0);
        for (uint64_t v = 0; v < n; ++v) {
            if (has[v]) continue;
            const uint32_t c = comm(v);
            const uint64_t sz = start[c + 1] - start[c];
            uint64_t u = sz > 1 ? start[c] + r.below(sz) : r.below(n);
            if (u == v) u = (v + 1) % n;
            a.push_back((uint32_t)v);
            b.push_back((uint32_t)u);
            has[u] = 1;
        }
        build_sym_csr(n, a, b, [](uint32_t, uint32_t) { return 1.f; }, g_sbm.rows, g_sbm.cols, g_sbm.w);
        g_sbm.key = key;
        g_sbm.valid = true;
    }
    if (community_out)
        for (uint64_t i = 0; i < n; ++i) community_out[i] = comm(i);
    return copy_out(g_sbm, row_ptr, cols, w, n_edges_out);
}

extern "C" int epg_sbm_tokens(uint64_t n, const uint32_t* community, uint32_t tok_min, uint32_t tok_max,
                              uint32_t sub_vocab, uint32_t global_vocab, double p_local, uint32_t slot_bits,
                              uint64_t seed, uint64_t* fptr, uint32_t* fids, uint32_t* slot_of_feature,
                              uint64_t* n_fids_out, uint32_t* n_feat_out) {
    if (!community || tok_min == 0 || tok_max < tok_min || slot_bits == 0 || slot_bits > 31 || !n_fids_out || !n_feat_out)
        return EP_ERR_INVALID_ARG;
    uint32_t max_comm = 0;
    for (uint64_t i = 0; i < n; ++i) max_comm = std::max(max_comm, community[i]);
    const uint64_t global_base = (uint64_t)(max_comm + 1) * sub_vocab;
    std::unordered_map<uint32_t, uint32_t> intern;
    std::vector<uint32_t> slots;
    uint64_t total = 0;
    if (fptr) fptr[0] = 0;
    for (uint64_t v = 0; v < n; ++v) {
        Rng r(seed, 3, v);
        const uint32_t k = tok_min + (uint32_t)r.below(tok_max - tok_min + 1);
        for (uint32_t j = 0; j < k; ++j) {
            uint64_t tok;
            if (r.uniform() < p_local) tok = (uint64_t)community[v] * sub_vocab + r.below(sub_vocab);
            else tok = global_base + r.below(global_vocab);
            const uint32_t slot = (uint32_t)(fmix64(tok + 0x5bd1e995ull) & ((1ull << slot_bits) - 1));
            auto it = intern.find(slot);
            uint32_t id;
            if (it == intern.end()) {
                id = (uint32_t)slots.size();
                intern.emplace(slot, id);
                slots.push_back(slot);
            } else {
                id = it->second;
            }
            if (fids) fids[total] = id;
            ++total;
        }
        if (fptr) fptr[v + 1] = total;
    }
    *n_fids_out = total;
    *n_feat_out = (uint32_t)slots.size();
    if (slot_of_feature) memcpy(slot_of_feature, slots.data(), slots.size() * 4);
    return EP_OK;
}

extern "C" int epg_chung_lu(uint64_t n, double exponent, double mean_degree, double max_degree, int bipartite,
                            float w_lo, float w_hi, uint64_t seed, uint64_t* row_ptr, uint32_t* cols, float* w,
                            uint64_t* n_edges_out) {
    if (n < 4 || n > 0xfffffffeull || exponent <= 1.0 || mean_degree <= 0 || max_degree < 1 || !n_edges_out)
        return EP_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(g_cl.mu);
    const uint64_t key = hash_params({(double)n, exponent, mean_degree, max_degree, (double)bipartite, w_lo, w_hi, (double)seed});
    if (!(g_cl.valid && g_cl.key == key)) {
        // expected degrees: w_i ~ (i+1)^(-1/(exponent-1)), clipped to [1, max]
        // with the scale bisected so that the clipped mean is mean_degree
        std::vector<double> base(n);
        const double ex = -1.0 / (exponent - 1.0);
        for (uint64_t i = 0; i < n; ++i) base[i] = std::pow((double)(i + 1), ex);
        auto clipped_mean = [&](double s) {
            double acc = 0;
#pragma omp parallel for reduction(+ : acc) schedule(static)
            for (int64_t i = 0; i < (int64_t)n; ++i) acc += std::min(std::max(s * base[i], 1.0), max_degree);
            return acc / (double)n;
        };
        double lo = 1e-12, hi = 1.0;
        while (clipped_mean(hi) < mean_degree && hi < 1e30) hi *= 2;
        for (int it = 0; it < 200; ++it) {
            const double mid = std::sqrt(lo * hi);
            (clipped_mean(mid) < mean_degree ? lo : hi) = mid;
        }
        std::vector<double> wexp(n);
        for (uint64_t i = 0; i < n; ++i) wexp[i] = std::min(std::max(hi * base[i], 1.0), max_degree);
        // random node labels, so that high-degree nodes are spread over the id
        // range (bipartite: over each side's range, users [0, n/2) and items
        // [n/2, n))
        const uint64_t half = n / 2;
        std::vector<uint32_t> label(n);
        std::iota(label.begin(), label.end(), 0u);
        {
            Rng r(seed, 4, 0);
            if (bipartite) {
                for (uint64_t i = half; i > 1; --i) std::swap(label[i - 1], label[r.below(i)]);
                for (uint64_t i = n - half; i > 1; --i) std::swap(label[half + i - 1], label[half + r.below(i)]);
            } else {
                for (uint64_t i = n; i > 1; --i) std::swap(label[i - 1], label[r.below(i)]);
            }
        }
        std::vector<double> w_all(wexp);
        std::vector<double> wa, wb;
        if (bipartite) {
            // users take the even-ranked weights, items the odd-ranked ones
            wa.resize(half); wb.resize(n - half);
            for (uint64_t i = 0; i < half; ++i) wa[i] = wexp[2 * i < n ? 2 * i : n - 1];
            for (uint64_t i = 0; i < n - half; ++i) wb[i] = wexp[2 * i + 1 < n ? 2 * i + 1 : n - 1];
        }
        const Alias al_all(w_all);
        const Alias* al_a = nullptr;
        const Alias* al_b = nullptr;
        std::unique_ptr<Alias> pa, pb;
        if (bipartite) { pa.reset(new Alias(wa)); pb.reset(new Alias(wb)); al_a = pa.get(); al_b = pb.get(); }
        const uint64_t m = (uint64_t)std::llround((double)n * mean_degree / 2.0);
        std::vector<uint32_t> a(m), b(m);
        const uint64_t BLK = 1ull << 16;
        const int64_t nblk = (int64_t)((m + BLK - 1) / BLK);
#pragma omp parallel for schedule(dynamic, 1)
        for (int64_t blk = 0; blk < nblk; ++blk) {
            Rng r(seed, 5, (uint64_t)blk);
            const uint64_t e0 = (uint64_t)blk * BLK, e1 = std::min(m, e0 + BLK);
            for (uint64_t e = e0; e < e1; ++e) {
                if (bipartite) {
                    a[e] = label[al_a->draw(r)];
                    b[e] = label[half + al_b->draw(r)];
                } else {
                    a[e] = label[al_all.draw(r)];
                    b[e] = label[al_all.draw(r)];
                }
            }
        }
        // nodes left without an edge get one
        std::vector<uint8_t> has(n, 0);
        for (uint64_t e = 0; e < m; ++e)
            if (a[e] != b[e]) { has[a[e]] = 1; has[b[e]] = 1; }
        Rng r(seed, 6, 0);
        std::vector<uint32_t> inv(n);
        for (uint64_t i = 0; i < n; ++i) inv[label[i]] = (uint32_t)i;
        for (uint64_t v = 0; v < n; ++v) {
            if (has[v]) continue;
            uint32_t u;
            if (bipartite) {
                const bool user = inv[v] < half;
                u = user ? label[half + al_b->draw(r)] : label[al_a->draw(r)];
            } else {
                do { u = label[al_all.draw(r)]; } while (u == v);
            }
            a.push_back((uint32_t)v);
            b.push_back(u);
            has[u] = 1;
        }
        const bool weighted = w_hi > w_lo;
        auto wf = [&](uint32_t x, uint32_t y) {
            if (!weighted) return 1.f;
            const uint64_t h = fmix64(((uint64_t)x << 32 | y) ^ seed);
            return w_lo + (w_hi - w_lo) * (float)((double)(h >> 11) * (1.0 / 9007199254740992.0));
        };
        build_sym_csr(n, a, b, wf, g_cl.rows, g_cl.cols, g_cl.w);
        g_cl.key = key;
        g_cl.valid = true;
    }
    return copy_out(g_cl, row_ptr, cols, w, n_edges_out);
}

extern "C" int epg_zipf_features(uint64_t n, double lambda, uint32_t cmin, uint32_t cmax, double s, uint32_t n_slots,
                                 uint64_t seed, uint64_t* fptr, uint32_t* fids, uint64_t* n_fids_out) {
    if (cmin == 0 || cmax < cmin || n_slots == 0 || !n_fids_out) return EP_ERR_INVALID_ARG;
    const uint64_t BLK = 1ull << 14;
    const int64_t nblk = (int64_t)((n + BLK - 1) / BLK);
    std::vector<uint32_t> cnt(n);
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t blk = 0; blk < nblk; ++blk) {
        Rng r(seed, 7, (uint64_t)blk);
        for (uint64_t v = (uint64_t)blk * BLK; v < std::min(n, (uint64_t)(blk + 1) * BLK); ++v) {
            uint32_t k = lambda > 0 ? r.poisson(lambda) : cmin + (uint32_t)r.below(cmax - cmin + 1);
            cnt[v] = std::min(std::max(k, cmin), cmax);
        }
    }
    uint64_t total = 0;
    for (uint64_t v = 0; v < n; ++v) total += cnt[v];
    *n_fids_out = total;
    if (!fptr) return EP_OK;
    fptr[0] = 0;
    for (uint64_t v = 0; v < n; ++v) fptr[v + 1] = fptr[v] + cnt[v];
    if (!fids) return EP_OK;
    std::vector<double> zw(n_slots);
    for (uint32_t k = 0; k < n_slots; ++k) zw[k] = std::pow((double)(k + 1), -s);
    const Alias al(zw);
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t blk = 0; blk < nblk; ++blk) {
        Rng r(seed, 8, (uint64_t)blk);
        for (uint64_t v = (uint64_t)blk * BLK; v < std::min(n, (uint64_t)(blk + 1) * BLK); ++v)
            for (uint64_t j = fptr[v]; j < fptr[v + 1]; ++j) fids[j] = al.draw(r);
    }
    return EP_OK;
}

