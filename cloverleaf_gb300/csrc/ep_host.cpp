// ep_host.cpp -- host-side graph construction (the graph.rs part of the C
// ABI), the embedding and graph text formats, the vocabulary, and feature
// propagation.
//
// Plain C++17 + OpenMP; no CUDA.  Identical results on x86_64 and aarch64:
// no intrinsics and no floating-point contraction (built with
// -ffp-contract=off).
#include <algorithm>
#include <atomic>
#include <charconv>
#include <cctype>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <memory>
#include <mutex>
#include <numeric>
#include <string>
#include <unordered_map>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../../include/ep_gb300.h"

// ---------------------------------------------------------------------------
// graph.rs restatement on the boundary
// ---------------------------------------------------------------------------
extern "C" int ep_csr_from_edges(uint64_t n_edges, const uint32_t* from, const uint32_t* to, const float* w, int dedup,
                                 uint64_t* rows_out, uint32_t* cols_out, float* w_out, uint64_t* n_nodes_out,
                                 uint64_t* n_edges_out) {
    if ((!from || !to || !w) && n_edges) return EP_ERR_INVALID_ARG;
    if (!rows_out || !n_nodes_out || !n_edges_out) return EP_ERR_INVALID_ARG;
    std::vector<uint64_t> order(n_edges);
    std::iota(order.begin(), order.end(), 0);
    std::vector<uint32_t> f(from, from + n_edges), t(to, to + n_edges);
    std::vector<float> ww(w, w + n_edges);
    uint64_t m = n_edges;
    if (dedup && n_edges) {
        // graph.rs:120-142: stable sort by (from, to), duplicates summed in order
        std::stable_sort(order.begin(), order.end(), [&](uint64_t x, uint64_t y) {
            return f[x] != f[y] ? f[x] < f[y] : t[x] < t[y];
        });
        std::vector<uint32_t> f2, t2;
        std::vector<float> w2;
        f2.reserve(n_edges); t2.reserve(n_edges); w2.reserve(n_edges);
        for (uint64_t i = 0; i < n_edges; ++i) {
            const uint64_t e = order[i];
            if (!f2.empty() && f2.back() == f[e] && t2.back() == t[e]) w2.back() += ww[e];
            else { f2.push_back(f[e]); t2.push_back(t[e]); w2.push_back(ww[e]); }
        }
        f.swap(f2); t.swap(t2); ww.swap(w2);
        m = f.size();
    }
    uint64_t max_node = 0;
    for (uint64_t i = 0; i < m; ++i) max_node = std::max<uint64_t>(max_node, std::max(f[i], t[i]));
    const uint64_t nn = max_node + 1;
    std::fill(rows_out, rows_out + nn + 1, 0);
    for (uint64_t i = 0; i < m; ++i) rows_out[(uint64_t)f[i] + 1]++;
    for (uint64_t i = 1; i <= nn; ++i) rows_out[i] += rows_out[i - 1];
    std::vector<uint64_t> cnt(nn, 0);
    for (uint64_t i = 0; i < m; ++i) {
        const uint64_t idx = rows_out[f[i]] + cnt[f[i]]++;
        if (cols_out) cols_out[idx] = t[i];
        if (w_out) w_out[idx] = ww[i];
    }
    *n_nodes_out = nn;
    *n_edges_out = m;
    return EP_OK;
}

extern "C" int ep_cdf_convert(uint64_t n_nodes, const uint64_t* rows, float* w) {
    if (!rows || (!w && rows[n_nodes])) return EP_ERR_INVALID_ARG;
    for (uint64_t v = 0; v < n_nodes; ++v) {   // graph.rs:664-691
        const uint64_t s = rows[v], e = rows[v + 1];
        if (s >= e) continue;
        float denom = 0.f;
        for (uint64_t j = s; j < e; ++j) denom += w[j];
        if (denom == 0.f) {
            for (uint64_t j = s; j < e; ++j) w[j] = 1.f;
            denom = (float)(e - s);
        }
        float acc = 0.f;
        for (uint64_t j = s; j < e; ++j) {
            acc += w[j];
            w[j] = std::min(acc / denom, 1.f);
        }
        w[e - 1] = 1.f;
    }
    return EP_OK;
}

// ---------------------------------------------------------------------------
// NodeEmbeddings text format (EmbeddingWriter::stream, src/io.rs:44-76, and
// line_to_embedding, src/io.rs:246-262): one line per node,
// "<type>\t<name>\t[v0,v1,...]".  Values are written as the shortest decimal
// that reads back to the same f32 (std::to_chars), and read with
// std::from_chars; rows are formatted and parsed in parallel.
// ---------------------------------------------------------------------------
extern "C" int64_t ep_format_embeddings(uint64_t n, uint32_t dims, const float* table, const char* types,
                                        const uint64_t* type_off, const char* names, const uint64_t* name_off,
                                        uint64_t first_id, char* out, uint64_t out_cap) {
    if (dims == 0 || (n && (!table || !types || !out)) || (names && !name_off)) return EP_ERR_INVALID_ARG;
    const uint64_t one_type_len = type_off ? 0 : strlen(types);
    constexpr uint32_t MAXV = 16;   // longest shortest-form f32, "-1.17549435e-38", and a comma
    // each thread formats one contiguous range of rows into its own buffer;
    // the buffers are then placed back to back
    const int nt = (int)std::min<uint64_t>((uint64_t)omp_get_max_threads(), std::max<uint64_t>(1, n / 64));
    std::vector<std::string> part(nt);
    std::vector<uint64_t> part_off(nt + 1, 0);
#pragma omp parallel num_threads(nt)
    {
        const int t = omp_get_thread_num();
        const uint64_t lo = n * t / nt, hi = n * (t + 1) / nt;
        std::string& o = part[t];
        char num[32];
        for (uint64_t i = lo; i < hi; ++i) {
            if (type_off) o.append(types + type_off[i], type_off[i + 1] - type_off[i]);
            else o.append(types, one_type_len);
            o.push_back('\t');
            if (names) {
                o.append(names + name_off[i], name_off[i + 1] - name_off[i]);
            } else {
                char* z = std::to_chars(num, num + sizeof num, first_id + i).ptr;
                o.append(num, z - num);
            }
            o.append("\t[", 2);
            const size_t at = o.size();
            o.resize(at + (size_t)dims * MAXV);
            char* p = &o[at];
            const float* row = table + i * dims;
            for (uint32_t k = 0; k < dims; ++k) {
                if (k) *p++ = ',';
                p = std::to_chars(p, p + MAXV, row[k]).ptr;
            }
            o.resize((size_t)(p - o.data()));
            o.append("]\n", 2);
        }
    }
    for (int t = 0; t < nt; ++t) part_off[t + 1] = part_off[t] + part[t].size();
    if (part_off[nt] > out_cap) return EP_ERR_INVALID_ARG;
#pragma omp parallel for num_threads(nt)
    for (int t = 0; t < nt; ++t) memcpy(out + part_off[t], part[t].data(), part[t].size());
    return (int64_t)part_off[nt];
}

extern "C" int64_t ep_parse_embeddings(const char* buf, uint64_t len, uint32_t* dims, float* values,
                                       uint64_t* tok_off, uint64_t* bad_line) {
    if ((len && !buf) || !dims) return EP_ERR_INVALID_ARG;
    if (bad_line) *bad_line = 0;
    // line starts; blank lines are skipped
    std::vector<uint64_t> start;
    for (uint64_t i = 0; i < len;) {
        const void* nl = memchr(buf + i, '\n', len - i);
        const uint64_t e = nl ? (uint64_t)((const char*)nl - buf) : len;
        if (e > i && !(e == i + 1 && buf[i] == '\r')) start.push_back(i);
        i = e + 1;
    }
    const int64_t rows = (int64_t)start.size();
    // line_to_embedding (src/io.rs:246-262): exactly three tab-separated
    // fields; the third loses its first and last byte (the brackets) and is
    // split on ',', each piece trimmed and read as an f32.  Values past cap
    // are counted but not stored.
    auto parse_row = [&](int64_t r, float* dst, uint32_t cap, uint64_t* tok, uint32_t* count) -> bool {
        const uint64_t b = start[r];
        const void* nl = memchr(buf + b, '\n', len - b);
        uint64_t e = nl ? (uint64_t)((const char*)nl - buf) : len;
        if (e > b && buf[e - 1] == '\r') --e;
        const char* t1 = (const char*)memchr(buf + b, '\t', e - b);
        if (!t1) return false;
        const uint64_t f1 = (uint64_t)(t1 - buf);
        const char* t2 = (const char*)memchr(buf + f1 + 1, '\t', e - f1 - 1);
        if (!t2) return false;
        const uint64_t f2 = (uint64_t)(t2 - buf);
        if (memchr(buf + f2 + 1, '\t', e - f2 - 1)) return false;
        if (tok) { tok[0] = b; tok[1] = f1; tok[2] = f1 + 1; tok[3] = f2; }
        if (e - f2 - 1 < 2) return false;
        uint64_t p = f2 + 2;
        const uint64_t end = e - 1;
        uint32_t k = 0;
        for (;;) {
            const void* c = memchr(buf + p, ',', end - p);
            const uint64_t q = c ? (uint64_t)((const char*)c - buf) : end;
            uint64_t a = p, z = q;
            while (a < z && isspace((unsigned char)buf[a])) ++a;
            while (z > a && isspace((unsigned char)buf[z - 1])) --z;
            const char* s0 = buf + a;
            if (a + 1 < z && *s0 == '+' && s0[1] != '-') ++s0;     // a leading '+' is allowed
            float v = 0.f;
            auto res = std::from_chars(s0, buf + z, v);
            if (res.ec == std::errc::result_out_of_range) {
                // beyond f32's range: round through f64 (overflow to inf,
                // underflow to zero), as a saturating float parser does
                double dv = 0.0;
                res = std::from_chars(s0, buf + z, dv);
                v = (float)dv;
            }
            // from_chars also takes the inf / infinity / nan spellings, in any case
            if (a == z || res.ec != std::errc() || res.ptr != buf + z) return false;
            if (dst && k < cap) dst[k] = v;
            ++k;
            if (q >= end) break;
            p = q + 1;
        }
        *count = k;
        return true;
    };
    if (!values) {      // counting call: rows, and the width of the first row (0: malformed)
        uint32_t k = 0;
        *dims = rows && parse_row(0, nullptr, 0, nullptr, &k) ? k : 0;
        return rows;
    }
    const uint32_t d = *dims;
    std::atomic<int64_t> first_bad{INT64_MAX};
#pragma omp parallel for schedule(dynamic, 512)
    for (int64_t r = 0; r < rows; ++r) {
        uint32_t k = 0;
        const bool ok = parse_row(r, values + (uint64_t)r * d, d, tok_off ? tok_off + 4 * (uint64_t)r : nullptr, &k);
        if (!ok || k != d) {
            int64_t cur = first_bad.load();
            while (r < cur && !first_bad.compare_exchange_weak(cur, r)) {}
        }
    }
    if (first_bad.load() != INT64_MAX) {
        if (bad_line) *bad_line = (uint64_t)first_bad.load() + 1;
        return EP_ERR_INVALID_ARG;
    }
    return rows;
}

// ---------------------------------------------------------------------------
// propagate_features (src/algos/feat_propagation.rs:13-93).  Nodes without
// features take the k heaviest features of their neighbours, each feature
// weighted by the sum of the edge probabilities (differences of the row's
// CDF) of the neighbours carrying it; features with weight / L2 norm <=
// threshold are dropped.  Sweeps run over the nodes in order and update in
// place, so a node sees the features its predecessors received in the same
// sweep.  A node is final once every neighbour had features when it was
// visited; sweeps stop when all are final or after max_iters.  Equal weights
// are ordered by feature id (the reference leaves them in hash-map order).
// ---------------------------------------------------------------------------
extern "C" int64_t ep_propagate_features(uint64_t n, const uint64_t* rows, const uint32_t* cols, const float* cdf,
                                         const uint64_t* fptr, const uint32_t* fids, uint32_t max_iters, uint32_t k,
                                         float threshold, uint64_t* fptr_out, uint32_t* fids_out, uint64_t out_cap) {
    if (n && (!rows || !cols || !cdf || !fptr || !fptr_out)) return EP_ERR_INVALID_ARG;
    uint32_t n_feat = 0;
    for (uint64_t i = 0; i < (n ? fptr[n] : 0); ++i) n_feat = std::max(n_feat, fids[i] + 1);
    std::vector<std::vector<uint32_t>> own(n);      // lists of nodes that started without features
    std::vector<uint8_t> done(n, 0);
    uint64_t missing = 0;
    for (uint64_t v = 0; v < n; ++v) {
        if (fptr[v + 1] < fptr[v]) return EP_ERR_INVALID_ARG;
        done[v] = fptr[v + 1] > fptr[v];
        missing += !done[v];
    }
    for (uint64_t e = 0; e < (n ? rows[n] : 0); ++e)
        if (cols[e] >= n) return EP_ERR_INVALID_ARG;
    const std::vector<uint8_t> had(done);
    auto feats = [&](uint64_t u, const uint32_t*& b, size_t& len) {
        if (had[u]) { b = fids + fptr[u]; len = (size_t)(fptr[u + 1] - fptr[u]); }
        else { b = own[u].data(); len = own[u].size(); }
    };
    std::vector<float> wsum(n_feat, 0.f);
    std::vector<uint8_t> seen(n_feat, 0);
    std::vector<uint32_t> touched;
    std::vector<std::pair<float, uint32_t>> order;
    for (uint32_t it = 0; it < max_iters && missing; ++it) {
        bool all_final = true;
        for (uint64_t v = 0; v < n; ++v) {
            if (done[v]) continue;
            bool nbrs_final = true;
            float prev = 0.f;
            for (uint64_t e = rows[v]; e < rows[v + 1]; ++e) {
                const float px = cdf[e] - prev;
                prev = cdf[e];
                const uint32_t* b;
                size_t len;
                feats(cols[e], b, len);
                nbrs_final = nbrs_final && len > 0;
                for (size_t j = 0; j < len; ++j) {
                    const uint32_t f = b[j];
                    if (!seen[f]) { seen[f] = 1; wsum[f] = 0.f; touched.push_back(f); }
                    wsum[f] += px;
                }
            }
            order.clear();
            for (uint32_t f : touched) { order.emplace_back(wsum[f], f); seen[f] = 0; }
            touched.clear();
            std::sort(order.begin(), order.end(), [](const std::pair<float, uint32_t>& a, const std::pair<float, uint32_t>& b) {
                return a.first > b.first || (a.first == b.first && a.second < b.second);
            });
            float sq = 0.f;
            for (const auto& x : order) sq += x.first * x.first;
            const float norm = std::sqrt(sq);
            std::vector<uint32_t>& out = own[v];
            out.clear();
            for (const auto& x : order) {
                if (out.size() >= k) break;
                if (x.first / norm > threshold) out.push_back(x.second);
            }
            if (nbrs_final) { done[v] = 1; --missing; }
            else all_final = false;
        }
        if (all_final) break;
    }
    uint64_t o = 0;
    fptr_out[0] = 0;
    for (uint64_t v = 0; v < n; ++v) {
        const uint32_t* b;
        size_t len;
        feats(v, b, len);
        if (o + len > out_cap) return EP_ERR_INVALID_ARG;
        if (len) memcpy(fids_out + o, b, len * sizeof(uint32_t));
        o += len;
        fptr_out[v + 1] = o;
    }
    return (int64_t)o;
}

// ---------------------------------------------------------------------------
// Vocabulary of (node type, name) pairs -> dense ids in first-seen order
// (Vocab, src/vocab.rs), and the graph text format of GraphReader::load
// (src/io.rs:270-323) and Graph::save (src/lib.rs:414-430):
// "from_type\tfrom\tto_type\tto\tweight" lines.
//
// The vocabulary keeps every key as "type\0name" in one byte arena and an
// open-addressing table of ids keyed by a 64-bit hash of the key.
// ---------------------------------------------------------------------------
namespace {
inline uint64_t key_hash(const char* t, size_t tl, const char* n, size_t nl) {
    // FNV-1a over type, a separator and name, then a murmur-style finalizer
    uint64_t h = 1469598103934665603ull;
    for (size_t i = 0; i < tl; ++i) h = (h ^ (unsigned char)t[i]) * 1099511628211ull;
    h = (h ^ 0xffu) * 1099511628211ull;
    for (size_t i = 0; i < nl; ++i) h = (h ^ (unsigned char)n[i]) * 1099511628211ull;
    h ^= h >> 33;
    h *= 0xff51afd7ed558ccdull;
    h ^= h >> 33;
    return h;
}
}  // namespace

struct ep_vocab {
    std::vector<char> arena;            // keys back to back: type, '\0', name
    std::vector<uint64_t> off;          // key i is arena[off[i], off[i+1]); off.size() = size + 1
    std::vector<uint32_t> type_len;     // bytes of the type of key i
    std::vector<uint32_t> slots;        // id + 1, 0 = empty
    uint64_t mask = 0;
    uint64_t max_key = 0;               // longest type + name, in bytes
    ep_vocab() : off(1, 0) {}
    uint64_t size() const { return off.size() - 1; }
    bool same(uint64_t id, const char* t, size_t tl, const char* n, size_t nl) const {
        if (type_len[id] != tl || off[id + 1] - off[id] != tl + 1 + nl) return false;
        const char* k = arena.data() + off[id];
        return memcmp(k, t, tl) == 0 && memcmp(k + tl + 1, n, nl) == 0;
    }
    void grow() {
        const uint64_t cap = slots.empty() ? 1024 : slots.size() * 2;
        slots.assign(cap, 0);
        mask = cap - 1;
        for (uint64_t id = 0; id < size(); ++id) {
            const char* k = arena.data() + off[id];
            const uint32_t tl = type_len[id];
            uint64_t h = key_hash(k, tl, k + tl + 1, off[id + 1] - off[id] - tl - 1) & mask;
            while (slots[h]) h = (h + 1) & mask;
            slots[h] = (uint32_t)(id + 1);
        }
    }
    int64_t find(const char* t, size_t tl, const char* n, size_t nl, uint64_t hash) const {
        if (slots.empty()) return -1;
        for (uint64_t h = hash & mask;; h = (h + 1) & mask) {
            const uint32_t s = slots[h];
            if (!s) return -1;
            if (same(s - 1, t, tl, n, nl)) return (int64_t)(s - 1);
        }
    }
    // id of the key, inserted at the end when new; -1 when the vocabulary is full
    int64_t intern(const char* t, size_t tl, const char* n, size_t nl, uint64_t hash) {
        if ((size() + 1) * 2 > slots.size()) grow();
        uint64_t h = hash & mask;
        for (;; h = (h + 1) & mask) {
            const uint32_t s = slots[h];
            if (!s) break;
            if (same(s - 1, t, tl, n, nl)) return (int64_t)(s - 1);
        }
        const uint64_t id = size();
        if (id >= 0xffffffffull) return -1;
        arena.insert(arena.end(), t, t + tl);
        arena.push_back('\0');
        arena.insert(arena.end(), n, n + nl);
        off.push_back(arena.size());
        type_len.push_back((uint32_t)tl);
        max_key = std::max<uint64_t>(max_key, tl + nl);
        slots[h] = (uint32_t)(id + 1);
        return (int64_t)id;
    }
};

extern "C" int ep_vocab_create(ep_vocab** out) {
    if (!out) return EP_ERR_INVALID_ARG;
    *out = new (std::nothrow) ep_vocab();
    return *out ? EP_OK : EP_ERR_OOM;
}

extern "C" void ep_vocab_destroy(ep_vocab* v) { delete v; }

extern "C" uint64_t ep_vocab_len(const ep_vocab* v) { return v ? v->size() : 0; }

extern "C" uint64_t ep_vocab_max_key(const ep_vocab* v) { return v ? v->max_key : 0; }

extern "C" int64_t ep_vocab_intern(ep_vocab* v, const char* type, uint64_t type_len, const char* name,
                                   uint64_t name_len) {
    if (!v || (type_len && !type) || (name_len && !name)) return EP_ERR_INVALID_ARG;
    const int64_t id = v->intern(type, type_len, name, name_len, key_hash(type, type_len, name, name_len));
    return id < 0 ? EP_ERR_INVALID_ARG : id;
}

extern "C" int64_t ep_vocab_find(const ep_vocab* v, const char* type, uint64_t type_len, const char* name,
                                 uint64_t name_len) {
    if (!v || (type_len && !type) || (name_len && !name)) return EP_ERR_INVALID_ARG;
    return v->find(type, type_len, name, name_len, key_hash(type, type_len, name, name_len));
}

extern "C" int ep_vocab_intern_tokens(ep_vocab* v, const char* buf, const uint64_t* tok, uint64_t n, uint32_t* ids) {
    if (!v || (n && (!buf || !tok || !ids))) return EP_ERR_INVALID_ARG;
    std::vector<uint64_t> h(n);
#pragma omp parallel for schedule(static) if (n > 4096)
    for (int64_t i = 0; i < (int64_t)n; ++i) {
        const uint64_t* t = tok + 4 * i;
        h[i] = key_hash(buf + t[0], t[1] - t[0], buf + t[2], t[3] - t[2]);
    }
    for (uint64_t i = 0; i < n; ++i) {
        const uint64_t* t = tok + 4 * i;
        const int64_t id = v->intern(buf + t[0], t[1] - t[0], buf + t[2], t[3] - t[2], h[i]);
        if (id < 0) return EP_ERR_INVALID_ARG;
        ids[i] = (uint32_t)id;
    }
    return EP_OK;
}

extern "C" int ep_vocab_range_bytes(const ep_vocab* v, uint64_t lo, uint64_t hi, uint64_t* type_bytes,
                                    uint64_t* name_bytes) {
    if (!v || lo > hi || hi > v->size()) return EP_ERR_INVALID_ARG;
    uint64_t tb = 0, nb = 0;
    for (uint64_t i = lo; i < hi; ++i) {
        tb += v->type_len[i];
        nb += v->off[i + 1] - v->off[i] - v->type_len[i] - 1;
    }
    if (type_bytes) *type_bytes = tb;
    if (name_bytes) *name_bytes = nb;
    return EP_OK;
}

extern "C" int ep_vocab_export(const ep_vocab* v, uint64_t lo, uint64_t hi, char* types, uint64_t* type_off,
                               char* names, uint64_t* name_off) {
    if (!v || lo > hi || hi > v->size() || !type_off || !name_off) return EP_ERR_INVALID_ARG;
    uint64_t tb = 0, nb = 0;
    type_off[0] = name_off[0] = 0;
    for (uint64_t i = lo; i < hi; ++i) {
        const char* k = v->arena.data() + v->off[i];
        const uint64_t tl = v->type_len[i], nl = v->off[i + 1] - v->off[i] - tl - 1;
        if (types) memcpy(types + tb, k, tl);
        if (names) memcpy(names + nb, k + tl + 1, nl);
        tb += tl;
        nb += nl;
        type_off[i - lo + 1] = tb;
        name_off[i - lo + 1] = nb;
    }
    return EP_OK;
}

extern "C" int64_t ep_parse_edges(ep_vocab* v, const char* buf, uint64_t len, int weighted, uint32_t* src,
                                  uint32_t* dst, float* w, uint64_t cap, uint64_t* bad_line) {
    if (!v || (len && !buf) || !src || !dst || !w) return EP_ERR_INVALID_ARG;
    if (bad_line) *bad_line = 0;
    std::vector<uint64_t> start;
    for (uint64_t i = 0; i < len;) {
        const void* nl = memchr(buf + i, '\n', len - i);
        const uint64_t e = nl ? (uint64_t)((const char*)nl - buf) : len;
        if (e > i && !(e == i + 1 && buf[i] == '\r')) start.push_back(i);
        i = e + 1;
    }
    const int64_t rows = (int64_t)start.size();
    if ((uint64_t)rows > cap) return EP_ERR_INVALID_ARG;
    // fields and key hashes in parallel; ids in line order afterwards
    struct Line { uint64_t f[5][2]; uint64_t h0, h1; };
    std::vector<Line> L((size_t)rows);
    std::atomic<int64_t> first_bad{INT64_MAX};
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t r = 0; r < rows; ++r) {
        const uint64_t b = start[r];
        const void* nl = memchr(buf + b, '\n', len - b);
        uint64_t e = nl ? (uint64_t)((const char*)nl - buf) : len;
        if (e > b && buf[e - 1] == '\r') --e;
        Line& x = L[r];
        uint64_t p = b;
        bool ok = true;
        for (int k = 0; k < 5 && ok; ++k) {
            const void* t = k < 4 ? memchr(buf + p, '\t', e - p) : nullptr;
            const uint64_t q = k < 4 ? (t ? (uint64_t)((const char*)t - buf) : e) : e;
            if (k < 4 && !t) ok = false;
            x.f[k][0] = p;
            x.f[k][1] = q;
            p = q + 1;
        }
        if (ok && memchr(buf + x.f[4][0], '\t', x.f[4][1] - x.f[4][0])) ok = false;     // more than 5 fields
        float wt = 1.f;
        if (ok && weighted) {
            const char* s0 = buf + x.f[4][0];
            const char* s1 = buf + x.f[4][1];
            if (s1 - s0 > 1 && *s0 == '+' && s0[1] != '-') ++s0;
            auto res = std::from_chars(s0, s1, wt);
            if (res.ec == std::errc::result_out_of_range) {
                double dv = 0.0;
                res = std::from_chars(s0, s1, dv);
                wt = (float)dv;
            }
            ok = s0 < s1 && res.ec == std::errc() && res.ptr == s1;
        }
        if (!ok) {
            int64_t cur = first_bad.load();
            while (r < cur && !first_bad.compare_exchange_weak(cur, r)) {}
            continue;
        }
        w[r] = wt;
        x.h0 = key_hash(buf + x.f[0][0], x.f[0][1] - x.f[0][0], buf + x.f[1][0], x.f[1][1] - x.f[1][0]);
        x.h1 = key_hash(buf + x.f[2][0], x.f[2][1] - x.f[2][0], buf + x.f[3][0], x.f[3][1] - x.f[3][0]);
    }
    if (first_bad.load() != INT64_MAX) {
        if (bad_line) *bad_line = (uint64_t)first_bad.load() + 1;
        return EP_ERR_INVALID_ARG;
    }
    for (int64_t r = 0; r < rows; ++r) {
        const Line& x = L[r];
        const int64_t a = v->intern(buf + x.f[0][0], x.f[0][1] - x.f[0][0], buf + x.f[1][0], x.f[1][1] - x.f[1][0], x.h0);
        const int64_t c = v->intern(buf + x.f[2][0], x.f[2][1] - x.f[2][0], buf + x.f[3][0], x.f[3][1] - x.f[3][0], x.h1);
        if (a < 0 || c < 0) return EP_ERR_INVALID_ARG;
        src[r] = (uint32_t)a;
        dst[r] = (uint32_t)c;
    }
    return rows;
}

extern "C" int64_t ep_format_edges(const ep_vocab* v, const char* anon_type, uint64_t n_nodes, const uint64_t* rows,
                                   const uint32_t* cols, const float* cdf, uint64_t lo, uint64_t hi, char* out,
                                   uint64_t out_cap) {
    if ((!v && !anon_type) || !rows || lo > hi || hi > n_nodes || (v && v->size() < n_nodes) || (hi > lo && !out))
        return EP_ERR_INVALID_ARG;
    const uint64_t anon_len = v ? 0 : strlen(anon_type);
    // the key of node u: its vocabulary entry, or (anon_type, decimal u)
    auto key = [&](uint64_t u, char* dec, const char*& t, uint64_t& tl, const char*& nm, uint64_t& nl) {
        if (v) {
            t = v->arena.data() + v->off[u];
            tl = v->type_len[u];
            nm = t + tl + 1;
            nl = v->off[u + 1] - v->off[u] - tl - 1;
        } else {
            t = anon_type;
            tl = anon_len;
            nm = dec;
            nl = (uint64_t)(std::to_chars(dec, dec + 24, u).ptr - dec);
        }
    };
    const int nt = (int)std::min<uint64_t>((uint64_t)omp_get_max_threads(), std::max<uint64_t>(1, (hi - lo) / 256));
    std::vector<std::string> part(nt);
    std::atomic<int> bad{0};
#pragma omp parallel num_threads(nt)
    {
        const int t = omp_get_thread_num();
        const uint64_t a = lo + (hi - lo) * t / nt, b = lo + (hi - lo) * (t + 1) / nt;
        std::string& o = part[t];
        char num[64], fdec[24], tdec[24];
        for (uint64_t u = a; u < b; ++u) {
            const char *ft, *fn;
            uint64_t ftl, fnl;
            key(u, fdec, ft, ftl, fn, fnl);
            float prev = 0.f;
            for (uint64_t e = rows[u]; e < rows[u + 1]; ++e) {
                const uint32_t x = cols[e];
                if (x >= n_nodes) { bad = 1; break; }
                const float p = cdf[e] - prev;     // CDFtoP (src/graph.rs:630-661)
                prev = cdf[e];
                const char *tt, *tn;
                uint64_t ttl, tnl;
                key(x, tdec, tt, ttl, tn, tnl);
                o.append(ft, ftl); o.push_back('\t');
                o.append(fn, fnl); o.push_back('\t');
                o.append(tt, ttl); o.push_back('\t');
                o.append(tn, tnl); o.push_back('\t');
                // f32 as Rust's Display writes it: shortest round-trip digits, positional
                char* z = std::to_chars(num, num + sizeof num, p, std::chars_format::fixed).ptr;
                o.append(num, z - num);
                o.push_back('\n');
            }
        }
    }
    if (bad) return EP_ERR_INVALID_ARG;
    uint64_t total = 0;
    for (const auto& x : part) total += x.size();
    if (total > out_cap) return EP_ERR_INVALID_ARG;
    uint64_t o = 0;
    for (const auto& x : part) { memcpy(out + o, x.data(), x.size()); o += x.size(); }
    return (int64_t)total;
}
