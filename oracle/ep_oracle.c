/*
 * ep_oracle.c -- CPU restatement of cloverleaf's Embedding Propagation
 * training path.  TEST INFRASTRUCTURE ONLY (see ep_oracle.h for callers and
 * for what is and is not pinned by the reference's own tests).
 *
 * The restatement keeps the reference's structure: per-node feature maps,
 * first-occurrence gradient extraction, a per-batch gradient map, batches
 * processed in parallel with unsynchronised ("hogwild") Adam writes.  It does
 * not rebuild simple_grad's autograd graph (the closed-form gradients of the
 * same expressions are used) and stores per-batch gradients in an arena rather
 * than one heap vector per feature, so it runs faster than the Rust reference
 * would on the same cores.
 */
#include "ep_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------------ */
/* Insertion-ordered map u32 -> count (stands in for hashbrown::HashMap with  */
/* (ANode, f32) values, model.rs:254).                                        */
/* ------------------------------------------------------------------------ */
typedef struct fmap_t {
    uint32_t* keys;
    float* cnt;      /* f32 like the reference's counts (model.rs:268-271) */
    uint32_t n, cap;
    int32_t* slots;
    uint32_t slot_cap; /* power of two */
} fmap_t;

static uint32_t hash_u32(uint32_t x) {
    x ^= x >> 16; x *= 0x7feb352dU; x ^= x >> 15; x *= 0x846ca68bU; x ^= x >> 16;
    return x;
}

static void fmap_free(fmap_t* m) {
    free(m->keys); free(m->cnt); free(m->slots);
    memset(m, 0, sizeof(*m));
}

static void fmap_clear(fmap_t* m) {
    for (uint32_t i = 0; i < m->n; ++i) {
        uint32_t s = hash_u32(m->keys[i]) & (m->slot_cap - 1);
        while (m->slots[s] != -1) { m->slots[s] = -1; s = (s + 1) & (m->slot_cap - 1); }
    }
    m->n = 0;
}

static int32_t fmap_find(const fmap_t* m, uint32_t key) {
    if (!m->slot_cap) return -1;
    uint32_t s = hash_u32(key) & (m->slot_cap - 1);
    while (m->slots[s] != -1) {
        if (m->keys[m->slots[s]] == key) return m->slots[s];
        s = (s + 1) & (m->slot_cap - 1);
    }
    return -1;
}

static void fmap_grow(fmap_t* m) {
    uint32_t ncap = m->cap ? m->cap * 2 : 64;
    m->keys = (uint32_t*)realloc(m->keys, sizeof(uint32_t) * ncap);
    m->cnt = (float*)realloc(m->cnt, sizeof(float) * ncap);
    m->cap = ncap;
    uint32_t nslot = ncap * 2;
    free(m->slots);
    m->slots = (int32_t*)malloc(sizeof(int32_t) * nslot);
    for (uint32_t i = 0; i < nslot; ++i) m->slots[i] = -1;
    m->slot_cap = nslot;
    for (uint32_t i = 0; i < m->n; ++i) {
        uint32_t s = hash_u32(m->keys[i]) & (nslot - 1);
        while (m->slots[s] != -1) s = (s + 1) & (nslot - 1);
        m->slots[s] = (int32_t)i;
    }
}

/* count[key] += c, inserting in first-seen order.  Returns the index. */
static int32_t fmap_add(fmap_t* m, uint32_t key, float c) {
    int32_t i = fmap_find(m, key);
    if (i >= 0) { m->cnt[i] += c; return i; }
    if (m->n + 1 > m->cap) fmap_grow(m);
    i = (int32_t)m->n++;
    m->keys[i] = key;
    m->cnt[i] = c;
    uint32_t s = hash_u32(key) & (m->slot_cap - 1);
    while (m->slots[s] != -1) s = (s + 1) & (m->slot_cap - 1);
    m->slots[s] = i;
    return i;
}

/* Gradient accumulator: feature -> d-vector (the per-batch std HashMap of
 * mod.rs:223-233), rows stored contiguously in first-insertion order. */
typedef struct gacc_t {
    fmap_t map;
    unsigned char* rows;
    uint64_t rows_cap; /* in rows */
    uint32_t d;
} gacc_t;

static void gacc_init(gacc_t* a, uint32_t d) {
    memset(a, 0, sizeof(*a));
    a->d = d;
}
static void gacc_free(gacc_t* a) { fmap_free(&a->map); free(a->rows); memset(a, 0, sizeof(*a)); }
static void gacc_clear(gacc_t* a) { fmap_clear(&a->map); }
static void* gacc_slot(gacc_t* a, uint32_t i, size_t esz) { return a->rows + (uint64_t)i * a->d * esz; }
/* Returns the row for feature f, zero-initialised on first use. */
static void* gacc_row(gacc_t* a, uint32_t f, size_t esz) {
    int32_t i = fmap_find(&a->map, f);
    if (i >= 0) return gacc_slot(a, (uint32_t)i, esz);
    i = fmap_add(&a->map, f, 0.f);
    if ((uint64_t)i + 1 > a->rows_cap) {
        uint64_t nc = a->rows_cap ? a->rows_cap * 2 : 256;
        a->rows = (unsigned char*)realloc(a->rows, nc * a->d * esz);
        a->rows_cap = nc;
    }
    void* r = gacc_slot(a, (uint32_t)i, esz);
    memset(r, 0, a->d * esz);
    return r;
}

/* All features of node v, each counting `weight` (model.rs:266-277 with
 * Sample::All: choose_multiple of every feature). */
static void add_node_all(fmap_t* m, const uint64_t* fptr, const uint32_t* fids, uint32_t v, float weight) {
    for (uint64_t j = fptr[v]; j < fptr[(uint64_t)v + 1]; ++j) fmap_add(m, fids[j], weight);
}

#define REAL float
#define SFX f32
#include "ep_oracle_batch.inc"
#undef REAL
#undef SFX
#define REAL double
#define SFX f64
#include "ep_oracle_batch.inc"
#undef REAL
#undef SFX

/* ------------------------------------------------------------------------ */
/* graph.rs                                                                  */
/* ------------------------------------------------------------------------ */
typedef struct { uint64_t f, t; float w; } edge_t;

/* Stable merge sort by (from, to), as rayon's par_sort_by_key
 * (graph.rs:124). */
static void msort_edges(edge_t* a, edge_t* tmp, uint64_t n) {
    if (n < 2) return;
    uint64_t h = n / 2;
    msort_edges(a, tmp, h);
    msort_edges(a + h, tmp, n - h);
    uint64_t i = 0, j = h, k = 0;
    while (i < h && j < n) {
        int le = (a[i].f < a[j].f) || (a[i].f == a[j].f && a[i].t <= a[j].t);
        tmp[k++] = le ? a[i++] : a[j++];
    }
    while (i < h) tmp[k++] = a[i++];
    while (j < n) tmp[k++] = a[j++];
    memcpy(a, tmp, n * sizeof(edge_t));
}

int orc_csr_from_edges(uint64_t n_edges, const uint64_t* from, const uint64_t* to,
                       const float* w, int dedup, uint64_t* rows_out,
                       uint64_t* cols_out, float* w_out,
                       uint64_t* n_nodes_out, uint64_t* n_edges_out) {
    edge_t* e = (edge_t*)malloc(sizeof(edge_t) * (n_edges ? n_edges : 1));
    for (uint64_t i = 0; i < n_edges; ++i) { e[i].f = from[i]; e[i].t = to[i]; e[i].w = w[i]; }
    uint64_t m = n_edges;
    if (dedup && n_edges > 0) {
        edge_t* tmp = (edge_t*)malloc(sizeof(edge_t) * n_edges);
        msort_edges(e, tmp, n_edges);
        free(tmp);
        uint64_t cur = 0;           /* graph.rs:126-140: sum duplicate weights */
        for (uint64_t i = 1; i < n_edges; ++i) {
            if (e[i].f == e[cur].f && e[i].t == e[cur].t) e[cur].w += e[i].w;
            else e[++cur] = e[i];
        }
        m = cur + 1;
    }
    uint64_t max_node = 0;
    for (uint64_t i = 0; i < m; ++i) {
        uint64_t mx = e[i].f > e[i].t ? e[i].f : e[i].t;
        if (mx > max_node) max_node = mx;
    }
    uint64_t nn = max_node + 1;
    for (uint64_t i = 0; i <= nn; ++i) rows_out[i] = 0;
    for (uint64_t i = 0; i < m; ++i) rows_out[e[i].f + 1]++;
    for (uint64_t i = 1; i <= nn; ++i) rows_out[i] += rows_out[i - 1];
    uint64_t* cnt = (uint64_t*)calloc(nn, sizeof(uint64_t));
    for (uint64_t i = 0; i < m; ++i) {
        uint64_t idx = rows_out[e[i].f] + cnt[e[i].f]++;
        cols_out[idx] = e[i].t;
        w_out[idx] = e[i].w;
    }
    free(cnt);
    free(e);
    *n_nodes_out = nn;
    *n_edges_out = m;
    return 0;
}

void orc_cdf_convert(uint64_t n_nodes, const uint64_t* rows, float* w) {
    for (uint64_t v = 0; v < n_nodes; ++v) {
        uint64_t s = rows[v], e = rows[v + 1];
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
            float c = acc / denom;
            w[j] = c < 1.f ? c : 1.f;
        }
        w[e - 1] = 1.f;
    }
}

/* ------------------------------------------------------------------------ */
/* grad_utils                                                                */
/* ------------------------------------------------------------------------ */
static void adam_row(float* e, float* m, float* v, const float* g, uint32_t d, float lr, float t) {
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    for (uint32_t k = 0; k < d; ++k) if (g[k] != g[k]) return;  /* optimizer.rs:56 */
    float c1 = 1.f - powf(b1, t), c2 = 1.f - powf(b2, t);
    for (uint32_t k = 0; k < d; ++k) {
        m[k] = b1 * m[k] + (1.f - b1) * g[k];
        v[k] = b2 * v[k] + (1.f - b2) * powf(g[k], 2.f);
    }
    for (uint32_t k = 0; k < d; ++k) {
        float mk = m[k] / c1;
        float vk = v[k] / c2;
        e[k] -= lr * (mk / (sqrtf(vk) + eps));
    }
}

void orc_adam(float* table, float* m, float* v, uint32_t d, uint32_t n_feat,
              const float* grad, const uint8_t* touched, float lr, uint32_t pass) {
    float t = (float)pass + 1.f;
    for (uint32_t f = 0; f < n_feat; ++f) {
        if (!touched[f]) continue;
        uint64_t o = (uint64_t)f * d;
        adam_row(table + o, m + o, v + o, grad + o, d, lr, t);
    }
}

float orc_lr_cos_decay(float min_alpha, float alpha, uint64_t warmup, uint64_t max_steps,
                       uint64_t cur_step) {
    if (cur_step > warmup) {
        float ratio = (float)cur_step / (float)max_steps;
        return min_alpha + 0.5f * (alpha - min_alpha) * (1.f + cosf(3.14159265358979323846f * ratio));
    }
    float ratio = (float)cur_step / (float)warmup;
    return min_alpha + ratio * (alpha - min_alpha);
}

/* ------------------------------------------------------------------------ */
/* Training loop (mod.rs:92-287)                                             */
/* ------------------------------------------------------------------------ */
/* xorshift128+ seeded through splitmix64.  The reference uses rand_xorshift;
 * this restatement does not reproduce its stream (trajectories of the
 * reference are nondeterministic anyway: parallel batches with hogwild
 * writes), only the distributions drawn from it. */
typedef struct { uint64_t s0, s1; } rng_t;
static uint64_t splitmix64(uint64_t* x) {
    uint64_t z = (*x += 0x9e3779b97f4a7c15ULL);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}
static void rng_seed(rng_t* r, uint64_t seed) {
    uint64_t x = seed;
    r->s0 = splitmix64(&x);
    r->s1 = splitmix64(&x);
}
static uint64_t rng_next(rng_t* r) {
    uint64_t a = r->s0, b = r->s1, res = a + b;
    b ^= a;
    r->s0 = ((a << 55) | (a >> 9)) ^ b ^ (b << 14);
    r->s1 = (b << 36) | (b >> 28);
    return res;
}
static float rng_f32(rng_t* r) { return (float)(rng_next(r) >> 40) * (1.0f / 16777216.0f); }
/* uniform in [0, n) */
static uint64_t rng_below(rng_t* r, uint64_t n) {
    if (n <= 1) return 0;
    uint64_t lim = (~(uint64_t)0) - ((~(uint64_t)0) % n);
    uint64_t x;
    do { x = rng_next(r); } while (x >= lim);
    return x % n;
}
static void shuffle_u32(uint32_t* a, uint64_t n, rng_t* r) {
    for (uint64_t i = n; i > 1; --i) {
        uint64_t j = rng_below(r, i);
        uint32_t t = a[i - 1]; a[i - 1] = a[j]; a[j] = t;
    }
}

/* Sample::sample (utils.rs:193-216) with at_least_one = true. */
static void sample_count(int kind, float val, uint64_t n, rng_t* r, uint64_t* k, float* scalar) {
    if (kind == ORC_SAMPLE_FIXED) {
        uint64_t kk = (uint64_t)val;
        uint64_t rr = kk < n ? kk : n;
        *k = rr;
        *scalar = (float)n / (float)rr;
    } else if (kind == ORC_SAMPLE_PROB) {
        uint64_t c = 0;
        for (uint64_t i = 0; i < n; ++i) c += (rng_f32(r) < val);
        if (c == 0) { *k = 1; *scalar = (1.f - powf(val, (float)n)) / val; }
        else { *k = c; *scalar = 1.f / val; }
    } else {
        *k = n;
        *scalar = 1.f;
    }
}

typedef struct {
    fmap_t* maps;
    fmap_t seen;
    gacc_t acc;
    float* vec;
    float* grad;
    float* tmp;
    uint32_t* idx;       /* scratch for choose_multiple / reservoir */
    float* idxw;
    uint64_t idx_cap;
} scratch_t;

static void ensure_idx(scratch_t* s, uint64_t n) {
    if (n <= s->idx_cap) return;
    s->idx = (uint32_t*)realloc(s->idx, n * sizeof(uint32_t));
    s->idxw = (float*)realloc(s->idxw, n * sizeof(float));
    s->idx_cap = n;
}

/* collect_embeddings_from_node (model.rs:257-278). */
static void collect_node(fmap_t* m, const uint64_t* fptr, const uint32_t* fids, uint32_t v,
                         float weight, const orc_train_cfg* cfg, rng_t* r, scratch_t* s) {
    (void)s;
    uint64_t fs = fptr[v], n = fptr[(uint64_t)v + 1] - fs;
    uint64_t k;
    float scalar;
    sample_count(cfg->max_features_kind, cfg->max_features, n, r, &k, &scalar);
    weight += scalar;
    if (k >= n) {
        for (uint64_t j = 0; j < n; ++j) fmap_add(m, fids[fs + j], weight);
        return;
    }
    /* choose_multiple: uniform k-subset by partial Fisher-Yates */
    uint32_t* idx = (uint32_t*)malloc(n * sizeof(uint32_t));
    for (uint64_t j = 0; j < n; ++j) idx[j] = (uint32_t)j;
    for (uint64_t j = 0; j < k; ++j) {
        uint64_t p = j + rng_below(r, n - j);
        uint32_t t = idx[j]; idx[j] = idx[p]; idx[p] = t;
        fmap_add(m, fids[fs + idx[j]], weight);
    }
    free(idx);
}

/* random_walk (node_sampler.rs:109-145): from the anchor, uniform neighbour
 * steps; after the second step each step ends the walk with probability p
 * when off the anchor; at most max_steps steps.  Yields the end node when it
 * is neither the anchor nor one of the anchor's neighbours. */
static int random_walk(uint32_t anchor, const uint64_t* rows, const uint32_t* cols, rng_t* r, float p,
                       uint32_t max_steps, uint32_t* out) {
    uint32_t node = anchor;
    for (uint32_t i = 1;; ++i) {
        const uint64_t s = rows[node], n = rows[(uint64_t)node + 1] - s;
        if (n == 0 || i > max_steps) break;
        node = cols[s + rng_below(r, n)];
        if (i > 1 && rng_f32(r) < p && node != anchor) break;
    }
    if (node == anchor) return 0;
    const uint64_t as = rows[anchor], an = rows[(uint64_t)anchor + 1] - as;
    for (uint64_t j = 0; j < an; ++j)
        if (cols[as + j] == node) return 0;
    *out = node;
    return 1;
}

/* random_walk of the PPR loss (loss.rs:190-222): at most max_steps uniform
 * moves from the anchor; from the second move on the walk stops with
 * probability p unless it stands on the anchor.  Yields the end node, or when
 * that is the anchor a uniform neighbour of it; nothing when the anchor has
 * no edges. */
static int ppr_walk(uint32_t anchor, const uint64_t* rows, const uint32_t* cols, rng_t* r, float p,
                    uint32_t max_steps, uint32_t* out) {
    uint32_t node = anchor;
    for (uint32_t i = 1;; ++i) {
        const uint64_t s = rows[node], n = rows[(uint64_t)node + 1] - s;
        if (n == 0 || i > max_steps) break;
        node = cols[s + rng_below(r, n)];
        if (i > 1 && rng_f32(r) < p && node != anchor) break;
    }
    if (node != anchor) { *out = node; return 1; }
    const uint64_t as = rows[anchor], an = rows[(uint64_t)anchor + 1] - as;
    if (an == 0) return 0;
    *out = cols[as + rng_below(r, an)];
    return 1;
}

/* run_forward_pass (mod.rs:289-327) building the role maps for anchor v. */
static void build_roles(uint32_t v, const uint64_t* rows, const uint32_t* cols,
                        const uint64_t* fptr, const uint32_t* fids,
                        const uint32_t* neg_pool, uint64_t neg_pool_n,
                        const orc_train_cfg* cfg, rng_t* r, scratch_t* s) {
    const uint32_t R = cfg->negatives;
    for (uint32_t q = 0; q < R + 2; ++q) fmap_clear(&s->maps[q]);
    /* h(v) */
    collect_node(&s->maps[0], fptr, fids, v, 1.f, cfg, r, s);
    /* ~h(v): reconstruct_node_embedding (model.rs:342-386), or for PPR the
     * end nodes of R walks with weight 1 each, v itself when there are none
     * (construct_positive, loss.rs:166-187) */
    uint64_t es = rows[v], deg = rows[(uint64_t)v + 1] - es;
    uint64_t ns;
    float sw;
    if (cfg->loss.loss == ORC_LOSS_PPR) {
        uint32_t got = 0;
        for (uint32_t t = 0; t < R; ++t) {
            uint32_t u;
            if (ppr_walk(v, rows, cols, r, cfg->ppr_restart_p, 10, &u)) {
                collect_node(&s->maps[1], fptr, fids, u, 1.f, cfg, r, s);
                ++got;
            }
        }
        if (!got) collect_node(&s->maps[1], fptr, fids, v, 1.f, cfg, r, s);
        ns = deg = 0;
        sw = 1.f;
    } else {
        sample_count(cfg->max_nodes_kind, cfg->max_nodes, deg, r, &ns, &sw);
    }
    if (cfg->loss.loss == ORC_LOSS_PPR) {
        /* done above */
    } else if (deg == ns) {
        for (uint64_t j = 0; j < deg; ++j) collect_node(&s->maps[1], fptr, fids, cols[es + j], sw, cfg, r, s);
    } else {
        /* reservoir_sample (utils.rs:128-145), including its Uniform(0, i) draw */
        ensure_idx(s, ns ? ns : 1);
        uint64_t filled = 0;
        for (uint64_t i = 0; i < deg; ++i) {
            if (i < ns) { s->idx[filled++] = cols[es + i]; }
            else {
                uint64_t j = rng_below(r, i);
                if (j < ns) s->idx[j] = cols[es + i];
            }
        }
        for (uint64_t j = 0; j < filled; ++j) collect_node(&s->maps[1], fptr, fids, s->idx[j], sw, cfg, r, s);
    }
    /* negatives (RandomWalkHardSampler, node_sampler.rs:83-107): up to
     * min(hard, R) distinct walk end nodes from 2 * that many walks, then
     * uniform over the pool */
    uint32_t negs[4096];
    uint32_t nneg = 0;
    const uint32_t H = cfg->hard_negatives < R ? cfg->hard_negatives : R;
    for (uint32_t t = 0; t < 2 * H && nneg < H; ++t) {
        uint32_t u;
        if (random_walk(v, rows, cols, r, 0.25f, 10, &u)) {
            int dup = 0;
            for (uint32_t k = 0; k < nneg; ++k) dup |= negs[k] == u;
            if (!dup) negs[nneg++] = u;
        }
    }
    while (nneg < R) negs[nneg++] = neg_pool[rng_below(r, neg_pool_n)];
    for (uint32_t i = 0; i < R; ++i) collect_node(&s->maps[2 + i], fptr, fids, negs[i], 1.f, cfg, r, s);
}

static double now_s(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

int orc_train(const uint64_t* rows, const uint32_t* cols, const float* wcdf,
              uint64_t n_nodes, const uint64_t* fptr, const uint32_t* fids,
              uint32_t n_feat, const orc_train_cfg* cfg, float* table, int init_given,
              orc_train_stats* stats) {
    (void)wcdf;
    const uint32_t d = cfg->dims, R = cfg->negatives, NR = R + 2, B = cfg->batch_size;
    if (R > 1024 || B == 0 || d == 0) return -1;
    rng_t master;
    rng_seed(&master, cfg->seed);
    if (!init_given) {               /* randomize_embedding_store, mod.rs:381-392 */
        for (uint64_t f = 0; f < n_feat; ++f) {
            float* e = table + f * d;
            float norm = 0.f;
            for (uint32_t k = 0; k < d; ++k) { e[k] = 2.f * rng_f32(&master) - 1.f; norm += powf(e[k], 2.f); }
            norm = sqrtf(norm);
            for (uint32_t k = 0; k < d; ++k) e[k] /= norm;
        }
    }
    float* mom = (float*)calloc((uint64_t)n_feat * d, sizeof(float));
    float* var = (float*)calloc((uint64_t)n_feat * d, sizeof(float));
    /* touch the moment arrays before the timed region: a bounded sample of
     * batches then measures the steady per-batch rate, not the one-time page
     * faults of fresh zero pages that a full pass spreads over all batches */
    {
        const int64_t nel = (int64_t)n_feat * d;
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < nel; i += 1024) {
            mom[i] = 0.f;
            var[i] = 0.f;
        }
    }
    uint32_t* idxs = (uint32_t*)malloc(sizeof(uint32_t) * (n_nodes ? n_nodes : 1));
    for (uint64_t i = 0; i < n_nodes; ++i) idxs[i] = (uint32_t)i;
    shuffle_u32(idxs, n_nodes, &master);
    uint64_t n_valid = (uint64_t)((float)n_nodes * cfg->valid_pct);
    uint64_t n_train = n_nodes - n_valid;
    uint32_t* train = idxs;
    uint32_t* valid = idxs + n_train;
    uint32_t* pool = (uint32_t*)malloc(sizeof(uint32_t) * (n_train ? n_train : 1));
    memcpy(pool, train, sizeof(uint32_t) * n_train);
    uint64_t steps = (uint64_t)ceilf((float)n_train / (float)B);
    uint64_t total = steps * cfg->passes;
    uint64_t warmup = (uint64_t)((float)total / 5.f);
    float min_alpha = cfg->alpha / 100.f;
    uint64_t step = 1;
    uint64_t batches_left = cfg->max_batches ? cfg->max_batches : (uint64_t)-1;
    uint64_t anchors_done = 0, batches_done = 0;
    float last_err = INFINITY, valid_err = INFINITY;
    int nthreads = cfg->threads;
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#else
    nthreads = 1;
#endif
    double shuffle_s = 0.0;
    double t0 = now_s();
    for (uint32_t pass = 1; pass <= cfg->passes && batches_left > 0; ++pass) {
        const double ts0 = now_s();
        shuffle_u32(train, n_train, &master);
        shuffle_s += now_s() - ts0;
        uint64_t nb = steps < batches_left ? steps : batches_left;
        double err_sum = 0.0;
        uint64_t err_cnt = 0;
        uint64_t anchors_pass = 0;
#pragma omp parallel num_threads(nthreads) reduction(+ : err_sum, err_cnt, anchors_pass)
        {
            scratch_t s;
            memset(&s, 0, sizeof(s));
            s.maps = (fmap_t*)calloc(NR, sizeof(fmap_t));
            gacc_init(&s.acc, d);
            s.vec = (float*)malloc(sizeof(float) * NR * d);
            s.grad = (float*)malloc(sizeof(float) * NR * d);
            s.tmp = (float*)malloc(sizeof(float) * (2 * R + 6) * d);
#pragma omp for schedule(dynamic, 1)
            for (uint64_t i = 0; i < nb; ++i) {
                uint64_t b0 = i * B, b1 = b0 + B < n_train ? b0 + B : n_train;
                gacc_clear(&s.acc);
                float err = 0.f;
                uint64_t cnt = 0;
                for (uint64_t j = b0; j < b1; ++j) {
                    uint32_t v = train[j];
                    rng_t r;
                    rng_seed(&r, cfg->seed + i + v);   /* mod.rs:185 */
                    build_roles(v, rows, cols, fptr, fids, pool, n_train, cfg, &r, &s);
                    float wdiv = 1.f;
                    if (cfg->loss.loss_weighting == ORC_LW_LOG)
                        wdiv = logf(1.f + (float)(rows[v + 1] - rows[v]));
                    else if (cfg->loss.loss_weighting == ORC_LW_EXP)
                        wdiv = powf((float)(rows[v + 1] - rows[v]), cfg->loss.lw_exp);
                    float L;
                    int st = anchor_f32(&cfg->loss, s.maps, R, table, d, wdiv, s.vec, s.grad, s.tmp,
                                        &s.seen, &L, &s.acc);
                    if (st == 0) { err += L; ++cnt; }
                }
                uint64_t cur_step;
#pragma omp atomic capture
                cur_step = step++;
                if (cnt > 0) {
                    float lr = orc_lr_cos_decay(min_alpha, cfg->alpha, warmup, total, cur_step);
                    float t = (float)pass + 1.f;
                    for (uint32_t q = 0; q < s.acc.map.n; ++q) {
                        uint32_t f = s.acc.map.keys[q];
                        const float* g = (const float*)gacc_slot(&s.acc, q, sizeof(float));
                        uint64_t o = (uint64_t)f * d;
                        adam_row(table + o, mom + o, var + o, g, d, lr, t);   /* hogwild */
                    }
                }
                float be = cnt > 0 ? err / (float)(b1 - b0) : 0.f;
                if (isinf(be)) be = 0.f;
                err_sum += be;
                err_cnt += 1;
                anchors_pass += b1 - b0;
            }
            for (uint32_t q = 0; q < NR; ++q) fmap_free(&s.maps[q]);
            free(s.maps);
            fmap_free(&s.seen);
            gacc_free(&s.acc);
            free(s.vec); free(s.grad); free(s.tmp); free(s.idx); free(s.idxw);
        }
        batches_left -= nb;
        batches_done += nb;
        anchors_done += anchors_pass;
        last_err = (float)(err_sum / (double)(err_cnt ? err_cnt : 1));
        if (n_valid > 0 && batches_left > 0) {
            double vsum = 0.0;
#pragma omp parallel num_threads(nthreads) reduction(+ : vsum)
            {
                scratch_t s;
                memset(&s, 0, sizeof(s));
                s.maps = (fmap_t*)calloc(NR, sizeof(fmap_t));
                s.vec = (float*)malloc(sizeof(float) * NR * d);
                s.grad = (float*)malloc(sizeof(float) * NR * d);
                s.tmp = (float*)malloc(sizeof(float) * (2 * R + 6) * d);
#pragma omp for schedule(dynamic, 64)
                for (uint64_t j = 0; j < n_valid; ++j) {
                    rng_t r;
                    rng_seed(&r, cfg->seed - 1);        /* mod.rs:273 */
                    build_roles(valid[j], rows, cols, fptr, fids, valid, n_valid, cfg, &r, &s);
                    float L;
                    anchor_f32(&cfg->loss, s.maps, R, table, d, 1.f, s.vec, s.grad, s.tmp, &s.seen, &L, NULL);
                    vsum += L;
                }
                for (uint32_t q = 0; q < NR; ++q) fmap_free(&s.maps[q]);
                free(s.maps);
                fmap_free(&s.seen);
                free(s.vec); free(s.grad); free(s.tmp); free(s.idx); free(s.idxw);
            }
            valid_err = (float)(vsum / (double)n_valid);
        }
    }
    double t1 = now_s();
    if (stats) {
        stats->seconds = t1 - t0;
        stats->shuffle_seconds = shuffle_s;
        stats->steps_per_pass = steps;
        stats->anchors = anchors_done;
        stats->batches = batches_done;
        stats->last_train_loss = last_err;
        stats->last_valid_loss = valid_err;
    }
    free(mom); free(var); free(idxs); free(pool);
    return 0;
}

/* Exported aliases for the batch routine (names without the underscore). */
int orc_batch_f32(const uint64_t* fptr, const uint32_t* fids, uint32_t n_feat,
                  const float* table, uint32_t d, const uint64_t* graph_rows,
                  uint32_t B, const uint32_t* anchors, const uint32_t* nbr_ptr,
                  const uint32_t* nbr, const float* nbr_w, uint32_t R,
                  const uint32_t* neg, const orc_loss_cfg* cfg,
                  float* loss_out, int32_t* status_out, float* grad_out,
                  uint8_t* touched) {
    return batch_impl_f32(fptr, fids, n_feat, table, d, graph_rows, B, anchors, nbr_ptr,
                              nbr, nbr_w, R, neg, cfg, loss_out, status_out, grad_out, touched);
}
int orc_batch_f64(const uint64_t* fptr, const uint32_t* fids, uint32_t n_feat,
                  const float* table, uint32_t d, const uint64_t* graph_rows,
                  uint32_t B, const uint32_t* anchors, const uint32_t* nbr_ptr,
                  const uint32_t* nbr, const float* nbr_w, uint32_t R,
                  const uint32_t* neg, const orc_loss_cfg* cfg,
                  double* loss_out, int32_t* status_out, double* grad_out,
                  uint8_t* touched) {
    return batch_impl_f64(fptr, fids, n_feat, table, d, graph_rows, B, anchors, nbr_ptr,
                              nbr, nbr_w, R, neg, cfg, loss_out, status_out, grad_out, touched);
}
