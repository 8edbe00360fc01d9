// ep_fwd.cu -- sampling, gather-mean + loss + gradient-direction kernel, and
// the per-batch bookkeeping kernels.
//
// Reference behaviour restated here (cloverleaf, Rust):
//   anchor order per pass      src/algos/ep/mod.rs:172-174 (shuffle, chunks)
//   neighbour reconstruction   src/algos/ep/model.rs:342-386, utils.rs:193-216
//   negatives                  src/algos/grad_utils/node_sampler.rs:243-246
//   role means                 src/algos/ep/model.rs:257-301, 388-416, 448-463
//   losses                     src/algos/ep/loss.rs:56-129, 229-243
//   loss weighting             src/algos/ep/mod.rs:190-200
//   learning rate              src/algos/grad_utils/scheduler.rs:120-137
#include <cuda_runtime.h>
#include <math.h>

#include <algorithm>
#include <type_traits>

#include "ep_device.cuh"
#include "ep_internal.h"
#include "ep_launch.cuh"

namespace ep {

enum { LOSS_MARGIN = 0, LOSS_STARSPACE = 1, LOSS_CONTRASTIVE = 2, LOSS_RANK = 3, LOSS_RANKSPACE = 4 };
enum { S_ALL = 0, S_FIXED = 1, S_PROB = 2 };
enum { LW_NONE = 0, LW_LOG = 1, LW_EXP = 2 };

// ---------------------------------------------------------------------------
// Feature dropout (max_features; model.rs:257-278 with Sample::sample,
// utils.rs:193-216).  Node u in slot q of anchor v (q = 0 the anchor, then
// its sampled neighbours, then its negatives) keeps a subset of its n
// features and adds the sample's scalar to its count weight:
//   Fixed(k)  the min(k, n) positions with the smallest keys (equal keys in
//             position order): a uniform k-subset; scalar n / min(k, n)
//   Prob(p)   the positions whose key < p * 2^32 (Bernoulli(p) each); if
//             none, the one with the smallest key, scalar (1 - p^n) / p;
//             else scalar 1 / p
//   All       every position; scalar 1
// Keys are Philox draws of (v, step, q, position).  k_sample counts the kept
// positions and the gathers enumerate them from the same keys, so the item
// offsets and the emitted items agree exactly.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t fd_key(const FeatDrop& fd, uint32_t v, uint32_t salt, uint32_t q, uint32_t j) {
    return rand_u32(fd.seed, v, salt, ST_FSEL, ((q & 0x3ffu) << 16) | (j & 0xffffu));
}

// Kept count of one node (one thread) and the scalar added to its weight.
__device__ __forceinline__ uint32_t fd_kept(const FeatDrop& fd, uint32_t v, uint32_t salt, uint32_t q, uint32_t n,
                                            float& scalar) {
    scalar = 1.f;
    if (fd.kind == S_ALL || n == 0) return n;
    if (fd.kind == S_FIXED) {
        const uint32_t k = min(fd.k, n);
        scalar = (float)n / (float)k;
        return k;
    }
    uint32_t c = 0;
    for (uint32_t j = 0; j < n; ++j) c += fd_key(fd, v, salt, q, j) < fd.thr;
    if (c == 0) {
        scalar = (1.f - powf(fd.p, (float)n)) / fd.p;
        return 1;
    }
    scalar = 1.f / fd.p;
    return c;
}

// Probability sampling of one node (warp): whether no position passed, and
// the position with the smallest key.
struct FdNode {
    bool none;
    uint32_t argmin;
};

__device__ __forceinline__ FdNode fd_node(const FeatDrop& fd, uint32_t v, uint32_t salt, uint32_t q, uint32_t n,
                                          int lane) {
    FdNode r{false, 0u};
    if (fd.kind != S_PROB || n == 0) return r;
    uint32_t cnt = 0;
    unsigned long long best = ~0ull;
    for (uint32_t j0 = 0; j0 < n; j0 += 32) {
        const uint32_t j = j0 + lane;
        const bool in = j < n;
        const uint32_t key = in ? fd_key(fd, v, salt, q, j) : 0xffffffffu;
        cnt += __popc(__ballot_sync(FULL, in && key < fd.thr));
        if (in) best = min(best, ((unsigned long long)key << 32) | j);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) best = min(best, __shfl_xor_sync(FULL, best, o));
    r.none = cnt == 0;
    r.argmin = (uint32_t)best;
    return r;
}

// Kept positions j0 .. j0+31 of one node as a lane mask (warp).
__device__ __forceinline__ unsigned fd_mask(const FeatDrop& fd, const FdNode& nd, uint32_t v, uint32_t salt,
                                            uint32_t q, uint32_t n, uint32_t j0, int lane) {
    const uint32_t j = j0 + lane;
    const bool in = j < n;
    bool sel = in;
    if (fd.kind == S_PROB) {
        sel = in && (nd.none ? j == nd.argmin : fd_key(fd, v, salt, q, j) < fd.thr);
    } else if (fd.kind == S_FIXED && min(fd.k, n) < n) {
        const uint32_t k = min(fd.k, n);
        const uint32_t kj = in ? fd_key(fd, v, salt, q, j) : 0xffffffffu;
        uint32_t rank = 0;
        for (uint32_t i0 = 0; i0 < n; i0 += 32) {
            const uint32_t ki = i0 + lane < n ? fd_key(fd, v, salt, q, i0 + lane) : 0xffffffffu;
            for (int t = 0; t < 32; ++t) {
                const uint32_t kt = __shfl_sync(FULL, ki, t);
                const uint32_t it = i0 + (uint32_t)t;
                rank += (it < n) && (kt < kj || (kt == kj && it < j));
            }
        }
        sel = in && rank < k;
    }
    return __ballot_sync(FULL, sel);
}

// ---------------------------------------------------------------------------
// Per-pass anchor order: a keyed Feistel bijection on [0, 2^(2h)) restricted
// to [0, n) by cycle walking.  Replaces the host shuffle of mod.rs:173 with an
// O(1)-per-position permutation that needs no buffer and no sort.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t feistel(uint32_t x, uint32_t h, const uint32_t* k) {
    const uint32_t mask = h >= 32 ? 0xffffffffu : ((1u << h) - 1u);
    uint32_t L = (h >= 32) ? 0 : (x >> h), Rr = x & mask;
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        uint32_t F = mix32(Rr ^ k[r]) & mask;
        uint32_t nL = Rr;
        Rr = L ^ F;
        L = nL;
    }
    return (L << h) | Rr;
}

__device__ __forceinline__ uint32_t permute(uint32_t pos, uint32_t n, uint32_t h, const uint32_t* k,
                                            uint32_t* err) {
    uint32_t x = pos;
    for (int it = 0; it < 128; ++it) {
        x = feistel(x, h, k);
        if (x < n) return x;
    }
    atomicOr(err, ERR_FEISTEL);
    return pos % n;
}

// ---------------------------------------------------------------------------
// k_batch_begin: batch range, learning rate and Adam bias corrections.
// ---------------------------------------------------------------------------
__global__ void k_batch_begin(BatchState* st, uint32_t n_order, uint32_t cap, uint64_t total,
                              uint64_t warmup, float alpha, int injected, float noise, float noise_decay) {
    pdl_wait();
    pdl_trigger();
    if (threadIdx.x != 0) return;
    if (!injected) {
        uint32_t b0 = st->batch * cap;
        st->b0 = b0;
        st->n_anchors = b0 < n_order ? min(cap, n_order - b0) : 0;
    }
    // LRScheduler::CosDecay(alpha/100, alpha, warmup, total) (mod.rs:133-137)
    const float min_alpha = alpha / 100.f;
    const uint64_t s = st->step;
    float lr;
    if (s > warmup) {
        float ratio = (float)s / (float)total;
        lr = min_alpha + 0.5f * (alpha - min_alpha) * (1.f + cosf(3.14159265358979323846f * ratio));
    } else {
        float ratio = (float)s / (float)warmup;
        lr = min_alpha + ratio * (alpha - min_alpha);
    }
    st->lr = lr;
    st->step_cur = (uint32_t)s;
    // gradient noise: LRScheduler::exp_decay(0, noise, decay) at this step
    // (mod.rs:140-146; scheduler.rs:50-52); injected batches keep their value
    if (!injected) st->noise_sigma = noise > 1e-9f ? fmaxf(noise * powf(noise_decay, (float)s), 0.f) : 0.f;
    const float t = (float)st->pass + 1.f;
    st->bc1 = 1.f - powf(0.9f, t);
    st->bc2 = 1.f - powf(0.999f, t);
    st->n_items = 0;
    st->fwd_next = 0;
    st->red_next = 0;
    st->n_long[s & 1u] = 0;
}

// ---------------------------------------------------------------------------
// Weighted neighbour sampling with weighted averaging: weighted_reservoir_
// sample (utils.rs:147-161) with the averaging weights w_i = scale * p_i * deg
// (CDFtoP, graph.rs:630-661) keeps the r positions with the largest
// U_i^(1/w_i) (Efraimidis-Spirakis A-Res), compared here as log(U_i) / w_i.
// Both selectors write the chosen positions (as float bits) to outw[0, r)
// and their node ids to out[0, r); the caller turns positions into weights.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float ares_key(const SampleParams& p, uint64_t rs, uint32_t i, uint32_t deg, float sw,
                                          uint32_t v, uint32_t salt) {
    const float pi = p.wcdf[rs + i] - (i ? p.wcdf[rs + i - 1] : 0.f);
    const float wi = sw * pi * (float)deg;
    const float u = ((float)(rand_u32(p.cfg.seed, v, salt, ST_WRES, i) >> 8) + 0.5f) * (1.0f / 16777216.0f);
    return wi > 0.f ? __logf(u) / wi : -INFINITY;
}

// r <= 32: lane t < r holds one member of the running set; 32 candidates at a
// time enter while they beat the set's smallest key.
__device__ void ares_small(const SampleParams& p, uint64_t rs, uint32_t deg, float sw, uint32_t r, uint32_t v,
                           uint32_t salt, uint32_t* out, float* outw, int lane) {
    float skey = -INFINITY;
    uint32_t spos = 0xffffffffu;
    if ((uint32_t)lane < r) { spos = (uint32_t)lane; skey = ares_key(p, rs, lane, deg, sw, v, salt); }
    for (uint32_t base = r; base < deg; base += 32) {
        const uint32_t i = base + lane;
        float ck = i < deg ? ares_key(p, rs, i, deg, sw, v, salt) : -INFINITY;
        for (uint32_t guard = 0; guard <= 32; ++guard) {
            // the set's smallest key and the lane holding it
            float mk = (uint32_t)lane < r ? skey : INFINITY;
            int ml = lane;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const float ok2 = __shfl_xor_sync(FULL, mk, o);
                const int ol = __shfl_xor_sync(FULL, ml, o);
                if (ok2 < mk || (ok2 == mk && ol < ml)) { mk = ok2; ml = ol; }
            }
            const bool better = ck > mk;
            if (!__ballot_sync(FULL, better)) break;
            // the best candidate replaces the smallest member
            float bk = better ? ck : -INFINITY;
            int bl = lane;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const float ok2 = __shfl_xor_sync(FULL, bk, o);
                const int ol = __shfl_xor_sync(FULL, bl, o);
                if (ok2 > bk || (ok2 == bk && ol < bl)) { bk = ok2; bl = ol; }
            }
            const uint32_t bpos = __shfl_sync(FULL, i, bl);
            if (lane == ml) { skey = bk; spos = bpos; }
            if (lane == bl) ck = -INFINITY;
        }
    }
    if ((uint32_t)lane < r) { out[lane] = p.cols[rs + spos]; outw[lane] = __uint_as_float(spos); }
}

// Order-preserving image of a float key as an unsigned integer.
__device__ __forceinline__ uint32_t key_ord(float k) {
    const uint32_t b = __float_as_uint(k);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

// Any r < deg: the r-th largest key by an MSB-first radix select over key_ord
// (four 8-bit passes over a 256-bin warp histogram in shared memory, the keys
// recomputed from the same draws each pass), then every position above that
// key plus the lowest-placed ties, in position order.
__device__ void ares_select(const SampleParams& p, uint64_t rs, uint32_t deg, float sw, uint32_t r, uint32_t v,
                            uint32_t salt, uint32_t* out, float* outw, uint32_t* hist, int lane) {
    uint32_t prefix = 0, pmask = 0, need = r;        // need: rank of the target within the prefix group
    for (int shift = 24; shift >= 0; shift -= 8) {
        for (uint32_t b = lane; b < 256; b += 32) hist[b] = 0;
        __syncwarp();
        for (uint32_t i0 = 0; i0 < deg; i0 += 32) {
            const uint32_t i = i0 + lane;
            if (i < deg) {
                const uint32_t o = key_ord(ares_key(p, rs, i, deg, sw, v, salt));
                if ((o & pmask) == prefix) atomicAdd(&hist[(o >> shift) & 255u], 1u);
            }
        }
        __syncwarp();
        // bins from the top: lane l holds bins 255 - 8l ... 248 - 8l
        uint32_t cnt[8], tot = 0;
#pragma unroll
        for (int j = 0; j < 8; ++j) { cnt[j] = hist[255 - (lane * 8 + j)]; tot += cnt[j]; }
        const uint32_t incl = warp_incl_scan(tot, lane), excl = incl - tot;
        const unsigned hit = __ballot_sync(FULL, excl < need && need <= incl);
        const int L = __ffs(hit) - 1;                 // need <= group size, so one lane holds it
        uint32_t dig = 0, above = 0;
        if (lane == L) {
            uint32_t acc = excl;
            for (int j = 0; j < 8; ++j) {
                if (acc + cnt[j] >= need) { dig = 255u - (uint32_t)(lane * 8 + j); above = acc; break; }
                acc += cnt[j];
            }
        }
        dig = __shfl_sync(FULL, dig, L);
        above = __shfl_sync(FULL, above, L);
        need -= above;
        prefix |= dig << shift;
        pmask |= 255u << shift;
        __syncwarp();
    }
    // prefix: the r-th largest image; need: how many of its ties to keep
    uint32_t taken = 0, ties = 0;
    for (uint32_t i0 = 0; i0 < deg && taken < r; i0 += 32) {
        const uint32_t i = i0 + lane;
        const uint32_t o = i < deg ? key_ord(ares_key(p, rs, i, deg, sw, v, salt)) : 0u;
        const bool eq = i < deg && o == prefix;
        const unsigned em = __ballot_sync(FULL, eq);
        const bool take = (i < deg && o > prefix) || (eq && ties + __popc(em & ((1u << lane) - 1u)) < need);
        const unsigned tm = __ballot_sync(FULL, take);
        if (take) {
            const uint32_t slot = taken + __popc(tm & ((1u << lane) - 1u));
            out[slot] = p.cols[rs + i];
            outw[slot] = __uint_as_float(i);
        }
        taken += __popc(tm);
        ties += __popc(em);
    }
}

// ---------------------------------------------------------------------------
// k_sample: one warp per anchor.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_sample(SampleParams p) {
    __shared__ uint32_t s_hist[8][256];   // per warp: ares_select's histogram
    pdl_wait();
    pdl_trigger();
    const int lane = threadIdx.x & 31;
    const uint32_t a = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    BatchState* st = p.st;
    const uint32_t n = st->n_anchors;
    if (a >= n) return;
    const SampleCfg& c = p.cfg;
    const uint32_t salt = p.eval ? 0xffffffffu : (uint32_t)st->step;
    uint32_t v;
    if (p.injected == 1) {
        v = p.anchors[a];
    } else {
        if (p.injected == 2) {
            v = p.anchors[a];
        } else {
            const uint32_t pos = st->b0 + a;
            uint32_t idx = pos;
            if (!p.eval) {
                uint32_t k[4];
                u32x4 kk = philox(u32x4{st->pass, 0x9e3779b9u, 0x7f4a7c15u, 0x1234567u}, c.seed);
                k[0] = kk.x; k[1] = kk.y; k[2] = kk.z; k[3] = kk.w;
                idx = permute(pos, p.n_order, p.feistel_half, k, &st->error);
            }
            v = p.order[idx];
            if (lane == 0) p.anchors[a] = v;
        }

        // --- neighbours (reconstruct_node_embedding, model.rs:342-386) ---
        const uint64_t rs = p.row_ptr[v];
        const uint32_t deg = (uint32_t)(p.row_ptr[v + 1] - rs);
        uint32_t* out = p.nbr + (uint64_t)a * c.Kcap;
        float* outw = p.nbr_w + (uint64_t)a * c.Kcap;
        uint32_t cnt = 0;
        float sw = 1.f;
        int take_all = 0;
        if (c.ppr) {
            // PPR positives (loss.rs:166-187): the end nodes of R random
            // walks from v (random_walk, loss.rs:190-222), weight 1 each, in
            // walk order; v itself when no walk yields one.  A walk makes at
            // most 10 moves and, from the second move on, stops with
            // probability restart_p unless it stands on v; ending on v
            // yields a uniform neighbour of v instead (none when deg = 0).
            uint32_t got = 0;
            for (uint32_t w0 = 0; w0 < c.R; w0 += 32) {
                const uint32_t t = w0 + lane;
                uint32_t node = v;
                bool some = false;
                if (t < c.R) {
                    for (uint32_t i = 1; i <= 10; ++i) {
                        const uint64_t ns = p.row_ptr[node];
                        const uint32_t nd = (uint32_t)(p.row_ptr[node + 1] - ns);
                        if (nd == 0) break;
                        node = p.cols[ns + below(rand_u32(c.seed, v, salt, ST_PPR, t * 32 + 2 * i), nd)];
                        if (i > 1 && node != v &&
                            unit_f32(rand_u32(c.seed, v, salt, ST_PPR, t * 32 + 2 * i + 1)) < c.ppr_restart)
                            break;
                    }
                    if (node != v) {
                        some = true;
                    } else if (deg > 0) {
                        node = p.cols[rs + below(rand_u32(c.seed, v, salt, ST_PPR, t * 32 + 31), deg)];
                        some = true;
                    }
                }
                const unsigned m = __ballot_sync(FULL, some);
                const uint32_t rank = __popc(m & ((1u << lane) - 1u));
                if (some) { out[got + rank] = node; outw[got + rank] = 1.f; }
                got += (uint32_t)__popc(m);
            }
            if (got == 0) {
                if (lane == 0) { out[0] = v; outw[0] = 1.f; }
                got = 1;
            }
            cnt = got;
            __syncwarp();
        } else if (c.nodes_kind == S_ALL) {
            take_all = 1;
        } else if (c.nodes_kind == S_FIXED) {
            const uint32_t r = min(c.K, deg);
            sw = (float)deg / (float)r;
            if (r == deg) {
                take_all = 1;
            } else if (c.weighted_sampling && c.weighted_avg && p.wcdf) {
                if (r <= 32) ares_small(p, rs, deg, sw, r, v, salt, out, outw, lane);
                else ares_select(p, rs, deg, sw, r, v, salt, out, outw, s_hist[(threadIdx.x >> 5) & 7], lane);
                cnt = r;
            } else if (r <= 32) {
                // Floyd's algorithm: a uniform r-subset of [0, deg); lane i
                // holds the i-th chosen position.  The draw of step it does
                // not depend on the set chosen so far, so lane it makes it
                // up front and the steps only test membership.
                uint32_t mine = 0xffffffffu;
                const uint32_t my_draw =
                    (uint32_t)lane < r ? below(rand_u32(c.seed, v, salt, ST_NBR, (uint32_t)lane), deg - r + (uint32_t)lane + 1)
                                       : 0u;
                for (uint32_t it = 0; it < r; ++it) {
                    const uint32_t j = deg - r + it;
                    const uint32_t tpos = __shfl_sync(FULL, my_draw, (int)it);
                    const unsigned hit = __ballot_sync(FULL, mine == tpos);
                    const uint32_t pick = hit ? j : tpos;
                    if (lane == (int)it) mine = pick;
                }
                if ((uint32_t)lane < r) { out[lane] = p.cols[rs + mine]; outw[lane] = __uint_as_float(mine); }
                cnt = r;
            } else if (r <= c.Kcap) {
                // Floyd with the chosen set kept in the output slots (the
                // draws made 32 steps at a time, lane i for step it0 + i).
                uint32_t my_draw = 0;
                for (uint32_t it = 0; it < r; ++it) {
                    const uint32_t j = deg - r + it;
                    if ((it & 31u) == 0) {
                        const uint32_t q = it + (uint32_t)lane;
                        my_draw = q < r ? below(rand_u32(c.seed, v, salt, ST_NBR, q), deg - r + q + 1) : 0u;
                    }
                    const uint32_t tpos = __shfl_sync(FULL, my_draw, (int)(it & 31u));
                    bool found = false;
                    for (uint32_t b = 0; b < it; b += 32) {
                        const uint32_t q = b + lane;
                        const bool m = q < it && out[q] == tpos;
                        if (__any_sync(FULL, m)) { found = true; break; }
                    }
                    if (lane == 0) out[it] = found ? j : tpos;
                    __syncwarp();
                }
                for (uint32_t q = lane; q < r; q += 32) {
                    const uint32_t pos2 = out[q];
                    outw[q] = __uint_as_float(pos2);
                    out[q] = p.cols[rs + pos2];
                }
                cnt = r;
            } else {
                if (lane == 0) atomicOr(&st->error, ERR_NBR_OVERFLOW);
                cnt = 0;
            }
            __syncwarp();
        } else if (c.weighted_sampling && c.weighted_avg && p.wcdf) {
            // S_PROB with weighted sampling: the Binomial(deg, p) count (at
            // least one), then that many by weight
            const float pr = c.nodes_val;
            uint32_t r = 0;
            for (uint32_t b = 0; b < deg; b += 32) {
                const uint32_t q = b + lane;
                r += __popc(__ballot_sync(FULL, q < deg && unit_f32(rand_u32(c.seed, v, salt, ST_NSEL, q)) < pr));
            }
            sw = 1.f / pr;
            if (r == 0 && deg > 0) { r = 1; sw = (1.f - powf(pr, (float)deg)) / pr; }
            if (r == deg) {
                take_all = 1;
            } else if (r <= c.Kcap) {
                if (r <= 32) ares_small(p, rs, deg, sw, r, v, salt, out, outw, lane);
                else ares_select(p, rs, deg, sw, r, v, salt, out, outw, s_hist[(threadIdx.x >> 5) & 7], lane);
                cnt = r;
            } else {
                if (lane == 0) atomicOr(&st->error, ERR_NBR_OVERFLOW);
                cnt = 0;
            }
            __syncwarp();
        } else {  // S_PROB: independent Bernoulli(p) per neighbour == Binomial count + uniform subset
            const float pr = c.nodes_val;
            uint32_t sel_total = 0;
            for (uint32_t b = 0; b < deg; b += 32) {
                uint32_t q = b + lane;
                bool s = q < deg && unit_f32(rand_u32(c.seed, v, salt, ST_NSEL, q)) < pr;
                unsigned bm = __ballot_sync(FULL, s);
                uint32_t off = sel_total + __popc(bm & ((1u << lane) - 1u));
                if (s && off < c.Kcap) { out[off] = p.cols[rs + q]; outw[off] = __uint_as_float(q); }
                sel_total += __popc(bm);
            }
            if (sel_total > c.Kcap) {
                if (lane == 0) atomicOr(&st->error, ERR_NBR_OVERFLOW);
                sel_total = c.Kcap;
            }
            if (sel_total == 0 && deg > 0) {
                uint32_t q = below(rand_u32(c.seed, v, salt, ST_NSEL, deg), deg);
                if (lane == 0) { out[0] = p.cols[rs + q]; outw[0] = __uint_as_float(q); }
                sel_total = 1;
                sw = (1.f - powf(pr, (float)deg)) / pr;
            } else {
                sw = 1.f / pr;
            }
            if (sel_total == deg) take_all = 1;
            else cnt = sel_total;
            __syncwarp();
        }
        if (take_all) {
            if (deg > c.Kcap) {
                if (lane == 0) atomicOr(&st->error, ERR_NBR_OVERFLOW);
                cnt = 0;
            } else {
                for (uint32_t q = lane; q < deg; q += 32) { out[q] = p.cols[rs + q]; outw[q] = __uint_as_float(q); }
                cnt = deg;
            }
        }
        __syncwarp();
        // weights: scale_weight, or scale * p_j * deg when averaging by edge
        // weight (CDFtoP, graph.rs:630-661)
        for (uint32_t q = lane; q < cnt && !c.ppr; q += 32) {
            float w = sw;
            if (c.weighted_avg && p.wcdf) {
                const uint32_t pos2 = __float_as_uint(outw[q]);
                float pj = p.wcdf[rs + pos2] - (pos2 ? p.wcdf[rs + pos2 - 1] : 0.f);
                w = sw * pj * (float)deg;
            }
            outw[q] = w;
        }
        if (lane == 0) p.nbr_cnt[a] = cnt;
        // --- negatives: first up to min(hard, R) hard negatives, the end nodes
        // of random walks from the anchor (RandomWalkHardSampler,
        // node_sampler.rs:83-145), then uniform over the pool, with replacement
        uint32_t* negs = p.neg + (uint64_t)a * c.R;
        uint32_t nh = 0;
        const uint32_t H = min(c.hard, c.R);
        if (H) {
            const uint32_t walks = 2 * H;
            const uint64_t ae = rs + deg;
            for (uint32_t w0 = 0; w0 < walks && nh < H; w0 += 32) {
                const uint32_t t = w0 + lane;
                uint32_t node = v;
                bool ok = false;
                if (t < walks) {
                    // restart probability 0.25 after the second step, at most
                    // 10 moves (random_walk, node_sampler.rs:109-145)
                    for (uint32_t i = 1; i <= 11; ++i) {
                        const uint64_t ns = p.row_ptr[node];
                        const uint32_t nd = (uint32_t)(p.row_ptr[node + 1] - ns);
                        if (nd == 0 || i > 10) break;
                        node = p.cols[ns + below(rand_u32(c.seed, v, salt, ST_HARD, t * 32 + 2 * i), nd)];
                        if (i > 1 && node != v && unit_f32(rand_u32(c.seed, v, salt, ST_HARD, t * 32 + 2 * i + 1)) < 0.25f)
                            break;
                    }
                    ok = node != v;
                }
                // not one of the anchor's neighbours: the warp scans the row,
                // each lane tests its own end node
                bool hit = false;
                for (uint64_t b = rs; b < ae; b += 32) {
                    const uint32_t x = b + lane < ae ? p.cols[b + lane] : 0u;
                    const uint32_t m = (uint32_t)min((uint64_t)32, ae - b);
                    for (uint32_t s2 = 0; s2 < m; ++s2) {
                        const uint32_t y = __shfl_sync(FULL, x, s2);   // every lane takes part
                        hit = hit || y == node;
                    }
                }
                ok = ok && !hit;
                // keep the first occurrence among valid end nodes, in walk order
                bool dup = false;
                for (int s2 = 0; s2 < 32; ++s2) {
                    const uint32_t ns2 = __shfl_sync(FULL, node, s2);
                    const bool ok2 = __shfl_sync(FULL, ok, s2);
                    dup = dup || (s2 < lane && ok2 && ns2 == node);
                }
                for (uint32_t k2 = 0; k2 < nh; ++k2) dup = dup || negs[k2] == node;
                const bool acc = ok && !dup;
                const unsigned am = __ballot_sync(FULL, acc);
                const uint32_t rank = __popc(am & ((1u << lane) - 1u));
                if (acc && nh + rank < H) negs[nh + rank] = node;
                __syncwarp();
                nh = min(H, nh + (uint32_t)__popc(am));
            }
        }
        for (uint32_t i = nh + lane; i < c.R; i += 32)
            negs[i] = p.pool[below(rand_u32(c.seed, v, salt, ST_NEG, i), p.n_pool)];
        __syncwarp();
    }
    // --- item count of this anchor: kept feature counts over its roles ---
    const uint32_t cnt = p.nbr_cnt[a];
    uint64_t occ = 0;
    float unused;
    if (lane == 0) occ += fd_kept(c.fd, v, salt, 0, (uint32_t)(p.fptr[v + 1] - p.fptr[v]), unused);
    const uint32_t* nb = p.nbr + (uint64_t)a * c.Kcap;
    for (uint32_t q = lane; q < cnt; q += 32) {
        const uint32_t u = nb[q];
        occ += fd_kept(c.fd, v, salt, 1 + q, (uint32_t)(p.fptr[u + 1] - p.fptr[u]), unused);
    }
    const uint32_t* ng = p.neg + (uint64_t)a * c.R;
    for (uint32_t q = lane; q < c.R; q += 32) {
        const uint32_t u = ng[q];
        occ += fd_kept(c.fd, v, salt, 1 + cnt + q, (uint32_t)(p.fptr[u + 1] - p.fptr[u]), unused);
    }
    occ = warp_sum<unsigned long long>((unsigned long long)occ);
    if (lane == 0) p.occ[a] = (uint32_t)min(occ, (uint64_t)0xffffffffu);
}

// ---------------------------------------------------------------------------
// k_scan_occ: exclusive scan of the per-anchor item counts (one CTA).  Each
// thread scans 8 consecutive counts in registers, so a batch of up to 8192
// anchors is one sweep: loads, a block scan of the thread totals, stores.
// ---------------------------------------------------------------------------
constexpr int SCAN_PER_THREAD = 8;

__global__ void __launch_bounds__(1024) k_scan_occ(BatchState* st, uint32_t* occ, uint64_t items_cap) {
    pdl_wait();
    pdl_trigger();
    __shared__ unsigned long long warp_tot[32];
    const uint32_t n = st->n_anchors;
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    unsigned long long carry = 0;
    for (uint32_t base = 0; base < n; base += 1024 * SCAN_PER_THREAD) {
        const uint32_t i0 = base + (uint32_t)tid * SCAN_PER_THREAD;
        uint32_t x[SCAN_PER_THREAD];
#pragma unroll
        for (int k = 0; k < SCAN_PER_THREAD; ++k) x[k] = i0 + k < n ? occ[i0 + k] : 0u;
        unsigned long long tsum = 0;
#pragma unroll
        for (int k = 0; k < SCAN_PER_THREAD; ++k) tsum += x[k];
        unsigned long long incl = tsum;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned long long t = __shfl_up_sync(FULL, incl, o);
            if (lane >= o) incl += t;
        }
        if (lane == 31) warp_tot[w] = incl;
        __syncthreads();
        if (w == 0) {
            unsigned long long s = warp_tot[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const unsigned long long t = __shfl_up_sync(FULL, s, o);
                if (lane >= o) s += t;
            }
            warp_tot[lane] = s;
        }
        __syncthreads();
        unsigned long long run = carry + (w ? warp_tot[w - 1] : 0ull) + incl - tsum;
#pragma unroll
        for (int k = 0; k < SCAN_PER_THREAD; ++k) {
            if (i0 + k < n) occ[i0 + k] = (uint32_t)min(run, 0xffffffffull);
            run += x[k];
        }
        carry += warp_tot[31];
        __syncthreads();
    }
    if (tid == 0) {
        unsigned long long total = carry;
        if (total > items_cap) {
            atomicOr(&st->error, ERR_ITEMS_OVERFLOW);
            total = 0;
        }
        occ[n] = (uint32_t)total;
        st->n_items = (uint32_t)total;
    }
}

// ---------------------------------------------------------------------------
// k_forward: one warp per anchor.
// ---------------------------------------------------------------------------
template <typename T, typename A, int VPL>
__device__ __forceinline__ void fma_row(A (&acc)[VPL], A c, const A (&r)[VPL]) {
    axpy_slice<A, VPL>(acc, c, r);
}

// Gathers one role: the (weighted) mean numerator over every feature
// occurrence of `count` nodes, returning the weight total.  Emits one item
// per occurrence at item positions pos, pos+1, ... (role-major, node order,
// feature order), which keeps items ordered by (anchor, role).
template <typename T, typename A, int VPL>
__device__ A gather_role(const ForwardParams& p, const T* __restrict__ table, const uint32_t* nodes,
                         const float* w, uint32_t count, uint32_t src, uint64_t& pos, bool emit,
                         A (&acc)[VPL], int lane, bool lane_on) {
#pragma unroll
    for (int k = 0; k < VPL; ++k) acc[k] = 0;
    A ntot = 0;
    const uint32_t dpad = p.dpad;
    for (uint32_t base = 0; base < count; base += 32) {
        const uint32_t q = base + lane;
        uint64_t fs = 0;
        uint32_t fn = 0;
        float c = 0.f;
        if (q < count) {
            const uint32_t u = nodes[q];
            fs = p.fptr[u];
            fn = (uint32_t)(p.fptr[u + 1] - fs);
            c = (w ? w[q] : 1.f) + 1.f;   // Sample::All features: scalar 1
        }
        const uint32_t incl = warp_incl_scan(fn, lane);
        const uint32_t total = __shfl_sync(FULL, incl, 31);
        ntot += warp_sum<A>((A)c * (A)fn);
        for (uint32_t ob = 0; ob < total; ob += 32) {
            const uint32_t o = ob + lane;
            int qq = 0;
#pragma unroll
            for (int s = 16; s >= 1; s >>= 1) {
                uint32_t iv = __shfl_sync(FULL, incl, qq + s - 1);
                if (iv <= o) qq += s;
            }
            const int qs = qq > 31 ? 31 : qq;
            const uint32_t excl_q = __shfl_sync(FULL, incl - fn, qs);
            const uint32_t fs_lo = __shfl_sync(FULL, (uint32_t)fs, qs);
            const uint32_t fs_hi = __shfl_sync(FULL, (uint32_t)(fs >> 32), qs);
            const float cq = __shfl_sync(FULL, c, qs);
            const bool active = o < total;
            uint32_t f = 0;
            if (active) f = p.fids[(((uint64_t)fs_hi << 32) | fs_lo) + (o - excl_q)];
            if (emit && active) {
                p.item_f[pos + o] = f;
                p.item_src[pos + o] = src;
                p.item_c[pos + o] = cq;
            }
            const uint32_t m = min(32u, total - ob);
            uint32_t j = 0;
            for (; j + 4 <= m; j += 4) {
                const uint32_t f0 = __shfl_sync(FULL, f, j), f1 = __shfl_sync(FULL, f, j + 1);
                const uint32_t f2 = __shfl_sync(FULL, f, j + 2), f3 = __shfl_sync(FULL, f, j + 3);
                const A c0 = (A)__shfl_sync(FULL, cq, j), c1 = (A)__shfl_sync(FULL, cq, j + 1);
                const A c2 = (A)__shfl_sync(FULL, cq, j + 2), c3 = (A)__shfl_sync(FULL, cq, j + 3);
                if (lane_on) {
                    A r0[VPL], r1[VPL], r2[VPL], r3[VPL];
                    RowIO<T, VPL>::load(table + (uint64_t)f0 * dpad, lane, r0);
                    RowIO<T, VPL>::load(table + (uint64_t)f1 * dpad, lane, r1);
                    RowIO<T, VPL>::load(table + (uint64_t)f2 * dpad, lane, r2);
                    RowIO<T, VPL>::load(table + (uint64_t)f3 * dpad, lane, r3);
                    fma_row<T, A, VPL>(acc, c0, r0);
                    fma_row<T, A, VPL>(acc, c1, r1);
                    fma_row<T, A, VPL>(acc, c2, r2);
                    fma_row<T, A, VPL>(acc, c3, r3);
                }
            }
            for (; j < m; ++j) {
                const uint32_t f0 = __shfl_sync(FULL, f, j);
                const A c0 = (A)__shfl_sync(FULL, cq, j);
                if (lane_on) {
                    A r0[VPL];
                    RowIO<T, VPL>::load(table + (uint64_t)f0 * dpad, lane, r0);
                    fma_row<T, A, VPL>(acc, c0, r0);
                }
            }
        }
        pos += total;
    }
    return ntot;
}

// gather_role with feature dropout: node by node, the kept positions (the
// keys k_sample counted) in position order, four rows in flight.
template <typename T, typename A, int VPL>
__device__ A gather_role_fd(const ForwardParams& p, const T* __restrict__ table, const uint32_t* nodes, const float* w,
                            uint32_t count, uint32_t slot0, uint32_t v, uint32_t salt, uint32_t src, uint64_t& pos,
                            bool emit, A (&acc)[VPL], int lane, bool lane_on) {
#pragma unroll
    for (int k = 0; k < VPL; ++k) acc[k] = 0;
    A ntot = 0;
    for (uint32_t idx = 0; idx < count; ++idx) {
        const uint32_t u = nodes[idx];
        const uint64_t fs = p.fptr[u];
        const uint32_t nall = (uint32_t)(p.fptr[u + 1] - fs);
        const uint32_t q = slot0 + idx;
        float scal;
        const uint32_t kept = fd_kept(p.fd, v, salt, q, nall, scal);
        const float c = (w ? w[idx] : 1.f) + scal;
        ntot += (A)c * (A)kept;
        const FdNode nd = fd_node(p.fd, v, salt, q, nall, lane);
        for (uint32_t j0 = 0; j0 < nall; j0 += 32) {
            const unsigned m = fd_mask(p.fd, nd, v, salt, q, nall, j0, lane);
            uint32_t f = 0;
            if ((m >> lane) & 1u) {
                f = p.fids[fs + j0 + lane];
                if (emit) {
                    const uint64_t oo = pos + __popc(m & ((1u << lane) - 1u));
                    p.item_f[oo] = f;
                    p.item_src[oo] = src;
                    p.item_c[oo] = c;
                }
            }
            unsigned mm = m;
            while (mm) {
                uint32_t fr[4];
                int nr = 0;
#pragma unroll
                for (int t = 0; t < 4; ++t) {
                    const int b = mm ? __ffs(mm) - 1 : 0;
                    fr[t] = __shfl_sync(FULL, f, b);
                    if (mm) { mm &= mm - 1; nr = t + 1; }
                }
                if (lane_on) {
                    A r4[4][VPL];
#pragma unroll
                    for (int t = 0; t < 4; ++t)
                        if (t < nr) RowIO<T, VPL>::load(table + (uint64_t)fr[t] * p.dpad, lane, r4[t]);
#pragma unroll
                    for (int t = 0; t < 4; ++t)
                        if (t < nr) fma_row<T, A, VPL>(acc, (A)c, r4[t]);
                }
            }
            pos += __popc(m);
        }
    }
    return ntot;
}

// ---------------------------------------------------------------------------
// Staged gather (the common case): per-warp shared-memory tables of the
// anchor's role nodes and of all their feature occurrences, so that the row
// pointers of all roles are loaded in one round, all feature ids in one more,
// and each role's rows are then read eight at a time from the table.
// ---------------------------------------------------------------------------
constexpr uint32_t NODE_CAP = 64;     // 1 + neighbours + negatives
constexpr uint32_t OCC_CAP = 512;     // feature occurrences of one anchor
constexpr uint32_t ROLE_CAP = 34;     // R + 2
constexpr int FWD_WARPS = 8;

struct WarpTables {
    uint32_t node_fs[NODE_CAP];       // first feature index (fptr) of the node
    uint32_t node_n[NODE_CAP];        // feature count of the node (before dropout)
    uint32_t node_incl[NODE_CAP];     // inclusive prefix of feature counts
    float node_c[NODE_CAP];           // count weight of the node's occurrences
    uint32_t role_ob[ROLE_CAP + 1];   // first occurrence of each role
    float role_n[ROLE_CAP];           // sum of count weights of each role
    uint32_t occ_f[OCC_CAP];
    float occ_c[OCC_CAP];
};

__device__ __forceinline__ uint32_t node_role(uint32_t q, uint32_t cnt) {
    return q == 0 ? 0u : (q <= cnt ? 1u : 2u + (q - 1u - cnt));
}

// Phases A and B.  Returns false (warp-uniform) when the anchor does not fit
// the tables; nothing has been emitted then.
template <typename A>
__device__ bool stage_anchor(const ForwardParams& p, WarpTables& W, uint32_t a, uint32_t v, uint32_t cnt,
                             uint64_t pos, bool emit, uint32_t sbase, uint32_t salt, int lane) {
    const uint32_t R = p.R;
    const uint32_t n_nodes = 1 + cnt + R;
    if (n_nodes > NODE_CAP || R + 2 > ROLE_CAP) return false;
    const uint32_t* nb = p.nbr + (uint64_t)a * p.Kcap;
    const float* nw = p.nbr_w + (uint64_t)a * p.Kcap;
    const uint32_t* ng = p.neg + (uint64_t)a * R;
    uint32_t carry = 0;
    float n1 = 0.f;                  // role 1 weight total (lane-partial)
    bool big = false;
    for (uint32_t q0 = 0; q0 < n_nodes; q0 += 32) {
        const uint32_t q = q0 + lane;
        uint32_t fn = 0;
        if (q < n_nodes) {
            uint32_t u;
            float c;
            if (q == 0) { u = v; c = 1.f; }
            else if (q <= cnt) { u = nb[q - 1]; c = nw[q - 1]; }
            else { u = ng[q - 1 - cnt]; c = 1.f; }
            const uint64_t fs = p.fptr[u];
            const uint32_t nall = (uint32_t)(p.fptr[u + 1] - fs);
            float scal;
            fn = fd_kept(p.fd, v, salt, q, nall, scal);
            c += scal;
            big = big || (fs + nall) > 0xffffffffull;
            W.node_fs[q] = (uint32_t)fs;
            W.node_n[q] = nall;
            W.node_c[q] = c;
            const uint32_t r = node_role(q, cnt);
            const float wsum = c * (float)fn;
            if (r == 1) n1 += wsum;
            else W.role_n[r] = wsum;
        }
        const uint32_t incl = warp_incl_scan(fn, lane) + carry;
        if (q < n_nodes) W.node_incl[q] = incl;
        carry = __shfl_sync(FULL, incl, 31);
    }
    if (__any_sync(FULL, big)) return false;
    const uint32_t total = carry;
    if (total > OCC_CAP) return false;
    n1 = warp_sum<float>(n1);
    __syncwarp();
    if (lane == 0) {
        W.role_n[1] = n1;
        W.role_ob[0] = 0;
        W.role_ob[1] = W.node_incl[0];
        W.role_ob[2] = W.node_incl[cnt];
        for (uint32_t i = 1; i <= R; ++i) W.role_ob[2 + i] = W.node_incl[cnt + i];
    }
    if (p.fd.kind != S_ALL) {
        // phase B with feature dropout: node by node, the kept positions in
        // position order (the same keys k_sample counted)
        __syncwarp();
        uint32_t o = 0;
        for (uint32_t q = 0; q < n_nodes; ++q) {
            const uint32_t nall = W.node_n[q], fs = W.node_fs[q];
            const float c = W.node_c[q];
            const uint32_t src = sbase + node_role(q, cnt);
            const FdNode nd = fd_node(p.fd, v, salt, q, nall, lane);
            for (uint32_t j0 = 0; j0 < nall; j0 += 32) {
                const unsigned m = fd_mask(p.fd, nd, v, salt, q, nall, j0, lane);
                if ((m >> lane) & 1u) {
                    const uint32_t oo = o + __popc(m & ((1u << lane) - 1u));
                    const uint32_t f = p.fids[(uint64_t)fs + j0 + lane];
                    W.occ_f[oo] = f;
                    W.occ_c[oo] = c;
                    if (emit) {
                        p.item_f[pos + oo] = f;
                        p.item_src[pos + oo] = src;
                        p.item_c[pos + oo] = c;
                    }
                }
                o += __popc(m);
            }
        }
        __syncwarp();
        return true;
    }
    // phase B: one feature id per lane, four batches of loads in flight
    for (uint32_t o0 = 0; o0 < total; o0 += 128) {
        uint32_t fid[4], q_of[4];
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            const uint32_t o = o0 + b * 32 + lane;
            fid[b] = 0;
            q_of[b] = 0;
            if (o < total) {
                // owner: the first node whose inclusive prefix exceeds o
                uint32_t lo = 0, hi = n_nodes - 1;
                while (lo < hi) {
                    const uint32_t mid = (lo + hi) >> 1;
                    if (W.node_incl[mid] > o) hi = mid; else lo = mid + 1;
                }
                const uint32_t excl = lo ? W.node_incl[lo - 1] : 0u;
                q_of[b] = lo;
                fid[b] = p.fids[(uint64_t)W.node_fs[lo] + (o - excl)];
            }
        }
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            const uint32_t o = o0 + b * 32 + lane;
            if (o < total) {
                const float c = W.node_c[q_of[b]];
                W.occ_f[o] = fid[b];
                W.occ_c[o] = c;
                if (emit) {
                    p.item_f[pos + o] = fid[b];
                    p.item_src[pos + o] = sbase + node_role(q_of[b], cnt);
                    p.item_c[pos + o] = c;
                }
            }
        }
    }
    __syncwarp();
    return true;
}

// Phase C: every role's rows in occurrence order (role-major), U rows in
// flight across role boundaries.  As each role closes, its mean
// sum(c * row) / sum(c) is written to the role's direction row and its weight
// total sum(c) to scale; the loss kernel reads both back.
template <typename T, typename A, int VPL>
__device__ __forceinline__ void roles_from_table(const ForwardParams& p, const T* __restrict__ table,
                                                 const WarpTables& W, uint32_t NR, uint64_t sbase, int lane,
                                                 bool lane_on) {
    using IO = RowIO<T, VPL>;
    constexpr int U = IO::INFLIGHT;
    const uint32_t dpad = p.dpad;
    A* dir = (A*)p.dir;
    A* scale = (A*)p.scale;
    const uint32_t total = W.role_ob[NR];
    A acc[VPL];
#pragma unroll
    for (int k = 0; k < VPL; ++k) acc[k] = 0;
    uint32_t r = 0, rend = W.role_ob[1];
    auto close_role = [&]() {
        const A n = (A)W.role_n[r];
        if (lane_on) {
            const A rn = (A)1 / n;
            A m[VPL];
#pragma unroll
            for (int k = 0; k < VPL; ++k) m[k] = acc[k] * rn;
            store_row<A, VPL, A>(dir + (sbase + r) * dpad, lane, m);
        }
        if (lane == 0) scale[sbase + r] = n;
#pragma unroll
        for (int k = 0; k < VPL; ++k) acc[k] = 0;
        ++r;
        if (r < NR) rend = W.role_ob[r + 1];
    };
    for (uint32_t j = 0; j < total; j += U) {
        typename IO::Raw rows[U];
        if (lane_on) {
#pragma unroll
            for (int u = 0; u < U; ++u)
                if (j + u < total) rows[u] = IO::load_raw(table + (uint64_t)W.occ_f[j + u] * dpad, lane);
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const uint32_t jj = j + u;
            if (jj < total) {
                while (jj >= rend) close_role();
                if (lane_on) IO::template fma<A>(acc, (A)W.occ_c[jj], rows[u]);
            }
        }
    }
    while (r < NR) close_role();
}

template <typename A, int VPL>
__device__ __forceinline__ A warp_dot(const A (&x)[VPL], const A (&y)[VPL]) {
    A s = 0;
#pragma unroll
    for (int k = 0; k < VPL; ++k) s += x[k] * y[k];
    return warp_sum<A>(s);
}

// Two dot products x1.y1 and x2.y2 reduced together (the two shuffle chains
// interleave).
template <typename A, int VPL>
__device__ __forceinline__ void warp_dot2(const A (&x1)[VPL], const A (&y1)[VPL], const A (&x2)[VPL],
                                          const A (&y2)[VPL], A& d1, A& d2) {
    A s = 0, t = 0;
#pragma unroll
    for (int k = 0; k < VPL; ++k) { s += x1[k] * y1[k]; t += x2[k] * y2[k]; }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        s += __shfl_xor_sync(FULL, s, o);
        t += __shfl_xor_sync(FULL, t, o);
    }
    d1 = s;
    d2 = t;
}

template <typename A, int VPL>
__device__ __forceinline__ bool warp_all_finite(const A (&x)[VPL]) {
    bool ok = true;
#pragma unroll
    for (int k = 0; k < VPL; ++k) ok = ok && isfinite(x[k]);
    return __all_sync(FULL, ok);
}

// k_fwd_gather: one warp per anchor; the mean of every role of the anchor
// (h(v), ~h(v), h(u_1..R)) into its direction row, the role's weight total
// into scale, and the anchor's gradient items.  STAGED = true: the common path
// through the per-warp tables; anchors that do not fit are flagged in
// p.deferred and skipped.  STAGED = false: the direct path, run afterwards for
// the flagged anchors only (every anchor when p.deferred is null).  Both
// produce identical items, means and totals.
// The staged gather of anchor a (phases A-C) by one warp; anchors that do not
// fit the tables are flagged for the direct path.
template <typename T, typename A, int VPL>
__device__ __forceinline__ void gather_staged(const ForwardParams& p, WarpTables& W, uint32_t a, int lane) {
    const uint32_t NR = p.R + 2;
    const bool lane_on = (uint32_t)(lane * VPL) < p.dpad;
    const uint32_t v = p.anchors[a];
    const bool emit = p.emit && p.st->n_items > 0;
    const uint64_t pos = emit ? p.occ_off[a] : 0;
    const uint64_t sbase = (uint64_t)a * NR;
    const uint32_t cnt = p.nbr_cnt[a];
    const uint32_t salt = p.eval ? 0xffffffffu : (uint32_t)p.st->step;   // as k_sample
    const bool staged = stage_anchor<A>(p, W, a, v, cnt, pos, emit, (uint32_t)sbase, salt, lane);
    if (lane == 0) p.deferred[a] = staged ? 0 : 1;
    if (staged) roles_from_table<T, A, VPL>(p, (const T*)p.table, W, NR, sbase, lane, lane_on);
    __syncwarp();
}

template <typename T, typename A, int VPL, bool STAGED>
__global__ void __launch_bounds__(256, STAGED ? (VPL <= 8 ? 4 : 3) : 1) k_fwd_gather(ForwardParams p) {
    pdl_wait();
    pdl_trigger();
    const int lane = threadIdx.x & 31;
    const uint32_t n = p.st->n_anchors;
    if constexpr (STAGED) {
        extern __shared__ __align__(16) unsigned char fwd_smem[];
        const uint32_t a = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
        if (a < n) gather_staged<T, A, VPL>(p, reinterpret_cast<WarpTables*>(fwd_smem)[threadIdx.x >> 5], a, lane);
        return;
    }
    const uint32_t a = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (a >= n) return;
    const uint32_t R = p.R, NR = R + 2, dpad = p.dpad;
    const bool lane_on = (uint32_t)(lane * VPL) < dpad;
    const T* __restrict__ table = (const T*)p.table;
    const uint32_t v = p.anchors[a];
    const bool emit = p.emit && p.st->n_items > 0;
    uint64_t pos = emit ? p.occ_off[a] : 0;
    const uint64_t sbase = (uint64_t)a * NR;
    const uint32_t cnt = p.nbr_cnt[a];
    const uint32_t salt = p.eval ? 0xffffffffu : (uint32_t)p.st->step;   // as k_sample
    {
        if (p.deferred && !p.deferred[a]) return;
        A* dir = (A*)p.dir;
        A* scale = (A*)p.scale;
        for (uint32_t r = 0; r < NR; ++r) {
            const uint32_t* nodes = r == 0 ? &v : (r == 1 ? p.nbr + (uint64_t)a * p.Kcap : p.neg + (uint64_t)a * R + (r - 2));
            const float* w = r == 1 ? p.nbr_w + (uint64_t)a * p.Kcap : nullptr;
            const uint32_t count = r == 1 ? cnt : 1u;
            const uint32_t slot0 = r == 0 ? 0u : (r == 1 ? 1u : 1u + cnt + (r - 2));
            A acc[VPL];
            const A nr = p.fd.kind == S_ALL
                             ? gather_role<T, A, VPL>(p, table, nodes, w, count, (uint32_t)(sbase + r), pos, emit, acc,
                                                      lane, lane_on)
                             : gather_role_fd<T, A, VPL>(p, table, nodes, w, count, slot0, v, salt,
                                                         (uint32_t)(sbase + r), pos, emit, acc, lane, lane_on);
            if (lane_on) {
                const A rn = (A)1 / nr;
#pragma unroll
                for (int k = 0; k < VPL; ++k) acc[k] *= rn;
                store_row<A, VPL, A>(dir + (sbase + r) * dpad, lane, acc);
            }
            if (lane == 0) scale[sbase + r] = nr;
        }
    }
}

// k_fwd_gather_queue: the staged gather as a persistent grid (gather_ctas
// CTAs).  Each warp takes the next anchor from the batch's work queue
// (BatchState::fwd_next, zeroed by k_batch_begin) until none is left, so a
// warp that drew short anchors takes more of them and no wave waits on its
// slowest warp.  MINB CTAs per SM (2 or 3, from the grid size) set the
// register budget of the loop (the one-shot kernel is at its 64-register
// limit at 4).
template <typename T, typename A, int VPL, int MINB>
__global__ void __launch_bounds__(256, MINB) k_fwd_gather_queue(ForwardParams p) {
    pdl_wait();
    pdl_trigger();
    extern __shared__ __align__(16) unsigned char fwd_smem[];
    WarpTables& W = reinterpret_cast<WarpTables*>(fwd_smem)[threadIdx.x >> 5];
    const int lane = threadIdx.x & 31;
    const uint32_t n = p.st->n_anchors;
    for (;;) {
        uint32_t a = 0;
        if (lane == 0) a = atomicAdd(&p.st->fwd_next, 1u);
        a = __shfl_sync(FULL, a, 0);
        if (a >= n) break;
        gather_staged<T, A, VPL>(p, W, a, lane);
    }
}

// k_fwd_emit: the gradient items of every anchor (feature id, role src,
// count weight at the anchor's item positions), exactly as the gathers emit
// them, without reading the table: the staged path's tables, or the direct
// path's role walk with no lane reading rows.  In replayed graphs it runs
// ahead of the radix sort on a second stream, so that the sort overlaps the
// gathers, which then run with emission off.
template <typename T, typename A, int VPL>
__global__ void __launch_bounds__(256) k_fwd_emit(ForwardParams p) {
    pdl_wait();
    pdl_trigger();
    const int lane = threadIdx.x & 31;
    const uint32_t a = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t n = p.st->n_anchors;
    if (a >= n || p.st->n_items == 0) return;
    const uint32_t R = p.R, NR = R + 2;
    const uint32_t v = p.anchors[a];
    uint64_t pos = p.occ_off[a];
    const uint64_t sbase = (uint64_t)a * NR;
    const uint32_t cnt = p.nbr_cnt[a];
    const uint32_t salt = p.eval ? 0xffffffffu : (uint32_t)p.st->step;   // as k_sample
    extern __shared__ __align__(16) unsigned char fwd_smem[];
    WarpTables& W = reinterpret_cast<WarpTables*>(fwd_smem)[threadIdx.x >> 5];
    if (stage_anchor<A>(p, W, a, v, cnt, pos, true, (uint32_t)sbase, salt, lane)) return;
    for (uint32_t r = 0; r < NR; ++r) {
        const uint32_t* nodes = r == 0 ? &v : (r == 1 ? p.nbr + (uint64_t)a * p.Kcap : p.neg + (uint64_t)a * R + (r - 2));
        const float* w = r == 1 ? p.nbr_w + (uint64_t)a * p.Kcap : nullptr;
        const uint32_t count = r == 1 ? cnt : 1u;
        const uint32_t slot0 = r == 0 ? 0u : (r == 1 ? 1u : 1u + cnt + (r - 2));
        A acc[VPL];
        if (p.fd.kind == S_ALL)
            gather_role<T, A, VPL>(p, nullptr, nodes, w, count, (uint32_t)(sbase + r), pos, true, acc, lane, false);
        else
            gather_role_fd<T, A, VPL>(p, nullptr, nodes, w, count, slot0, v, salt, (uint32_t)(sbase + r), pos, true, acc,
                                      lane, false);
    }
}

// k_fwd_loss: one warp per anchor; reads the role means and totals written by
// k_fwd_gather, evaluates the loss (loss.rs:56-129) and overwrites each role's
// mean with its gradient direction and its total with its gradient scale.
template <typename T, typename A, int VPL>
__global__ void __launch_bounds__(128) k_fwd_loss(ForwardParams p) {
    using D = typename DirOf<T, A>::type;
    pdl_wait();
    pdl_trigger();
    const int lane = threadIdx.x & 31;
    const uint32_t a = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t n = p.st->n_anchors;
    if (a >= n) return;
    const uint32_t R = p.R, NR = R + 2, dpad = p.dpad;
    const bool lane_on = (uint32_t)(lane * VPL) < dpad;
    A* dir = (A*)p.dir;
    D* dout = std::is_same<D, A>::value ? (D*)p.dir : (D*)p.dir16;
    A* scale = (A*)p.scale;
    const uint32_t v = p.anchors[a];
    const uint64_t sbase = (uint64_t)a * NR;
    auto load_mean = [&](uint64_t src, A (&x)[VPL]) {
        if (lane_on) RowIO<A, VPL>::load_cg(dir + src * dpad, lane, x);
        else {
#pragma unroll
            for (int k = 0; k < VPL; ++k) x[k] = 0;
        }
    };
    // Once the anchor's role means are read and its directions written
    // elsewhere (BF16 directions), nothing reads the means again: their L2
    // lines are dropped without a write-back (discard.global.L2), which keeps
    // L2 for the directions the reducer reads next.  Only whole 128-byte
    // lines of this anchor's rows are dropped.
    auto drop_means = [&]() {
        if constexpr (!std::is_same<D, A>::value) {
            const uint64_t rb = (uint64_t)dpad * sizeof(A);
            if (p.means_dead && (rb & 127u) == 0) {
                __syncwarp();
                const char* base = reinterpret_cast<const char*>(dir + sbase * dpad);
                const uint32_t lines = (uint32_t)(NR * rb / 128u);
                for (uint32_t l = lane; l < lines; l += 32)
                    asm volatile("discard.global.L2 [%0], 128;" ::"l"(base + (uint64_t)l * 128u) : "memory");
            }
        }
    };

    A hv[VPL], tv[VPL], u[VPL], un[VPL];
    load_mean(sbase, hv);
    load_mean(sbase + 1, tv);
    if (R) load_mean(sbase + 2, un);
    // role weight totals: lane i holds role i's (roles beyond 32 read directly)
    const A n_lane = (uint32_t)lane < NR ? scale[sbase + lane] : (A)0;
    const A n_h = __shfl_sync(FULL, n_lane, 0), n_t = __shfl_sync(FULL, n_lane, 1);

    // loss weighting divisor (mod.rs:190-200)
    A wdiv = 1;
    if (p.loss_weighting != LW_NONE) {
        const A deg = (A)(p.row_ptr[v + 1] - p.row_ptr[v]);
        wdiv = p.loss_weighting == LW_LOG ? (A)log((double)(1 + deg)) : (A)pow((double)deg, (double)p.lw_exp);
    }
    A up = 1;
    if (p.dloss) up = p.dloss_f64 ? (A)((const double*)p.dloss)[a] : (A)p.dloss[a];

    if (p.loss == LOSS_RANK || p.loss == LOSS_RANKSPACE) {
        // RankLoss (loss.rs:130-155): logits u_i.h and h.t, p = softmax(.)[h.t];
        // p < tau gives -ln p.  RankSpace (loss.rs:75-79) adds StarSpace with
        // gamma = tau.  Exact exponentials throughout (the reference's
        // approximate exp is its own fallback-checked shortcut).
        // d(-ln p)/d logit_j = softmax_j - [j is h.t]: dL/du_i = s_i h,
        // dL/dt = (p - 1) h, dL/dh = sum_i s_i u_i + (p - 1) t.
        const bool ss = p.loss == LOSS_RANKSPACE;
        const A tau = (A)p.gamma;
        A xa[VPL], xh[VPL];            // StarSpace: normalised t and h
        A nt = 1, nh = 1, rd = 0;
        if (ss) {
            A tt_, hh_;
            warp_dot2<A, VPL>(tv, tv, hv, hv, tt_, hh_);
            nt = sqrt(tt_);
            nh = sqrt(hh_);
            const A rnt = (A)1 / nt, rnh = (A)1 / nh;
#pragma unroll
            for (int k = 0; k < VPL; ++k) { xa[k] = tv[k] * rnt; xh[k] = hv[k] * rnh; }
            rd = warp_dot<A, VPL>(xa, xh);
        }
        const A lpos = warp_dot<A, VPL>(hv, tv);
        // pass 1: running max / sum of the exponentials, StarSpace margins
        A M = lpos, Z = 1, lsum = 0;
        uint32_t P = 0;
        auto logits = [&](const A (&uu_)[VPL], A& lg, A& cs, A& nu) {
            A uu = 0, hx = 0;
            if (ss) warp_dot2<A, VPL>(uu_, uu_, xh, uu_, uu, hx);
            lg = warp_dot<A, VPL>(uu_, hv);
            nu = sqrt(uu);
            cs = hx / nu;
        };
        for (uint32_t i = 0; i < R; ++i) {
            load_mean(sbase + 2 + i, u);
            A lg, cs, nu;
            logits(u, lg, cs, nu);
            if (lg > M) { Z = Z * exp(M - lg) + (A)1; M = lg; }
            else Z += exp(lg - M);
            if (ss) {
                const A li = tau - (rd - cs);
                if (li > 0) { ++P; lsum += li; }
            }
        }
        const A pp = exp(lpos - M) / Z;
        const bool rk = pp < tau;                 // rank term present
        const bool under = rk && !(pp > 0);       // -ln 0: simple_grad's gradients are NaN
        A L = (P ? lsum / (A)P : (A)0) + (rk ? -log(pp) : (A)0);
        L = L / wdiv;
        const bool is_nan = L != L;
        const bool ok = !is_nan && L > 0;
        const A inv = P ? (A)1 / (A)P : (A)0;
        // pass 2: every negative's gradient; sums for h
        A gs[VPL], gr[VPL];            // sum of kept normalised u (StarSpace), sum s_i u_i (rank)
#pragma unroll
        for (int k = 0; k < VPL; ++k) { gs[k] = 0; gr[k] = 0; }
        for (uint32_t i = 0; i < R; ++i) {
            const uint64_t src = sbase + 2 + i;
            load_mean(src, u);
            A lg, cs, nu;
            logits(u, lg, cs, nu);
            const A si = exp(lg - M) / Z;
            const bool kept = ss && tau - (rd - cs) > 0;
            const A rnu = (A)1 / nu;
            A d[VPL];
#pragma unroll
            for (int k = 0; k < VPL; ++k) {
                d[k] = rk ? si * hv[k] : (A)0;
                if (rk) gr[k] += si * u[k];
                if (kept) {
                    const A un_k = u[k] * rnu;
                    gs[k] += un_k;
                    d[k] += (xh[k] - un_k * cs) * rnu * inv;
                }
            }
            const bool fin = warp_all_finite<A, VPL>(d);
            const bool em = ok && (rk || kept) && fin && !under;
            if (em && lane_on) store_row<D, VPL, A>(dout + src * dpad, lane, d);
            __syncwarp();
            if (lane == 0) {
                const A n_u = scale[src];
                p.valid[src] = (uint8_t)em;
                scale[src] = em ? up / (n_u * wdiv) : (A)0;
            }
        }
        A dh[VPL], dt[VPL];
#pragma unroll
        for (int k = 0; k < VPL; ++k) {
            dh[k] = rk ? gr[k] + (pp - (A)1) * tv[k] : (A)0;
            dt[k] = rk ? (pp - (A)1) * hv[k] : (A)0;
        }
        if (P) {
            A gtn[VPL], ghn[VPL];
#pragma unroll
            for (int k = 0; k < VPL; ++k) {
                gtn[k] = -xh[k];                       // P terms, each -h^, times 1/P
                ghn[k] = (gs[k] - xa[k] * (A)P) * inv;
            }
            A st_, sh_;
            warp_dot2<A, VPL>(xa, gtn, xh, ghn, st_, sh_);
            const A rnt = (A)1 / nt, rnh = (A)1 / nh;
#pragma unroll
            for (int k = 0; k < VPL; ++k) {
                dt[k] += (gtn[k] - xa[k] * st_) * rnt;
                dh[k] += (ghn[k] - xh[k] * sh_) * rnh;
            }
        }
        const bool reach = rk || P;
        const bool fin_h = warp_all_finite<A, VPL>(dh);
        const bool fin_t = warp_all_finite<A, VPL>(dt);
        if (lane_on) {
            store_row<D, VPL, A>(dout + sbase * dpad, lane, dh);
            store_row<D, VPL, A>(dout + (sbase + 1) * dpad, lane, dt);
        }
        if (lane == 0) {
            p.valid[sbase] = (uint8_t)(ok && reach && fin_h && !under);
            p.valid[sbase + 1] = (uint8_t)(ok && reach && fin_t && !under);
            scale[sbase] = up / (n_h * wdiv);
            scale[sbase + 1] = up / (n_t * wdiv);
            if (p.loss_out) ((A*)p.loss_out)[a] = L;
            p.status[a] = is_nan ? 2 : (ok ? 0 : 1);
        }
        drop_means();
        return;
    }

    A gsum[VPL];
#pragma unroll
    for (int k = 0; k < VPL; ++k) gsum[k] = 0;
    A lsum = 0;
    uint32_t P = 0;

    A na = 0, d1 = 0, nt = 0, nh = 0, rd = 0;
    A xa[VPL];  // margin: t - h; cosine losses: normalised t
    A xh[VPL];  // cosine losses: normalised h
    if (p.loss == LOSS_MARGIN) {
#pragma unroll
        for (int k = 0; k < VPL; ++k) xa[k] = tv[k] - hv[k];
        na = sqrt(warp_dot<A, VPL>(xa, xa));
        d1 = (A)p.gamma + na;
    } else {
        A tt_, hh_;
        warp_dot2<A, VPL>(tv, tv, hv, hv, tt_, hh_);
        nt = sqrt(tt_);
        nh = sqrt(hh_);
        const A rnt = (A)1 / nt, rnh = (A)1 / nh;
#pragma unroll
        for (int k = 0; k < VPL; ++k) { xa[k] = tv[k] * rnt; xh[k] = hv[k] * rnh; }
        rd = warp_dot<A, VPL>(xa, xh);
    }

    for (uint32_t i = 0; i < R; ++i) {
        const uint64_t src = sbase + 2 + i;
#pragma unroll
        for (int k = 0; k < VPL; ++k) u[k] = un[k];
        if (i + 1 < R) load_mean(src + 1, un);      // next negative's mean in flight
        const A n_u = 2 + i < 32 ? __shfl_sync(FULL, n_lane, 2 + i) : scale[src];
        A d[VPL];
        bool kept;
        if (p.loss == LOSS_MARGIN) {
#pragma unroll
            for (int k = 0; k < VPL; ++k) d[k] = tv[k] - u[k];
            const A nb = sqrt(warp_dot<A, VPL>(d, d));
            const A li = d1 - nb;
            kept = li > 0;
            if (kept) {
                ++P;
                lsum += li;
                const A rnb = (A)1 / nb;
#pragma unroll
                for (int k = 0; k < VPL; ++k) { d[k] = d[k] * rnb; gsum[k] += d[k]; }
            }
        } else {
            // |u|^2 and h.u in one reduction: cos(h, u) = (h.u / |u|) / |h|
            A uu, hu;
            warp_dot2<A, VPL>(u, u, xh, u, uu, hu);
            const A nu = sqrt(uu);
            const A rnu = (A)1 / nu;
#pragma unroll
            for (int k = 0; k < VPL; ++k) u[k] *= rnu;
            const A cs = hu * rnu;
            const A li = p.loss == LOSS_STARSPACE ? (A)p.gamma - (rd - cs) : cs - (A)p.neg_margin;
            kept = li > 0;
            if (kept) {
                ++P;
                lsum += li;
#pragma unroll
                for (int k = 0; k < VPL; ++k) { gsum[k] += u[k]; d[k] = (xh[k] - u[k] * cs) * rnu; }
            }
        }
        bool fin = kept ? warp_all_finite<A, VPL>(d) : false;
        if (kept && lane_on) store_row<D, VPL, A>(dout + src * dpad, lane, d);
        __syncwarp();
        if (lane == 0) {
            p.valid[src] = (uint8_t)(kept && fin);
            scale[src] = kept ? (A)1 / n_u : (A)0;   // finalised below
        }
    }

    // --- loss value and role-0/1 directions ---
    uint32_t n_terms = P;
    int pos_kept = 0;
    if (p.loss == LOSS_CONTRASTIVE) {
        const A pos_l = (A)p.gamma - rd;
        if (pos_l > 0) { pos_kept = 1; ++n_terms; lsum += pos_l; }
    }
    A L = n_terms ? lsum / (A)n_terms : (A)0;
    L = L / wdiv;
    const bool is_nan = L != L;
    const bool ok = !is_nan && L > 0;
    const A inv = n_terms ? (A)1 / (A)n_terms : (A)0;

    A dh[VPL], dt[VPL];
    bool reach_t = true;
    if (p.loss == LOSS_MARGIN) {
        const A invP = P ? (A)1 / (A)P : (A)0;
        const A rna = (A)1 / na;
#pragma unroll
        for (int k = 0; k < VPL; ++k) {
            const A ak = xa[k] * rna;   // NaN when t == h, dropped by the extraction rule
            dh[k] = -ak;
            dt[k] = ak - gsum[k] * invP;
        }
    } else {
        const A cnt_t = p.loss == LOSS_STARSPACE ? (A)P : (A)pos_kept;
        reach_t = p.loss == LOSS_STARSPACE ? true : pos_kept != 0;
        A gtn[VPL], ghn[VPL];
#pragma unroll
        for (int k = 0; k < VPL; ++k) {
            gtn[k] = -xh[k] * cnt_t * inv;
            ghn[k] = (gsum[k] - xa[k] * cnt_t) * inv;
        }
        A st_, sh_;
        warp_dot2<A, VPL>(xa, gtn, xh, ghn, st_, sh_);
        const A rnt = (A)1 / nt, rnh = (A)1 / nh;
#pragma unroll
        for (int k = 0; k < VPL; ++k) {
            dt[k] = (gtn[k] - xa[k] * st_) * rnt;
            dh[k] = (ghn[k] - xh[k] * sh_) * rnh;
        }
    }
    const bool fin_h = warp_all_finite<A, VPL>(dh);
    const bool fin_t = warp_all_finite<A, VPL>(dt);
    if (lane_on) {
        store_row<D, VPL, A>(dout + sbase * dpad, lane, dh);
        store_row<D, VPL, A>(dout + (sbase + 1) * dpad, lane, dt);
    }
    if (lane == 0) {
        p.valid[sbase] = (uint8_t)(ok && fin_h);
        p.valid[sbase + 1] = (uint8_t)(ok && reach_t && fin_t);
        scale[sbase] = up / (n_h * wdiv);
        scale[sbase + 1] = up / (n_t * wdiv);
        if (p.loss_out) ((A*)p.loss_out)[a] = L;
        p.status[a] = is_nan ? 2 : (ok ? 0 : 1);
    }
    // negatives: scale = upstream * (1/terms) / (n_u * wdiv); clear when the anchor is dropped
    __syncwarp();
    const A neg_f = p.loss == LOSS_MARGIN ? (P ? (A)1 / (A)P : (A)0) : inv;
    for (uint32_t i = lane; i < R; i += 32) {
        const uint64_t src = sbase + 2 + i;
        if (!ok) p.valid[src] = 0;
        scale[src] = scale[src] * up * neg_f / wdiv;
    }
    drop_means();
}

// ---------------------------------------------------------------------------
// k_batch_end: deterministic per-batch loss sums and counters (one CTA).
// ---------------------------------------------------------------------------
template <typename A>
__global__ void __launch_bounds__(1024) k_batch_end(BatchState* st, const A* loss, const int32_t* status,
                                                    const uint32_t* nbr_cnt, uint32_t steps_per_pass, int eval) {
    pdl_wait();
    pdl_trigger();
    __shared__ double s_sum[32];
    __shared__ unsigned long long s_cnt[32], s_nan[32], s_smp[32];
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const uint32_t n = st->n_anchors;
    double sum = 0;
    unsigned long long cnt = 0, nan = 0, smp = 0;
    // eight anchors per thread, all loads issued before the sums
    constexpr int PT = 8;
    for (uint32_t base = 0; base < n; base += 1024 * PT) {
        int sv[PT];
        A lv[PT];
        uint32_t cv[PT];
#pragma unroll
        for (int k = 0; k < PT; ++k) {
            const uint32_t i = base + (uint32_t)k * 1024 + tid;
            const bool in = i < n;
            sv[k] = in ? status[i] : 3;
            lv[k] = in ? loss[i] : (A)0;
            cv[k] = in ? nbr_cnt[i] : 0u;
        }
#pragma unroll
        for (int k = 0; k < PT; ++k) {
            if (sv[k] == 3) continue;
            const double l = (double)lv[k];
            if (eval) sum += l;
            else if (sv[k] == 0) { sum += l; ++cnt; }
            nan += (sv[k] == 2);
            smp += cv[k];
        }
    }
    sum = warp_sum<double>(sum);
    cnt = warp_sum<unsigned long long>(cnt);
    nan = warp_sum<unsigned long long>(nan);
    smp = warp_sum<unsigned long long>(smp);
    if (lane == 0) { s_sum[w] = sum; s_cnt[w] = cnt; s_nan[w] = nan; s_smp[w] = smp; }
    __syncthreads();
    if (tid == 0) {
        double ts = 0;
        unsigned long long tc = 0, tn = 0, tsm = 0;
        for (int i = 0; i < 32; ++i) { ts += s_sum[i]; tc += s_cnt[i]; tn += s_nan[i]; tsm += s_smp[i]; }
        if (eval) {
            st->valid_sum += ts;
            st->batch += 1;
            return;
        }
        float be = (tc > 0 && n > 0) ? (float)(ts / (double)n) : 0.f;
        if (isinf(be)) be = 0.f;
        st->batch_err = be;
        st->batch_kept = (uint32_t)tc;
        st->pass_err_sum += be;
        st->pass_batches += 1;
        st->anchors += n;
        st->kept += tc;
        st->nan_anchors += tn;
        st->sampled += tsm;
        st->items += st->n_items;
        st->step += 1;
        st->batch += 1;
        if (st->batch >= steps_per_pass) { st->batch = 0; st->pass += 1; }
    }
}

// ---------------------------------------------------------------------------
// Table initialisation (mod.rs:381-392): U(-1, 1) rows, L2-normalised.  One
// warp per row; Philox draws keyed by (row, element).
// ---------------------------------------------------------------------------
template <typename T>
__global__ void k_init_table(T* table, uint64_t n_feat, uint32_t dims, uint32_t dpad, uint64_t seed) {
    const int lane = threadIdx.x & 31;
    const uint64_t row = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (row >= n_feat) return;
    float ss = 0.f;
    for (uint32_t k = lane; k < dims; k += 32) {
        float x = 2.f * unit_f32(rand_u32(seed, (uint32_t)row, (uint32_t)(row >> 32), ST_INIT, k)) - 1.f;
        ss += x * x;
    }
    ss = warp_sum<float>(ss);
    const float nrm = sqrtf(ss);
    for (uint32_t k = lane; k < dpad; k += 32) {
        float x = 0.f;
        if (k < dims) x = (2.f * unit_f32(rand_u32(seed, (uint32_t)row, (uint32_t)(row >> 32), ST_INIT, k)) - 1.f) / nrm;
        if constexpr (sizeof(T) == 2) table[row * dpad + k] = __float2bfloat16_rn(x);
        else table[row * dpad + k] = (T)x;
    }
}

// Dense FP32 [n_feat x dims] <-> device layout [n_feat x dpad] of type T.
template <typename T>
__global__ void k_convert(T* dev, float* host_layout, uint64_t n_feat, uint32_t dims, uint32_t dpad, int to_dev) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_feat * dpad) return;
    const uint64_t r = i / dpad;
    const uint32_t k = (uint32_t)(i % dpad);
    if (to_dev) {
        float x = k < dims ? host_layout[r * dims + k] : 0.f;
        if constexpr (sizeof(T) == 2) dev[i] = __float2bfloat16_rn(x);
        else dev[i] = (T)x;
    } else if (k < dims) {
        if constexpr (sizeof(T) == 2) host_layout[r * dims + k] = __bfloat162float(dev[i]);
        else host_layout[r * dims + k] = (float)dev[i];
    }
}

// Device layout [n_feat x dpad] of type T -> dense FP32 [n_feat x dims], four
// elements per thread (dims and dpad multiples of 4), written straight into
// page-locked host memory through its device address: the download needs no
// device staging buffer and no separate copy.
template <typename T>
__global__ void k_table_out4(const T* __restrict__ dev, float4* __restrict__ out, uint64_t n_feat, uint32_t dims,
                             uint32_t dpad) {
    const uint32_t q = dims / 4;
    const uint64_t n = n_feat * q;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t r = i / q;
        const uint32_t k = (uint32_t)(i - r * q) * 4u;
        const T* src = dev + r * dpad + k;
        float4 o;
        if constexpr (sizeof(T) == 2) {
            const uint2 w = *reinterpret_cast<const uint2*>(src);
            o = make_float4(__uint_as_float(w.x << 16), __uint_as_float(w.x & 0xffff0000u), __uint_as_float(w.y << 16),
                            __uint_as_float(w.y & 0xffff0000u));
        } else if constexpr (sizeof(T) == 4) {
            o = *reinterpret_cast<const float4*>(src);
        } else {
            o = make_float4((float)src[0], (float)src[1], (float)src[2], (float)src[3]);
        }
        out[i] = o;
    }
}

// ---------------------------------------------------------------------------
// Set-up kernels.
// k_node_bound: an upper bound on the items one anchor can emit:
//   F(v) + R * maxF + (positive part): the exact sum of the neighbours'
//   feature counts when all of them can be taken (All / Prob), else
//   min(K, deg) * (largest neighbour feature count); R * maxF for PPR walks.
// k_split: train / validation ids as the first n_train / remaining positions
//   of a seeded permutation of all nodes (mod.rs:118-122).
// ---------------------------------------------------------------------------
__global__ void k_node_bound(const uint64_t* row_ptr, const uint32_t* cols, const uint64_t* fptr, uint32_t n,
                             int nodes_kind, uint32_t K, uint32_t R, uint32_t max_feat, int ppr, uint32_t* bound) {
    const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n) return;
    const uint64_t rs = row_ptr[v], re = row_ptr[v + 1];
    const uint64_t deg = re - rs;
    uint64_t nb = 0;
    if (ppr) {
        nb = (uint64_t)R * max_feat;          // R walk end nodes
    } else if (nodes_kind == S_FIXED && deg > K) {
        uint64_t mx = 0;
        for (uint64_t j = rs; j < re; ++j) { const uint32_t u = cols[j]; mx = max(mx, fptr[u + 1] - fptr[u]); }
        nb = (uint64_t)K * mx;
    } else {
        for (uint64_t j = rs; j < re; ++j) { const uint32_t u = cols[j]; nb += fptr[u + 1] - fptr[u]; }
    }
    const uint64_t b = (fptr[v + 1] - fptr[v]) + (uint64_t)R * max_feat + nb;
    bound[v] = (uint32_t)min(b, (uint64_t)0xffffffffu);
}

__global__ void k_split(uint32_t* train, uint32_t n_train, uint32_t* valid, uint32_t n, uint64_t seed,
                        uint32_t half, uint32_t* err) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t k[4];
    const u32x4 kk = philox(u32x4{0u, 0x51ed270bu, 0x2545f491u, 0x9e3779b9u}, seed);
    k[0] = kk.x; k[1] = kk.y; k[2] = kk.z; k[3] = kk.w;
    const uint32_t node = permute(i, n, half, k, err);
    if (i < n_train) train[i] = node;
    else valid[i - n_train] = node;
}

void launch_node_bound(const uint64_t* row_ptr, const uint32_t* cols, const uint64_t* fptr, uint32_t n,
                       int nodes_kind, uint32_t K, uint32_t R, uint32_t max_feat, int ppr, uint32_t* bound,
                       cudaStream_t s) {
    k_node_bound<<<(n + 255) / 256, 256, 0, s>>>(row_ptr, cols, fptr, n, nodes_kind, K, R, max_feat, ppr, bound);
}

void launch_split(uint32_t* train, uint32_t n_train, uint32_t* valid, uint32_t n, uint64_t seed, uint32_t half,
                  uint32_t* err, cudaStream_t s) {
    k_split<<<(n + 255) / 256, 256, 0, s>>>(train, n_train, valid, n, seed, half, err);
}

// ---------------------------------------------------------------------------
// Launchers
// ---------------------------------------------------------------------------
void launch_batch_begin(BatchState* st, uint32_t n_order, uint32_t cap, uint32_t steps_per_pass,
                        uint64_t total, uint64_t warmup, float alpha, int injected, float noise, float noise_decay,
                        cudaStream_t s) {
    (void)steps_per_pass;
    launch_chain(k_batch_begin, 1, 32, 0, s, st, n_order, cap, total, warmup, alpha, injected, noise, noise_decay);
}

void launch_sample(const SampleParams& p, cudaStream_t s) {
    // warp per anchor in CTAs of sample_warps warps (1-8; 0 = 8)
    const uint32_t w = p.sample_warps >= 1 && p.sample_warps <= 8 ? p.sample_warps : 8;
    const uint32_t blocks = (p.batch_cap + w - 1) / w;
    launch_chain(k_sample, blocks, 32 * w, 0, s, p);
}

void launch_scan_occ(BatchState* st, uint32_t* occ, uint32_t cap, uint64_t items_cap, cudaStream_t s) {
    (void)cap;
    launch_chain(k_scan_occ, 1, 1024, 0, s, st, occ, items_cap);
}

template <typename T, typename A, int VPL>
static void fwd_launch(const ForwardParams& p, uint32_t cap, cudaStream_t s, int part) {
    const uint32_t blocks = (cap + FWD_WARPS - 1) / FWD_WARPS;
    const size_t smem = sizeof(WarpTables) * FWD_WARPS;
    static bool attr = false;   // opt in to > 48 KB of dynamic shared memory once
    if (!attr) {
        cudaFuncSetAttribute(k_fwd_gather<T, A, VPL, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        cudaFuncSetAttribute(k_fwd_gather_queue<T, A, VPL, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        cudaFuncSetAttribute(k_fwd_gather_queue<T, A, VPL, 3>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        attr = true;
    }
    // the one-warp-per-anchor kernels in CTAs of gather_warps warps (1-8):
    // smaller CTAs free their slots sooner when anchors differ in work
    const uint32_t gw = p.gather_warps >= 1 && p.gather_warps <= (uint32_t)FWD_WARPS ? p.gather_warps : FWD_WARPS;
    const uint32_t gblocks = (cap + gw - 1) / gw;
    const size_t gsmem = sizeof(WarpTables) * gw;
    if (part == FWD_EMIT) {
        launch_chain(k_fwd_emit<T, A, VPL>, gblocks, 32 * gw, gsmem, s, p);
        return;
    }
    if (part != FWD_LOSS) {
        if (p.gather_ctas > 2 * 152)
            launch_chain(k_fwd_gather_queue<T, A, VPL, 3>, std::min(p.gather_ctas, blocks), 32 * FWD_WARPS, smem, s, p);
        else if (p.gather_ctas)
            launch_chain(k_fwd_gather_queue<T, A, VPL, 2>, std::min(p.gather_ctas, blocks), 32 * FWD_WARPS, smem, s, p);
        else
            launch_chain(k_fwd_gather<T, A, VPL, true>, gblocks, 32 * gw, gsmem, s, p);
        launch_chain(k_fwd_gather<T, A, VPL, false>, blocks, 32 * FWD_WARPS, 0, s, p);
    }
    if (part != FWD_GATHER) launch_chain(k_fwd_loss<T, A, VPL>, (cap + 3) / 4, 128, 0, s, p);
}

template <typename T, typename A>
static void fwd_dispatch(int vpl, const ForwardParams& p, uint32_t cap, cudaStream_t s, int part) {
    switch (vpl) {
        case 1: fwd_launch<T, A, 1>(p, cap, s, part); break;
        case 2: fwd_launch<T, A, 2>(p, cap, s, part); break;
        case 4: fwd_launch<T, A, 4>(p, cap, s, part); break;
        case 8: fwd_launch<T, A, 8>(p, cap, s, part); break;
        default: fwd_launch<T, A, 16>(p, cap, s, part); break;
    }
}

void launch_forward(int tt, int vpl, const ForwardParams& p, uint32_t cap, cudaStream_t s, int part) {
    if (tt == TT_F32) fwd_dispatch<float, float>(vpl, p, cap, s, part);
    else if (tt == TT_BF16) fwd_dispatch<__nv_bfloat16, float>(vpl, p, cap, s, part);
    else fwd_dispatch<double, double>(vpl, p, cap, s, part);
}

void launch_batch_end(BatchState* st, const void* loss, const int32_t* status, const uint32_t* nbr_cnt,
                      uint32_t cap, uint32_t steps_per_pass, int eval, int loss_f64, cudaStream_t s) {
    (void)cap;
    if (loss_f64) launch_chain(k_batch_end<double>, 1, 1024, 0, s, st, (const double*)loss, status, nbr_cnt, steps_per_pass, eval);
    else launch_chain(k_batch_end<float>, 1, 1024, 0, s, st, (const float*)loss, status, nbr_cnt, steps_per_pass, eval);
}

void launch_init_table(int tt, void* table, uint64_t n_feat, uint32_t dims, uint32_t dpad, uint64_t seed,
                       cudaStream_t s) {
    const uint64_t blocks = (n_feat * 32 + 255) / 256;
    if (tt == TT_F32) k_init_table<float><<<(unsigned)blocks, 256, 0, s>>>((float*)table, n_feat, dims, dpad, seed);
    else if (tt == TT_BF16)
        k_init_table<__nv_bfloat16><<<(unsigned)blocks, 256, 0, s>>>((__nv_bfloat16*)table, n_feat, dims, dpad, seed);
    else k_init_table<double><<<(unsigned)blocks, 256, 0, s>>>((double*)table, n_feat, dims, dpad, seed);
}

bool launch_table_out(int tt, const void* table, float* out_dev, uint64_t n_feat, uint32_t dims, uint32_t dpad,
                      cudaStream_t s) {
    if ((dims & 3u) || (dpad & 3u) || (reinterpret_cast<uintptr_t>(out_dev) & 15u)) return false;
    if (!n_feat || !dims) return true;
    const unsigned blocks = 152 * 16;
    if (tt == TT_F32) k_table_out4<float><<<blocks, 256, 0, s>>>((const float*)table, (float4*)out_dev, n_feat, dims, dpad);
    else if (tt == TT_BF16)
        k_table_out4<__nv_bfloat16><<<blocks, 256, 0, s>>>((const __nv_bfloat16*)table, (float4*)out_dev, n_feat, dims, dpad);
    else k_table_out4<double><<<blocks, 256, 0, s>>>((const double*)table, (float4*)out_dev, n_feat, dims, dpad);
    return true;
}

void launch_convert_table(int tt, void* dst, const float* src, uint64_t n_feat, uint32_t dims, uint32_t dpad,
                          int to_dev, cudaStream_t s) {
    const uint64_t n = n_feat * dpad;
    const unsigned blocks = (unsigned)((n + 255) / 256);
    if (!n) return;
    float* hl = const_cast<float*>(src);
    if (tt == TT_F32) k_convert<float><<<blocks, 256, 0, s>>>((float*)dst, hl, n_feat, dims, dpad, to_dev);
    else if (tt == TT_BF16) k_convert<__nv_bfloat16><<<blocks, 256, 0, s>>>((__nv_bfloat16*)dst, hl, n_feat, dims, dpad, to_dev);
    else k_convert<double><<<blocks, 256, 0, s>>>((double*)dst, hl, n_feat, dims, dpad, to_dev);
}

}  // namespace ep
