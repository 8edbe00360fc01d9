// ep_red.cu -- deterministic per-feature gradient reduction, fused with Adam.
//
// Input: items sorted stably by feature id (ep_sort.cu), so the items of one
// feature are contiguous and ordered by (anchor, role).  For feature f the
// batch gradient is
//     G[f] = sum over kept items i of c_i * scale[src_i] * dir[src_i]
// where src = anchor * NR + role, c_i is the occurrence's count weight,
// scale folds 1/n_role, the loss-term normaliser, loss weighting and any
// upstream gradient, and dir is the role's gradient direction.
//
// Kept items (src/algos/ep/mod.rs:361-378): in REFERENCE mode, within one
// (feature, anchor) group only the items of the first role whose gradient is
// present and finite are kept ("first occurrence wins"); in TRUE mode every
// item of a valid role is kept.
//
// Work split: the sorted range is cut into fixed-size chunks, one warp per
// chunk, walking its items in order (so no atomics on gradient rows).  A
// feature entirely inside a chunk is finished in place: Adam on the row
// (optimizer.rs:43-81) or a dense gradient row.  A feature spanning chunks
// leaves partial sums (carries); k_fixup adds them in a fixed order and
// finishes the row, so results are bit-reproducible.  A feature none of whose
// items is kept is not in the batch's gradient map and is left untouched
// (no Adam step), as in mod.rs:223-233.
#include <cuda_runtime.h>
#include <algorithm>
#include <mutex>
#include <type_traits>

#include "ep_device.cuh"
#include "ep_internal.h"
#include "ep_launch.cuh"
#include "ep_gb300.h"

namespace ep {

constexpr uint32_t NONE = 0xffffffffu;
// Chunk flags: HEAD = the chunk's first feature started in an earlier chunk
// (its partial sum is in carry_head); THROUGH = that feature also continues
// past the chunk; OWNER = the chunk's last feature starts here and continues
// (partial in carry_tail); *_KEPT = the partial contains at least one kept item.
enum : uint32_t { CF_HEAD = 1u, CF_THROUGH = 2u, CF_OWNER = 4u, CF_HEAD_KEPT = 8u, CF_TAIL_KEPT = 16u };
constexpr int RED_THREADS = 256;
constexpr int FIX_THREADS = 128;
constexpr uint32_t RED_MAX_CTAS = 152 * 8;

uint32_t reduce_chunks(uint64_t cap, uint32_t chunk) { return (uint32_t)((cap + chunk - 1) / chunk); }

// Per-batch Adam constants, read once per kernel from the batch state.
struct AdamStep {
    float lr, rb1, rb2, sigma;    // learning rate, 1/(1 - beta^t), gradient-noise scale
    uint32_t step;
    static __device__ __forceinline__ AdamStep load(const BatchState* st) {
        AdamStep a;
        a.lr = st->lr;
        a.rb1 = 1.f / st->bc1;
        a.rb2 = 1.f / st->bc2;
        a.sigma = st->noise_sigma;
        a.step = st->step_cur;
        return a;
    }
    // the copy k_reduce made (kernels that run after it)
    static __device__ __forceinline__ AdamStep load_fx(const BatchState* st) {
        AdamStep a;
        a.lr = st->fx_lr;
        a.rb1 = 1.f / st->fx_bc1;
        a.rb2 = 1.f / st->fx_bc2;
        a.sigma = st->fx_sigma;
        a.step = st->fx_step;
        return a;
    }
};

// Square root of Adam's second-moment estimate on the SFU (PTX sqrt.approx:
// relative error within a few units of 2^-23); the denominator sqrt(v) + eps
// tolerates that, as it tolerates the fast divide.  Both flush subnormal
// inputs to zero (.ftz): a subnormal second moment (below 1.2e-38) then gives
// the denominator eps, as its square root (below 1.1e-19) added to eps would.
__device__ __forceinline__ float sqrt_sfu(float x) {
    float y;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float div_sfu(float x, float y) {
    float q;
    asm("div.approx.ftz.f32 %0, %1, %2;" : "=f"(q) : "f"(x), "f"(y));
    return q;
}

// Adam on one row (optimizer.rs:43-81): t = pass + 1, beta1 0.9, beta2 0.999,
// eps 1e-8; rows containing NaN are skipped (optimizer.rs:56).  adam_apply
// takes the row's loaded moments and weights (mm, vv, ee) and stores the
// updated row.
template <typename T, int VPL>
__device__ __forceinline__ void adam_apply(T* __restrict__ table, float* __restrict__ m, float* __restrict__ v,
                                           uint32_t f, uint32_t dpad, const float (&g)[VPL], float (&mm)[VPL],
                                           float (&vv)[VPL], float (&ee)[VPL], const AdamStep& as, uint64_t seed,
                                           int lane) {
    const uint64_t o = (uint64_t)f * dpad;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    const float lr = as.lr, rb1 = as.rb1, rb2 = as.rb2;
    const uint32_t step = as.step;
    float gn[VPL];
#pragma unroll
    for (int k = 0; k < VPL; ++k) gn[k] = g[k];
    if (as.sigma > 0.f) {
        // gradient noise g += sigma * N(0, 1) (mod.rs:239-247): Box-Muller on
        // two Philox draws per pair of elements, keyed by (row, step, column)
#pragma unroll
        for (int k = 0; k < VPL; k += 2) {
            const u32x4 r = philox(u32x4{f, step, (ST_NOISE << 24) | (uint32_t)(lane * VPL + k), 0u}, seed);
            const float u1 = ((float)(r.x >> 8) + 1.f) * (1.0f / 16777216.0f);   // (0, 1]
            const float u2 = (float)(r.y >> 8) * (1.0f / 16777216.0f);
            const float rad = sqrtf(-2.f * logf(u1));
            float sn, cs;
            sincosf(6.283185307179586f * u2, &sn, &cs);
            gn[k] += as.sigma * rad * cs;
            if (k + 1 < VPL) gn[k + 1] += as.sigma * rad * sn;
        }
    }
    if constexpr (VPL % 2 == 0) {
        // element pairs through the packed FP32 operations of sm_100+ (each
        // lane of a pair rounded as the scalar operation would be)
        const float2 B1 = make_float2(b1, b1), C1 = make_float2(1.f - b1, 1.f - b1);
        const float2 B2 = make_float2(b2, b2), C2 = make_float2(1.f - b2, 1.f - b2);
        const float2 R1 = make_float2(rb1, rb1), R2 = make_float2(rb2, rb2), E = make_float2(eps, eps);
        const float2 NL = make_float2(-lr, -lr);
#pragma unroll
        for (int k = 0; k < VPL; k += 2) {
            const float2 g = make_float2(gn[k], gn[k + 1]);
            const float2 m2 = __ffma2_rn(B1, make_float2(mm[k], mm[k + 1]), __fmul2_rn(C1, g));
            const float2 v2 = __ffma2_rn(B2, make_float2(vv[k], vv[k + 1]), __fmul2_rn(C2, __fmul2_rn(g, g)));
            const float2 mh = __fmul2_rn(m2, R1), vh = __fmul2_rn(v2, R2);
            const float2 den = __fadd2_rn(make_float2(sqrt_sfu(vh.x), sqrt_sfu(vh.y)), E);
            // the denominator is >= eps = 1e-8, inside the fast divide's full-accuracy range
            const float2 q = make_float2(div_sfu(mh.x, den.x), div_sfu(mh.y, den.y));
            const float2 e2 = __ffma2_rn(NL, q, make_float2(ee[k], ee[k + 1]));
            mm[k] = m2.x; mm[k + 1] = m2.y;
            vv[k] = v2.x; vv[k + 1] = v2.y;
            ee[k] = e2.x; ee[k + 1] = e2.y;
        }
    } else {
#pragma unroll
        for (int k = 0; k < VPL; ++k) {
            const float gk = gn[k];
            mm[k] = fmaf(b1, mm[k], (1.f - b1) * gk);
            vv[k] = fmaf(b2, vv[k], (1.f - b2) * (gk * gk));
            const float mh = mm[k] * rb1;
            const float vh = vv[k] * rb2;
            ee[k] = fmaf(-lr, div_sfu(mh, sqrt_sfu(vh) + eps), ee[k]);
        }
    }
    RowIO<float, VPL>::store_raw(m + o, lane, mm);
    RowIO<float, VPL>::store_raw(v + o, lane, vv);
    if constexpr (std::is_same<T, float>::value) {
        RowIO<float, VPL>::store_raw(table + o, lane, ee);
    } else {
        // BF16 table: stochastic rounding, 16 random bits per element; one
        // 32-bit hash (murmur3 finalizer of the element pair's coordinates
        // row, step, column) per pair of elements, rounded by one
        // stochastic-rounding conversion per pair.
        union {
            uint32_t w[(VPL + 1) / 2];
            __nv_bfloat16 b[VPL];
        } out;
        const uint32_t key = (uint32_t)seed ^ (uint32_t)(seed >> 32) ^ (f * 0x9E3779B1u) ^ (step * 0x85EBCA77u);
#pragma unroll
        for (int k = 0; k < VPL; k += 2) {
            const uint32_t h = mix32(key ^ ((uint32_t)(lane * VPL + k) * 0xC2B2AE3Du));
            if (k + 1 < VPL) out.w[k / 2] = bf16x2_stochastic(ee[k], ee[k + 1], h);
            else out.b[k] = bf16_stochastic(ee[k], h & 0xffffu);
        }
        RowIO<__nv_bfloat16, VPL>::store_raw(table + o, lane, out.b);
    }
}

template <typename T, int VPL, typename A>
__device__ __forceinline__ void adam_row(T* __restrict__ table, float* __restrict__ m, float* __restrict__ v,
                                         uint32_t f, uint32_t dpad, const A (&g)[VPL], const AdamStep& as,
                                         uint64_t seed, int lane, bool lane_on) {
    bool bad = false;
#pragma unroll
    for (int k = 0; k < VPL; ++k) bad = bad || (g[k] != g[k]);
    if (__any_sync(FULL, bad) || !lane_on) return;
    if constexpr (std::is_same<T, double>::value) {
        return;  // FP64 tables exist only for gradient checks
    } else {
        const uint64_t o = (uint64_t)f * dpad;
        float gg[VPL], mm[VPL], vv[VPL], ee[VPL];
#pragma unroll
        for (int k = 0; k < VPL; ++k) gg[k] = (float)g[k];
        RowIO<float, VPL>::load_cg(m + o, lane, mm);
        RowIO<float, VPL>::load_cg(v + o, lane, vv);
        RowIO<T, VPL>::load_cg(table + o, lane, ee);
        adam_apply<T, VPL>(table, m, v, f, dpad, gg, mm, vv, ee, as, seed, lane);
    }
}

// Per-warp list of features finished in OUT_DENSE mode, flushed to the
// touched list with one atomic per FIN_CAP entries (or at the end).
constexpr uint32_t FIN_CAP = 64;

__device__ __forceinline__ void fin_flush(const ReduceParams& p, uint32_t* fin, uint32_t& n_fin, int lane) {
    if (!n_fin) return;
    __syncwarp();
    uint32_t base = 0;
    if (lane == 0) base = atomicAdd(p.n_touched, n_fin);
    base = __shfl_sync(FULL, base, 0);
    for (uint32_t j = lane; j < n_fin; j += 32) p.touched[base + j] = fin[j];
    __syncwarp();
    n_fin = 0;
}

// OUT_QUEUE: a per-warp ring of QN slots in shared memory.  Queuing a
// finished feature row stores its gradient in the slot and starts
// asynchronous copies (cp.async) of the lane's slices of the feature's m, v
// and table rows into the slot; the copies of QN - 1 later rows are still in
// flight when the oldest slot is updated, so the update reads everything from
// shared memory and rarely waits.  Each lane copies and later reads only its
// own slices, so the per-thread cp.async groups order everything it needs.
constexpr uint32_t QN = 2;
constexpr int QUEUE_THREADS = 128;

template <typename T>
__host__ __device__ constexpr size_t queue_slot_bytes(uint32_t dpad) {
    return ((size_t)dpad * (3 * sizeof(float) + sizeof(T)) + 15) & ~(size_t)15;
}

struct WarpQueue {
    unsigned char* base;   // QN slots: g, m, v (float[dpad] each), table row (T[dpad])
    uint32_t* f;           // feature of each slot
    size_t sb;             // slot bytes
    uint32_t head, n;
};

__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

// Asynchronous copy of one lane slice of B bytes (B a multiple of 16, or 8 or 4).
template <int B>
__device__ __forceinline__ void cp_slice(void* dst, const void* src) {
    const uint32_t d = (uint32_t)__cvta_generic_to_shared(dst);
    if constexpr (B % 16 == 0) {
#pragma unroll
        for (int i = 0; i < B / 16; ++i)
            asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d + 16 * i),
                         "l"(reinterpret_cast<const char*>(src) + 16 * i)
                         : "memory");
    } else {
        static_assert(B == 8 || B == 4, "cp.async copies 4, 8 or 16 bytes");
        asm volatile("cp.async.ca.shared.global [%0], [%1], %2;" ::"r"(d), "l"(src), "n"(B) : "memory");
    }
}

// Slices of at least 4 bytes for every row go through cp.async; narrower
// rows (dims <= 64 with a BF16 table) are read synchronously at the update.
template <typename T, int VPL>
struct QueueAsync {
    static constexpr bool value = VPL * sizeof(T) >= 4 && VPL * sizeof(float) >= 4 && sizeof(T) != 8;
};

template <typename T, int VPL>
__device__ __forceinline__ void queue_slot_ptrs(const WarpQueue& q, uint32_t slot, uint32_t dpad, float*& g, float*& m,
                                                float*& v, T*& t) {
    g = reinterpret_cast<float*>(q.base + slot * q.sb);
    m = g + dpad;
    v = m + dpad;
    t = reinterpret_cast<T*>(v + dpad);
}

// Adam on the oldest slot (optimizer.rs:43-81).  The caller has waited for
// that slot's copies.
template <typename T, int VPL>
__device__ __forceinline__ void queue_pop(const ReduceParams& p, WarpQueue& q, int lane, bool lane_on,
                                          const AdamStep& as) {
    if constexpr (sizeof(T) != 8) {
        const uint32_t dpad = p.dpad;
        float *gs, *ms, *vs;
        T* ts;
        queue_slot_ptrs<T, VPL>(q, q.head, dpad, gs, ms, vs, ts);
        const uint32_t f = q.f[q.head];
        if (lane_on) {
            float gg[VPL], mm[VPL], vv[VPL], ee[VPL];
            RowIO<float, VPL>::load_generic(gs, lane, gg);
            if constexpr (QueueAsync<T, VPL>::value) {
                RowIO<float, VPL>::load_generic(ms, lane, mm);
                RowIO<float, VPL>::load_generic(vs, lane, vv);
                RowIO<T, VPL>::load_generic(ts, lane, ee);
            } else {
                const uint64_t o = (uint64_t)f * dpad;
                RowIO<float, VPL>::load_cg(p.m + o, lane, mm);
                RowIO<float, VPL>::load_cg(p.v + o, lane, vv);
                RowIO<T, VPL>::load_cg((const T*)p.table + o, lane, ee);
            }
            adam_apply<T, VPL>((T*)p.table, p.m, p.v, f, dpad, gg, mm, vv, ee, as, p.seed, lane);
        }
    }
    q.head = q.head + 1 == QN ? 0u : q.head + 1;
    --q.n;
}

// Queues a finished (NaN-free) row, then, when every slot is taken, updates
// the oldest: the new row's copies are issued first, so they are in flight
// while the oldest row is updated as well as while the next rows reduce.
template <typename T, typename A, int VPL>
__device__ __forceinline__ void queue_push(const ReduceParams& p, WarpQueue& q, uint32_t f, const A (&acc)[VPL], int lane,
                                           bool lane_on, const AdamStep& as) {
    uint32_t slot = q.head + q.n;
    if (slot >= QN) slot -= QN;
    float *gs, *ms, *vs;
    T* ts;
    const uint32_t dpad = p.dpad;
    queue_slot_ptrs<T, VPL>(q, slot, dpad, gs, ms, vs, ts);
    if (lane_on) {
        store_row<float, VPL, A>(gs, lane, acc);
        if constexpr (QueueAsync<T, VPL>::value) {
            const uint64_t o = (uint64_t)f * dpad + (uint64_t)lane * VPL;
            cp_slice<VPL * 4>(ms + lane * VPL, p.m + o);
            cp_slice<VPL * 4>(vs + lane * VPL, p.v + o);
            cp_slice<VPL * (int)sizeof(T)>(ts + lane * VPL, (const T*)p.table + o);
        }
    }
    cp_async_commit();
    if (lane == 0) q.f[slot] = f;
    ++q.n;
    if (q.n == QN) {
        cp_async_wait<QN - 1>();
        __syncwarp();
        queue_pop<T, VPL>(p, q, lane, lane_on, as);
    }
}

// Updates every queued slot (end of the warp's work).
template <typename T, int VPL>
__device__ __forceinline__ void queue_flush(const ReduceParams& p, WarpQueue& q, int lane, bool lane_on,
                                            const AdamStep& as) {
    cp_async_wait<0>();
    __syncwarp();
    while (q.n) queue_pop<T, VPL>(p, q, lane, lane_on, as);
}

// ---------------------------------------------------------------------------
// OUT_RING: warp-specialised reduction.  A CTA runs pw reducing warps and cw
// Adam warps around a ring of `slots` shared-memory slots, each holding one
// finished feature row: its gradient (stored by the reducing warp), and the
// feature's m, v and table rows, which one lane of the reducing warp fetches
// with three bulk copies (cp.async.bulk, the TMA's linear form) counted on
// the slot's `full` mbarrier.  Adam warp k takes tickets k, k + cw, ... in
// order, waits for the slot's copies, updates the row in place in HBM and
// releases the slot on its `empty` mbarrier.  The reducing warps thus never
// wait for HBM (only for a free slot), and the Adam warps never wait for the
// reduction's L2 traffic: the two latency chains overlap.
//
// Tickets are handed out by a shared-memory counter, so the slot of ticket t
// is t % slots in round t / slots.  A reducing warp takes its ticket without
// waiting, so it may hold a round of its slot several rounds ahead of the
// consumer; it therefore waits on the slot's count of consumed rounds (a
// word that only grows), not on an mbarrier parity, which only tells the
// current phase from the one before.  Adam warp k owns the slots congruent
// to k modulo cw (slots is a multiple of cw) and takes their rounds in
// order, so when it waits on a slot's `full` parity for round r it has itself
// seen round r - 1 complete, and no producer can have completed round r + 1
// (that producer waits for round r to be consumed): the parity is exact.
// No wait can close a cycle: the smallest unfilled ticket's producer only
// waits for earlier rounds of its slot, and every ticket before it is filled.
// Every poll loop is bounded (RING_WAIT_LIMIT); a loop that gives up sets
// ERR_RING_TIMEOUT and the CTA's abort word, so all warps stop waiting, and
// the CTA waits (bounded) for the bulk copies it issued before it exits.  The
// host reports the error bit.
// ---------------------------------------------------------------------------
constexpr uint32_t RING_WAIT_LIMIT = 1u << 21;   // polls of about 32 ns each
constexpr uint32_t RING_MAX_WARPS = 16;

struct RingHdr {
    unsigned long long full[64];              // mbarrier per slot: the row and its bulk copies landed
    uint32_t consumed[64];                    // rounds of the slot the Adam warp has finished
    uint32_t f[64];                           // feature of the row in the slot
    uint32_t issued[64];                      // rounds whose copies were issued, per slot
    uint32_t tail;                            // next ticket
    uint32_t done;                            // reducing warps finished
    uint32_t abort;
};
constexpr uint32_t RING_MAX_SLOTS = 64;

template <typename T>
__host__ __device__ constexpr size_t ring_slot_bytes(uint32_t dpad) {
    return (size_t)dpad * (3 * sizeof(float) + sizeof(T));   // g, m, v (FP32) + table row; 16-byte multiples
}
__host__ __device__ constexpr size_t ring_hdr_bytes() { return (sizeof(RingHdr) + 127) & ~(size_t)127; }

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint32_t ring_test(unsigned long long* bar, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return done;
}

__device__ __forceinline__ void ring_set_abort(const ReduceParams& p, RingHdr* rh) {
    atomicExch(&rh->abort, 1u);
    atomicOr(&p.st->error, ERR_RING_TIMEOUT);
}

// Waits (whole warp, lane 0 polling) until the Adam warp has finished
// `rounds` rounds of the slot.  Returns false when the CTA aborts or the wait
// gives up (then the abort is raised).
__device__ __forceinline__ bool ring_wait_consumed(const ReduceParams& p, RingHdr* rh, uint32_t slot,
                                                   uint32_t rounds) {
    uint32_t ok = 0;
    if ((threadIdx.x & 31) == 0) {
        volatile RingHdr* vh = rh;
        for (uint32_t it = 0; it < RING_WAIT_LIMIT; ++it) {
            if (vh->consumed[slot] >= rounds) { ok = 1; break; }
            if (vh->abort) break;
            __nanosleep(32);
        }
        if (!ok && !vh->abort) ring_set_abort(p, rh);
        __threadfence_block();   // the consumer's reads of the slot happen before our writes
    }
    return __shfl_sync(FULL, ok, 0) != 0;
}

// Reducing warp: queue a finished NaN-free row for the Adam warps.
template <typename T, typename A, int VPL>
__device__ __forceinline__ void ring_push(const ReduceParams& p, RingHdr* rh, unsigned char* slots, uint32_t f,
                                          const A (&acc)[VPL], int lane, bool lane_on) {
    const uint32_t S = p.ring_slots, dpad = p.dpad;
    uint32_t t = 0;
    if (lane == 0) t = atomicAdd(&rh->tail, 1u);
    t = __shfl_sync(FULL, t, 0);
    const uint32_t slot = t % S, round = t / S;
    if (round > 0 && !ring_wait_consumed(p, rh, slot, round)) return;   // row dropped: aborting
    unsigned char* base = slots + (size_t)slot * ring_slot_bytes<T>(dpad);
    float* g = reinterpret_cast<float*>(base);
    if (lane_on) store_row<float, VPL, A>(g, lane, acc);
    __threadfence_block();
    __syncwarp();
    if (lane == 0) {
        rh->f[slot] = f;
        rh->issued[slot] = round + 1;
        const uint32_t mb = dpad * 4u, tb = dpad * (uint32_t)sizeof(T);
        const uint32_t bar = smem_addr(&rh->full[slot]);
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(2 * mb + tb) : "memory");
        const char* src[3] = {reinterpret_cast<const char*>(p.m) + (uint64_t)f * mb,
                              reinterpret_cast<const char*>(p.v) + (uint64_t)f * mb,
                              reinterpret_cast<const char*>(p.table) + (uint64_t)f * tb};
        const uint32_t dst[3] = {smem_addr(base + mb), smem_addr(base + 2 * mb), smem_addr(base + 3 * mb)};
        const uint32_t len[3] = {mb, mb, tb};
#pragma unroll
        for (int i = 0; i < 3; ++i)
            asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                         ::"r"(dst[i]), "l"(src[i]), "r"(len[i]), "r"(bar)
                         : "memory");
    }
    __syncwarp();
}

// Adam warp `k` of the CTA: tickets k, k + cw, ... (its slots' rounds in
// order) until every reducing warp has finished and no later ticket was taken.
template <typename T, int VPL>
__device__ void ring_consume(const ReduceParams& p, RingHdr* rh, unsigned char* slots, uint32_t k, int lane,
                             bool lane_on, const AdamStep& as) {
    const uint32_t S = p.ring_slots, dpad = p.dpad;
    for (uint32_t h = k;; h += p.ring_cw) {
        const uint32_t slot = h % S, round = h / S;
        uint32_t mine = 0, got = 0;
        for (uint32_t it = 0;; ++it) {
            if (!mine) mine = ring_test(&rh->full[slot], round & 1u);
            if (__all_sync(FULL, mine)) { got = 1; break; }
            uint32_t stop = 0;
            if (lane == 0) {
                // `done` before `tail`: a reducing warp takes its last ticket
                // before it counts itself done, so once all are done the
                // ticket count read after the fence is final
                volatile RingHdr* vh = rh;
                const uint32_t d = vh->done;
                __threadfence_block();
                const uint32_t tl = vh->tail;
                stop = vh->abort || (d == p.ring_pw && tl <= h);
            }
            if (__shfl_sync(FULL, stop, 0) && !__any_sync(FULL, mine)) break;
            if (it >= RING_WAIT_LIMIT) {
                if (lane == 0) ring_set_abort(p, rh);
                break;
            }
            __nanosleep(32);
        }
        if (!got) return;
        const unsigned char* base = slots + (size_t)slot * ring_slot_bytes<T>(dpad);
        const uint32_t f = rh->f[slot];
        if (lane_on) {
            float gg[VPL], mm[VPL], vv[VPL], ee[VPL];
            const float* g = reinterpret_cast<const float*>(base);
            RowIO<float, VPL>::load_generic(g, lane, gg);
            RowIO<float, VPL>::load_generic(g + dpad, lane, mm);
            RowIO<float, VPL>::load_generic(g + 2 * dpad, lane, vv);
            RowIO<T, VPL>::load_generic(reinterpret_cast<const T*>(g + 3 * dpad), lane, ee);
            adam_apply<T, VPL>((T*)p.table, p.m, p.v, f, dpad, gg, mm, vv, ee, as, p.seed, lane);
        }
        __syncwarp();
        if (lane == 0) {
            __threadfence_block();   // our reads of the slot before the producer's reuse
            *(volatile uint32_t*)&rh->consumed[slot] = round + 1;
        }
    }
}

template <typename T, typename A, int VPL, int MODE>
__device__ __forceinline__ void finish_row(const ReduceParams& p, uint32_t f, const A (&acc)[VPL], int lane,
                                           bool lane_on, const AdamStep& as, uint32_t* fin, uint32_t& n_fin,
                                           WarpQueue* q = nullptr, RingHdr* rh = nullptr,
                                           unsigned char* ring_slots = nullptr) {
    if constexpr (MODE == OUT_RING) {
        // rows containing NaN get no Adam step (optimizer.rs:56): not queued
        bool bad = false;
#pragma unroll
        for (int k = 0; k < VPL; ++k) bad = bad || (acc[k] != acc[k]);
        if (!__any_sync(FULL, bad)) ring_push<T, A, VPL>(p, rh, ring_slots, f, acc, lane, lane_on);
    } else if constexpr (MODE == OUT_QUEUE) {
        // rows containing NaN get no Adam step (optimizer.rs:56): not queued
        bool bad = false;
#pragma unroll
        for (int k = 0; k < VPL; ++k) bad = bad || (acc[k] != acc[k]);
        if (!__any_sync(FULL, bad)) queue_push<T, A, VPL>(p, *q, f, acc, lane, lane_on, as);
    } else if constexpr (MODE == OUT_DENSE) {
        if (lane_on) store_row<A, VPL, A>((A*)p.gdense + (uint64_t)f * p.dpad, lane, acc);
        if (fin) {
            if (lane == 0) fin[n_fin] = f;
            if (++n_fin == FIN_CAP) fin_flush(p, fin, n_fin, lane);
        } else if (lane == 0) {
            p.touched[atomicAdd(p.n_touched, 1u)] = f;
        }
    } else {
        adam_row<T, VPL, A>((T*)p.table, p.m, p.v, f, p.dpad, acc, as, p.seed, lane, lane_on);
    }
}

// Bulk L2 prefetch (cp.async.bulk.prefetch) of one feature's Adam state:
// moment rows m, v and the table row.  Rows must be 16-byte multiples.
template <typename T>
__device__ __forceinline__ void prefetch_row_state(const ReduceParams& p, uint32_t f) {
    const uint32_t mb = p.dpad * 4u, tb = p.dpad * (uint32_t)sizeof(T);
    if ((mb & 15u) || (tb & 15u)) return;
    const char* m = reinterpret_cast<const char*>(p.m) + (uint64_t)f * mb;
    const char* v = reinterpret_cast<const char*>(p.v) + (uint64_t)f * mb;
    const char* t = reinterpret_cast<const char*>(p.table) + (uint64_t)f * tb;
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(m), "r"(mb) : "memory");
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(v), "r"(mb) : "memory");
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(t), "r"(tb) : "memory");
}

// For the 32 items starting at position b (clipped to end), the lanes whose
// item starts a feature segment prefetch that feature's Adam state.
template <typename T>
__device__ __forceinline__ void prefetch_segment_state(const ReduceParams& p, uint32_t b, uint32_t end, int lane) {
    if constexpr (sizeof(T) == 8) {
        return;   // FP64 tables exist only for gradient checks (no Adam)
    } else {
        const uint32_t i = b + lane;
        if (i < end && i > 0) {
            const uint32_t f = p.skey[i];
            if (f != p.skey[i - 1]) prefetch_row_state<T>(p, f);
        }
    }
}

// End of an OUT_RING CTA (every warp of both roles): once all warps are
// here, the bulk copies of each slot's last issued round must have landed
// before the CTA's shared memory is released.
__device__ __forceinline__ void ring_finish(const ReduceParams& p, RingHdr* rh) {
    asm volatile("bar.sync 1, %0;" ::"r"(blockDim.x) : "memory");
    if (threadIdx.x == 0) {
        for (uint32_t s = 0; s < p.ring_slots; ++s) {
            const uint32_t r = rh->issued[s];
            if (!r) continue;
            uint32_t it = 0;
            while (!ring_test(&rh->full[s], (r - 1) & 1u) && ++it < RING_WAIT_LIMIT) __nanosleep(32);
            if (it >= RING_WAIT_LIMIT) atomicOr(&p.st->error, ERR_RING_TIMEOUT);
        }
    }
}

// Per-warp lists of one window of RW sorted items, built by the warp's lanes
// in parallel and then walked in order: the kept items (direction row and
// weight) and the feature segments that start in the window (feature id and
// the number of kept items before it).  Walking the list costs one broadcast
// shared-memory load per kept item instead of a search of the batch's masks
// and two shuffles, and the direction rows of NF consecutive kept items are
// in flight together across feature boundaries.
constexpr uint32_t RW = 128;

template <typename A>
struct RedEntry {
    uint32_t src;   // role row of the direction buffer
    A w;            // count weight x role scale
};

template <typename A>
__host__ __device__ constexpr size_t list_bytes() {
    return RW * (sizeof(RedEntry<A>) + sizeof(uint2));
}

// Offset of the lists in the reducer's dynamic shared memory (after the
// OUT_QUEUE slots and their ids, or the OUT_RING header and slots).
template <typename T>
__host__ __device__ constexpr size_t queue_list_offset(uint32_t dpad, uint32_t warps) {
    return ((size_t)warps * QN * (queue_slot_bytes<T>(dpad) + sizeof(uint32_t)) + 15) & ~(size_t)15;
}

// A span (owner chunk c, feature f) is long when f still fills the start of
// chunk c + 1 + FIX_SHORT, i.e. its last chunk is more than FIX_SHORT past c.
constexpr uint32_t FIX_SHORT = 16;
__device__ __forceinline__ bool span_is_long(const ReduceParams& p, uint32_t c, uint32_t f, uint32_t M, uint32_t C) {
    const uint64_t probe = (uint64_t)(c + 1 + FIX_SHORT) * C;
    return probe < M && p.skey[probe] == f;
}

template <typename T, typename A, int VPL, int MODE>
__device__ __forceinline__ void reduce_body(const ReduceParams& p);

// k_reduce: one warp per chunk of C sorted items, in windows of RW items.
// Phase 1 takes the window 32 items (one per lane) at a time: the
// first-occurrence rule is evaluated for all 32 at once with ballots (group
// starts: new feature or new anchor; valid roles; for every item the first
// valid role of its (feature, anchor) group, carried across batches and, at a
// chunk start, found by walking back), and the kept items and the feature
// starts are appended to the warp's lists.  Item metadata is
// software-pipelined: while batch b is examined, the role flags and scales of
// batch b+1 and the keys of batch b+2 are in flight.  Phase 2 streams the
// kept items' direction rows in list order, NF in flight across feature
// boundaries; a feature is finished when the stream reaches the first kept
// item of the next one.
template <typename T, typename A, int VPL, int MODE>
__global__ void __launch_bounds__(MODE == OUT_RING ? RING_MAX_WARPS * 32 : (MODE == OUT_QUEUE ? QUEUE_THREADS : RED_THREADS),
                                  MODE == OUT_RING ? 1 : (VPL >= 16 ? 1 : (MODE == OUT_DENSE ? 3 : (MODE == OUT_QUEUE ? 4 : 2))))
    k_reduce(ReduceParams p) {
    reduce_body<T, A, VPL, MODE>(p);
}

// The per-warp queue reducer at five CTAs per SM instead of four: registers
// capped at 96 a thread (from 117; a few bytes spill) for 25% more resident
// warps.  Same arithmetic in the same order.
template <typename T, typename A, int VPL>
__global__ void __launch_bounds__(QUEUE_THREADS, 5) k_reduce_q5(ReduceParams p) {
    reduce_body<T, A, VPL, OUT_QUEUE>(p);
}

template <typename T, typename A, int VPL, int MODE>
__device__ __forceinline__ void reduce_body(const ReduceParams& p) {
    pdl_wait();
    pdl_trigger();
    using D = typename DirOf<T, A>::type;
    using IO = RowIO<D, VPL>;
    // rows in flight: about 24-32 registers of raw data in the rows-only mode,
    // fewer where a finished row is updated in place while others are in flight
    constexpr int NF = MODE == OUT_DENSE ? (sizeof(D) == 2 ? 4 : 3) : (MODE == OUT_QUEUE ? 3 : 2);
    __shared__ uint32_t fin_all[MODE == OUT_DENSE ? RED_THREADS / 32 : 1][FIN_CAP];
    extern __shared__ __align__(16) unsigned char red_queue[];   // OUT_QUEUE: [warps][QN] slots, then ids
    const int lane = threadIdx.x & 31;
    uint32_t* fin = fin_all[MODE == OUT_DENSE ? (threadIdx.x >> 5) : 0];
    uint32_t n_fin = 0;
    WarpQueue q;
    q.sb = queue_slot_bytes<T>(p.dpad);
    q.base = red_queue + (size_t)(threadIdx.x >> 5) * QN * q.sb;
    q.f = reinterpret_cast<uint32_t*>(red_queue + (size_t)(blockDim.x >> 5) * QN * q.sb) + (threadIdx.x >> 5) * QN;
    q.head = 0;
    q.n = 0;
    RingHdr* rh = reinterpret_cast<RingHdr*>(red_queue);
    unsigned char* ring_slots = red_queue + ring_hdr_bytes();
    const uint32_t warp = threadIdx.x >> 5;
    RedEntry<A>* ents;
    uint2* segs;
    {
        size_t off = 0;
        if constexpr (MODE == OUT_QUEUE) off = queue_list_offset<T>(p.dpad, blockDim.x >> 5);
        if constexpr (MODE == OUT_RING) off = ring_hdr_bytes() + (size_t)p.ring_slots * ring_slot_bytes<T>(p.dpad);
        unsigned char* lb = red_queue + off + (size_t)warp * list_bytes<A>();
        ents = reinterpret_cast<RedEntry<A>*>(lb);
        segs = reinterpret_cast<uint2*>(lb + RW * sizeof(RedEntry<A>));
    }
    if constexpr (MODE == OUT_RING) {
        if (threadIdx.x == 0) {
            for (uint32_t i = 0; i < p.ring_slots; ++i) {
                asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&rh->full[i])) : "memory");
                rh->issued[i] = 0;
                rh->consumed[i] = 0;
            }
            rh->tail = 0;
            rh->done = 0;
            rh->abort = 0;
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        }
        __syncthreads();
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {   // read by k_fixup / k_fixup_long / k_adam_dense
        BatchState* st = p.st;
        st->fx_items = st->n_items;
        st->fx_step = st->step_cur;
        st->fx_lr = st->lr;
        st->fx_bc1 = st->bc1;
        st->fx_bc2 = st->bc2;
        st->fx_sigma = st->noise_sigma;
    }
    const unsigned lt_mask = (1u << lane) - 1u;
    // OUT_RING: warps [0, ring_pw) reduce, the others run Adam
    const uint32_t gw = MODE == OUT_RING ? blockIdx.x * p.ring_pw + warp : (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nw = MODE == OUT_RING ? gridDim.x * p.ring_pw : (gridDim.x * blockDim.x) >> 5;
    const uint32_t M = p.st->n_items;
    const uint32_t C = p.chunk;
    const uint32_t nchunks = (M + C - 1) / C;
    const uint32_t NR = p.NR;
    const bool lane_on = (uint32_t)(lane * VPL) < p.dpad;
    // lanes past the row (dims < 32 x VPL) read its last slice and accumulate
    // what no store uses, so that the item loop has no lane-dependent branch
    const int lane_ld = lane_on ? lane : (int)(p.dpad / VPL) - 1;
    const AdamStep as = AdamStep::load(p.st);
    if constexpr (MODE == OUT_RING) {
        if (warp >= p.ring_pw) {
            ring_consume<T, VPL>(p, rh, ring_slots, warp - p.ring_pw, lane, lane_on, as);
            ring_finish(p, rh);
            return;
        }
    }
    const D* dir = std::is_same<D, A>::value ? (const D*)p.dir : (const D*)p.dir16;
    const A* scale = (const A*)p.scale;
    unsigned long long g_cnt = 0, u_cnt = 0;
    // chunks: a static stride over the grid's warps, or, with a persistent
    // grid (red_ctas > 0), the next chunk from the batch's work counter, so
    // that a warp whose chunk finishes early takes another at once instead
    // of idling until its CTA's other warps finish (the result is the same:
    // every chunk is reduced alone, and the fix-ups combine them in order)
    const bool take = MODE != OUT_RING && p.red_ctas != 0;
    auto next_chunk = [&]() {
        uint32_t t = 0;
        if (lane == 0) t = atomicAdd(&p.st->red_next, 1u);
        return __shfl_sync(FULL, t, 0);
    };
    for (uint32_t c = take ? next_chunk() : gw; c < nchunks; c = take ? next_chunk() : c + nw) {
        const uint32_t i0 = c * C, i1 = min(i0 + C, M);
        uint32_t cur_f = p.skey[i0];
        const bool head_partial = i0 > 0 && p.skey[i0 - 1] == cur_f;
        uint32_t cur_anchor = p.sval[i0].x / NR;
        uint32_t chosen = NONE;           // first valid role of the current group
        // the item before the batch (lane 0's predecessor)
        uint32_t prev_src = NONE, prev_f = NONE, prev_anchor = NONE;
        if (i0 > 0) {
            prev_src = p.sval[i0 - 1].x;
            prev_f = p.skey[i0 - 1];
            prev_anchor = prev_src / NR;
        }
        if (head_partial) {
            if (!p.grad_true) {
                int64_t j = (int64_t)i0 - 1;
                for (;;) {
                    const int64_t jj = j - lane;
                    bool in = false;
                    uint32_t s = 0;
                    if (jj >= 0 && p.skey[jj] == cur_f) {
                        s = p.sval[jj].x;
                        in = (s / NR) == cur_anchor;
                    }
                    const unsigned inm = __ballot_sync(FULL, in);
                    const unsigned run = (~inm) ? ((1u << (__ffs(~inm) - 1)) - 1u) : FULL;
                    const bool vv = in && ((run >> lane) & 1u) && p.valid[s];
                    const unsigned vm = __ballot_sync(FULL, vv);
                    if (vm) chosen = __shfl_sync(FULL, s, 31 - __clz(vm));
                    if (run != FULL) break;
                    j -= 32;
                }
            }
        }
        A acc[VPL];
#pragma unroll
        for (int k = 0; k < VPL; ++k) acc[k] = 0;
        bool started_here = !head_partial;
        bool any_kept = false;
        uint32_t flags = 0;
        if constexpr (MODE == OUT_ADAM) prefetch_segment_state<T>(p, i0, i1, lane);

        // metadata pipeline: (f0, s0, c0, v0, sc0) for the current batch,
        // (f1, s1, c1) for the next one; v1/sc1 are loaded one batch ahead
        uint32_t f0 = NONE, s0 = 0, f1 = NONE, s1 = 0;
        float c0 = 0.f, c1 = 0.f;
        bool v0 = false;
        A sc0 = 0;
        {
            const uint32_t i = i0 + lane;
            if (i < i1) {
                f0 = p.skey[i];
                const uint2 sv = p.sval[i];
                s0 = sv.x;
                c0 = __uint_as_float(sv.y);
            }
            const uint32_t j = i0 + 32 + lane;
            if (j < i1) {
                f1 = p.skey[j];
                const uint2 sv = p.sval[j];
                s1 = sv.x;
                c1 = __uint_as_float(sv.y);
            }
            if (i < i1) {
                v0 = p.valid[s0] != 0;
                sc0 = scale[s0];
            }
        }
        // closes the open feature (finished here, or a head partial for the
        // fix-up) and opens feature fnew
        auto close_open = [&](uint32_t fnew) {
            if (started_here) {
                if (any_kept) {
                    finish_row<T, A, VPL, MODE>(p, cur_f, acc, lane, lane_on, as, fin, n_fin, &q, rh, ring_slots);
                    ++u_cnt;
                }
            } else {
                if (lane_on) store_row<A, VPL, A>((A*)p.carry_head + (uint64_t)c * p.dpad, lane, acc);
                flags |= CF_HEAD | (any_kept ? CF_HEAD_KEPT : 0u);
            }
#pragma unroll
            for (int k = 0; k < VPL; ++k) acc[k] = 0;
            started_here = true;
            any_kept = false;
            cur_f = fnew;
        };
        for (uint32_t wb = i0; wb < i1; wb += RW) {
            const uint32_t we = min(wb + RW, i1);
            // phase 1, 32 items per step with the lanes in parallel: which
            // items are kept, their weights, where features start; appended
            // to the window's lists
            uint32_t nk = 0, ns = 0;
            for (uint32_t ib = wb; ib < we; ib += 32) {
                const uint32_t i = ib + lane;
                const bool act = i < i1;
                const uint32_t f = f0, s = s0;
                const float cf = c0;
                const bool v = v0;
                const A sc = sc0;
                // next batch's role flags and scales; the batch after's keys
                bool v1 = false;
                A sc1 = 0;
                uint32_t f2 = NONE, s2 = 0;
                float c2 = 0.f;
                if (ib + 32 + lane < i1) {
                    v1 = p.valid[s1] != 0;
                    sc1 = scale[s1];
                }
                if (ib + 64 + lane < i1) {
                    const uint32_t j = ib + 64 + lane;
                    f2 = p.skey[j];
                    const uint2 sv = p.sval[j];
                    s2 = sv.x;
                    c2 = __uint_as_float(sv.y);
                }
                if constexpr (MODE == OUT_ADAM) prefetch_segment_state<T>(p, ib + 32, i1, lane);
                const uint32_t anchor = s / NR;
                // predecessor of each lane (lane 0: the carried item before the batch)
                uint32_t pf = __shfl_up_sync(FULL, f, 1), pa = __shfl_up_sync(FULL, anchor, 1);
                uint32_t ps = __shfl_up_sync(FULL, s, 1);
                if (lane == 0) { pf = prev_f; pa = prev_anchor; ps = prev_src; }
                const bool seg_start = act && f != pf;
                const bool grp_start = act && (seg_start || anchor != pa);
                if (act) g_cnt += (seg_start || s != ps);
                const unsigned GS = __ballot_sync(FULL, grp_start);
                const unsigned V = __ballot_sync(FULL, act && v);
                bool keep;
                if (p.grad_true) {
                    keep = act && v;
                } else {
                    // lanes of this item's group up to and including itself
                    const unsigned gs_le = GS & (lt_mask | (1u << lane));
                    const int gstart = gs_le ? 31 - __clz(gs_le) : -1;
                    const unsigned grp = (lt_mask | (1u << lane)) & (gstart >= 0 ? ~((1u << gstart) - 1u) : FULL);
                    const unsigned vg = V & grp;
                    const int fv = vg ? __ffs(vg) - 1 : 0;
                    const uint32_t src_fv = __shfl_sync(FULL, s, fv);
                    uint32_t ch = NONE;
                    if (gstart < 0 && chosen != NONE) ch = chosen;      // group began before this batch
                    else if (vg) ch = src_fv;
                    keep = act && v && s == ch;
                    // carry the group state of the batch's last item
                    const int lastl = 31 - __clz(__ballot_sync(FULL, act));
                    chosen = __shfl_sync(FULL, ch, lastl);
                }
                const unsigned KM = __ballot_sync(FULL, keep);
                const uint32_t kr = nk + __popc(KM & lt_mask);
                if (keep) {
                    RedEntry<A> e;
                    e.src = s;
                    e.w = (A)cf * sc;
                    ents[kr] = e;
                }
                // the chunk's first item belongs to the feature opened above
                const bool opens = seg_start && i != i0;
                const unsigned SS = __ballot_sync(FULL, opens);
                if (opens) segs[ns + __popc(SS & lt_mask)] = make_uint2(f, kr);
                nk += __popc(KM);
                ns += __popc(SS);
                const int last = 31 - __clz(__ballot_sync(FULL, act));
                prev_f = __shfl_sync(FULL, f, last);
                prev_anchor = __shfl_sync(FULL, anchor, last);
                prev_src = __shfl_sync(FULL, s, last);
                f0 = f1; s0 = s1; c0 = c1; v0 = v1; sc0 = sc1;
                f1 = f2; s1 = s2; c1 = c2;
            }
            __syncwarp();
            // phase 2: the kept items in order, NF direction rows in flight;
            // features close where the next one's first kept item comes
            uint32_t j = 0;
            uint32_t next_b = ns ? segs[0].y : 0xffffffffu;
            for (uint32_t k = 0; k < nk; k += NF) {
                uint32_t src[NF];
                A wv[NF];
#pragma unroll
                for (int u = 0; u < NF; ++u) {
                    src[u] = 0;
                    wv[u] = 0;
                    if (k + u < nk) {
                        const RedEntry<A> e = ents[k + u];
                        src[u] = e.src;
                        wv[u] = e.w;
                    }
                }
                typename IO::Raw r[NF];
#pragma unroll
                for (int u = 0; u < NF; ++u)
                    if (k + u < nk) r[u] = IO::load_raw(dir + (uint64_t)src[u] * p.dpad, lane_ld);
                if (k + NF <= nk && k + NF <= next_b) {   // no feature starts among these NF
#pragma unroll
                    for (int u = 0; u < NF; ++u) IO::template fma<A>(acc, wv[u], r[u]);
                    any_kept = true;
                    continue;
                }
#pragma unroll
                for (int u = 0; u < NF; ++u) {
                    if (k + u < nk) {
                        while (k + u >= next_b) {
                            close_open(segs[j].x);
                            ++j;
                            next_b = j < ns ? segs[j].y : 0xffffffffu;
                        }
                        IO::template fma<A>(acc, wv[u], r[u]);
                        any_kept = true;
                    }
                }
            }
            // features of the window with no kept item after their start
            for (; j < ns; ++j) close_open(segs[j].x);
            __syncwarp();
        }
        const bool cont = i1 < M && p.skey[i1] == cur_f;
        if (started_here && !cont) {
            if (any_kept) {
                finish_row<T, A, VPL, MODE>(p, cur_f, acc, lane, lane_on, as, fin, n_fin, &q, rh, ring_slots);
                ++u_cnt;
            }
        } else if (!started_here) {
            if (lane_on) store_row<A, VPL, A>((A*)p.carry_head + (uint64_t)c * p.dpad, lane, acc);
            flags |= CF_HEAD | (cont ? CF_THROUGH : 0u) | (any_kept ? CF_HEAD_KEPT : 0u);
        } else {
            if (lane_on) store_row<A, VPL, A>((A*)p.carry_tail + (uint64_t)c * p.dpad, lane, acc);
            if (lane == 0) p.carry_f[c] = cur_f;
            flags |= CF_OWNER | (any_kept ? CF_TAIL_KEPT : 0u);
            if (lane == 0 && span_is_long(p, c, cur_f, M, C)) {
                const uint32_t par = as.step & 1u;
                p.long_list[(size_t)par * p.long_cap + atomicAdd(&p.st->n_long[par], 1u)] = c;
            }
        }
        if (lane == 0) p.carry_flags[c] = flags;
    }
    if constexpr (MODE == OUT_DENSE) fin_flush(p, fin, n_fin, lane);
    if constexpr (MODE == OUT_QUEUE) queue_flush<T, VPL>(p, q, lane, lane_on, as);
    if constexpr (MODE == OUT_RING) {
        __syncwarp();
        if (lane == 0) {
            __threadfence_block();
            atomicAdd(&rh->done, 1u);
        }
    }
    g_cnt = warp_sum<unsigned long long>(g_cnt);
    if (lane == 0) {
        if (g_cnt) atomicAdd(&p.st->gathered, g_cnt);
        if (u_cnt) atomicAdd(&p.st->unique_rows, u_cnt);
    }
    if constexpr (MODE == OUT_RING) ring_finish(p, rh);
}

// Chunk holding the last item of feature f, whose segment starts in chunk c
// and continues into c + 1: usually c + 1; otherwise a 32-ary warp search
// over [(c+2)*C - 1, M), where skey == f is a prefix.
__device__ __forceinline__ uint32_t owner_last(const ReduceParams& p, uint32_t c, uint32_t f, uint32_t M, uint32_t C,
                                               int lane) {
    if (!(p.carry_flags[c + 1] & CF_THROUGH)) return c + 1;
    uint32_t lo = (c + 2) * C - 1, hi = M;   // skey[lo] == f; skey[hi] != f or hi == M
    while (hi - lo > 1) {
        const uint32_t span = hi - lo;
        const uint32_t stepw = span > 32 ? span / 32 : 1;
        const uint32_t probe = lo + (uint32_t)(lane + 1) * stepw;
        const bool in = probe < hi && p.skey[probe] == f;
        const uint32_t k = __popc(__ballot_sync(FULL, in));
        const uint32_t nlo = lo + k * stepw;
        // probe k + 1 (outside f, or past hi) bounds the span; when all 32
        // probes are inside, nothing new is known above the last one
        if (k < 32) hi = min(hi, nlo + stepw);
        lo = nlo;
    }
    return lo / C;
}

// k_fixup: one warp per owner chunk (a chunk whose last feature continues into
// later chunks).  Spans of up to FIX_SHORT partials are summed by the warp in
// chunk order (owner's tail, then the heads of c+1 .. last) and finished;
// longer spans, which k_reduce queued, are left to k_fixup_long, so that the
// two kernels can run side by side.
// k_fixup_long block size: as many warps as the row width leaves registers for
__host__ __device__ constexpr int fixl_threads(int vpl) { return vpl >= 16 ? 256 : (vpl >= 8 ? 512 : 1024); }

template <typename T, typename A, int VPL, int MODE>
__global__ void __launch_bounds__(FIX_THREADS) k_fixup(ReduceParams p) {
    pdl_wait();
    pdl_trigger();
    const int lane = threadIdx.x & 31;
    const uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    const uint32_t M = p.st->fx_items;
    const uint32_t C = p.chunk;
    const uint32_t nchunks = (M + C - 1) / C;
    const bool lane_on = (uint32_t)(lane * VPL) < p.dpad;
    const AdamStep as = AdamStep::load_fx(p.st);
    unsigned long long u_cnt = 0;
    for (uint32_t c = gw; c < nchunks; c += nw) {
        const uint32_t fl = p.carry_flags[c];
        if (!(fl & CF_OWNER)) continue;                 // warp-uniform
        const uint32_t f = p.carry_f[c];
        if constexpr (MODE == OUT_ADAM && sizeof(T) != 8) {
            if (lane == 0) prefetch_row_state<T>(p, f);
        }
        if (span_is_long(p, c, f, M, C)) continue;      // k_fixup_long's
        const uint32_t last = owner_last(p, c, f, M, C, lane);
        A acc[VPL];
        if (lane_on) RowIO<A, VPL>::load_cg((const A*)p.carry_tail + (uint64_t)c * p.dpad, lane, acc);
        else {
#pragma unroll
            for (int k = 0; k < VPL; ++k) acc[k] = 0;
        }
        uint32_t kept = fl & CF_TAIL_KEPT;
        for (uint32_t j = c + 1; j <= last; j += 4) {
            A h[4][VPL];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                if (j + u <= last) {
                    kept |= p.carry_flags[j + u] & CF_HEAD_KEPT;
                    if (lane_on) RowIO<A, VPL>::load_cg((const A*)p.carry_head + (uint64_t)(j + u) * p.dpad, lane, h[u]);
                }
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                if (j + u <= last && lane_on) {
#pragma unroll
                    for (int k = 0; k < VPL; ++k) acc[k] += h[u][k];
                }
            }
        }
        if (kept) {
            uint32_t none = 0;
            finish_row<T, A, VPL, MODE>(p, f, acc, lane, lane_on, as, nullptr, none);
            ++u_cnt;
        }
    }
    if (lane == 0 && u_cnt) atomicAdd(&p.st->unique_rows, u_cnt);
}

// k_fixup_long: one CTA of NWARP warps per long span that k_reduce queued
// (its owner chunk c; warp 0 finds the span's last chunk).  Warp w adds
// the heads of chunks c+1+w, c+1+w+NWARP, ... in increasing order; warp 0 then
// adds the owner's tail and the NWARP warp sums in warp order: a fixed order,
// independent of timing and of the queue order.
template <typename T, typename A, int VPL, int MODE>
__global__ void __launch_bounds__(fixl_threads(VPL)) k_fixup_long(ReduceParams p) {
    pdl_wait();
    pdl_trigger();
    constexpr int NWARP = fixl_threads(VPL) / 32;
    extern __shared__ __align__(16) unsigned char fixl_smem[];
    A* wsum = reinterpret_cast<A*>(fixl_smem);          // [NWARP][dpad]
    __shared__ uint32_t s_kept;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const AdamStep as = AdamStep::load_fx(p.st);
    const uint32_t par = as.step & 1u;
    const uint32_t n_long = p.st->n_long[par];
    const uint32_t* long_list = p.long_list + (size_t)par * p.long_cap;
    const uint32_t M = p.st->fx_items, C = p.chunk;
    __shared__ uint32_t s_last;
    const bool lane_on = (uint32_t)(lane * VPL) < p.dpad;
    unsigned long long u_cnt = 0;
    for (uint32_t q = blockIdx.x; q < n_long; q += gridDim.x) {
        const uint32_t c = long_list[q];
        const uint32_t fl = p.carry_flags[c];
        const uint32_t f = p.carry_f[c];
        if (w == 0) {
            const uint32_t l = owner_last(p, c, f, M, C, lane);
            if (lane == 0) s_last = l;
        }
        if (threadIdx.x == 0) s_kept = 0;
        __syncthreads();
        const uint32_t last = s_last;
        A acc[VPL];
#pragma unroll
        for (int k = 0; k < VPL; ++k) acc[k] = 0;
        uint32_t kept = 0;
        // FL head rows in flight per warp
        constexpr int FL = sizeof(A) == 8 ? 4 : 8;
        for (uint32_t j = c + 1 + w; j <= last; j += FL * NWARP) {
            A h[FL][VPL];
#pragma unroll
            for (int u = 0; u < FL; ++u) {
                const uint32_t jj = j + u * NWARP;
                if (jj <= last) {
                    kept |= p.carry_flags[jj] & CF_HEAD_KEPT;
                    if (lane_on) RowIO<A, VPL>::load_cg((const A*)p.carry_head + (uint64_t)jj * p.dpad, lane, h[u]);
                }
            }
#pragma unroll
            for (int u = 0; u < FL; ++u) {
                if (j + u * NWARP <= last && lane_on) {
#pragma unroll
                    for (int k = 0; k < VPL; ++k) acc[k] += h[u][k];
                }
            }
        }
        if (lane_on) store_row<A, VPL, A>(wsum + (size_t)w * p.dpad, lane, acc);
        if (lane == 0 && kept) atomicOr(&s_kept, 1u);
        __syncthreads();
        if (w == 0) {
            A tot[VPL];
            if (lane_on) RowIO<A, VPL>::load_cg((const A*)p.carry_tail + (uint64_t)c * p.dpad, lane, tot);
            else {
#pragma unroll
                for (int k = 0; k < VPL; ++k) tot[k] = 0;
            }
            for (int ww = 0; ww < NWARP; ++ww) {
                if (lane_on) {
#pragma unroll
                    for (int k = 0; k < VPL; ++k) tot[k] += wsum[(size_t)ww * p.dpad + lane * VPL + k];
                }
            }
            if ((fl & CF_TAIL_KEPT) || s_kept) {
                uint32_t none = 0;
                finish_row<T, A, VPL, MODE>(p, f, tot, lane, lane_on, as, nullptr, none);
                ++u_cnt;
            }
        }
        __syncthreads();
    }
    if (threadIdx.x == 0 && u_cnt) atomicAdd(&p.st->unique_rows, u_cnt);
}

// Adam over the touched list, reading the dense gradient rows (PLAIN form,
// and the FUSED form's split reduction).  Two rows per warp iteration, with
// all eight row loads (g, m, v, table for each) issued before any is used.
template <typename T, int VPL>
__global__ void __launch_bounds__(RED_THREADS) k_adam_dense(BatchState* st, T* table, float* m, float* v,
                                                            const float* g, const uint32_t* touched,
                                                            const uint32_t* n_touched, uint32_t dpad, uint64_t seed) {
    pdl_wait();
    pdl_trigger();
    const int lane = threadIdx.x & 31;
    const uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    const uint32_t n = *n_touched;
    const bool lane_on = (uint32_t)(lane * VPL) < dpad;
    const AdamStep as = AdamStep::load_fx(st);
    for (uint32_t r0 = 2 * gw; r0 < n; r0 += 2 * nw) {
        uint32_t f[2];
        bool on[2];
        float gg[2][VPL], mm[2][VPL], vv[2][VPL], ee[2][VPL];
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            on[u] = r0 + u < n;
            f[u] = on[u] ? touched[r0 + u] : 0u;
        }
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            if (on[u] && lane_on) {
                const uint64_t o = (uint64_t)f[u] * dpad;
                RowIO<float, VPL>::load_cg(g + o, lane, gg[u]);
                RowIO<float, VPL>::load_cg(m + o, lane, mm[u]);
                RowIO<float, VPL>::load_cg(v + o, lane, vv[u]);
                RowIO<T, VPL>::load_cg(table + o, lane, ee[u]);
            } else {
#pragma unroll
                for (int k = 0; k < VPL; ++k) gg[u][k] = mm[u][k] = vv[u][k] = ee[u][k] = 0.f;
            }
        }
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            bool bad = false;
#pragma unroll
            for (int k = 0; k < VPL; ++k) bad = bad || (gg[u][k] != gg[u][k]);
            if (on[u] && !__any_sync(FULL, bad) && lane_on)
                adam_apply<T, VPL>(table, m, v, f[u], dpad, gg[u], mm[u], vv[u], ee[u], as, seed, lane);
        }
    }
}

// Self-check of the stochastic-rounding conversion against the bit rule it
// replaces: element pairs from a hash of (seed, i), with exponents across the
// whole FP32 range and every 16th pair drawn from special values (zeros,
// infinities, NaNs, subnormals, the largest finite values, values one ulp
// below a BF16 carry), rounded both ways with the same random bits.
__global__ void k_sr_selftest(uint64_t n, uint64_t seed, unsigned long long* mismatches) {
    const uint32_t specials[12] = {0x00000000u, 0x80000000u, 0x7f800000u, 0xff800000u, 0x7fc00000u, 0xffc00001u,
                                   0x00000001u, 0x807fffffu, 0x7f7fffffu, 0xff7fffffu, 0x3f80ffffu, 0xbf7fffffu};
    unsigned long long bad = 0;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t k = (uint32_t)seed ^ (uint32_t)(seed >> 32);
        const uint32_t h0 = mix32(k ^ mix32((uint32_t)i * 3u + 0x9E3779B1u) ^ (uint32_t)(i >> 32));
        const uint32_t h1 = mix32(h0 ^ 0x85EBCA77u), h2 = mix32(h1 ^ 0xC2B2AE3Du), r = mix32(h2 ^ 0x27D4EB2Fu);
        uint32_t a = h1, b = h2;
        if ((i & 15u) == 0) {
            a = specials[h1 % 12u];
            b = specials[h2 % 12u];
        }
        const float lo = __uint_as_float(a), hi = __uint_as_float(b);
        const uint32_t hw = bf16x2_stochastic(lo, hi, r);
        const uint32_t sw = (uint32_t)__bfloat16_as_ushort(bf16_stochastic(lo, r & 0xffffu)) |
                            ((uint32_t)__bfloat16_as_ushort(bf16_stochastic(hi, r >> 16)) << 16);
        bad += hw != sw;
    }
    bad = warp_sum<unsigned long long>(bad);
    if ((threadIdx.x & 31) == 0 && bad) atomicAdd(mismatches, bad);
}

extern "C" int ep_selftest_stochastic_rounding(int device, uint64_t n, uint64_t seed, uint64_t* mismatches) {
    if (!mismatches) return EP_ERR_INVALID_ARG;
    if (cudaSetDevice(device) != cudaSuccess) return EP_ERR_CUDA;
    unsigned long long* d = nullptr;
    if (cudaMalloc(&d, sizeof(*d)) != cudaSuccess) return EP_ERR_OOM;
    cudaError_t e = cudaMemset(d, 0, sizeof(*d));
    if (e == cudaSuccess) {
        k_sr_selftest<<<152 * 4, 256>>>(n, seed, d);
        e = cudaGetLastError();
    }
    unsigned long long h = 0;
    if (e == cudaSuccess) e = cudaMemcpy(&h, d, sizeof(h), cudaMemcpyDeviceToHost);
    cudaFree(d);
    *mismatches = h;
    return e == cudaSuccess ? EP_OK : EP_ERR_CUDA;
}

// OUT_QUEUE: the slots and their feature ids, then the per-warp item lists.
template <typename T, typename A>
static size_t queue_smem(uint32_t dpad) {
    return queue_list_offset<T>(dpad, QUEUE_THREADS / 32) + (size_t)(QUEUE_THREADS / 32) * list_bytes<A>();
}

template <typename T, typename A, int VPL>
static void red_launch(const ReduceParams& p, uint64_t cap, cudaStream_t s, int which) {
    const uint32_t nch = reduce_chunks(cap, p.chunk);
    const uint32_t warps = nch ? nch : 1;
    if (which == 0) {
        uint32_t ctas = (warps + RED_THREADS / 32 - 1) / (RED_THREADS / 32);
        if (ctas > RED_MAX_CTAS) ctas = RED_MAX_CTAS;
        if (p.red_ctas) ctas = std::min<uint32_t>(ctas, p.red_ctas);
        const size_t lists = (size_t)(RED_THREADS / 32) * list_bytes<A>();
        if (p.out_mode == OUT_DENSE) launch_chain(k_reduce<T, A, VPL, OUT_DENSE>, ctas, RED_THREADS, lists, s, p);
        else if (p.out_mode == OUT_QUEUE) {
            uint32_t qctas = (warps + QUEUE_THREADS / 32 - 1) / (QUEUE_THREADS / 32);
            if (qctas > 2 * RED_MAX_CTAS) qctas = 2 * RED_MAX_CTAS;
            if (p.red_ctas) qctas = std::min(qctas, p.red_ctas);
            bool q5 = false;
            if constexpr (VPL <= 8) {
                if (p.queue_ctas_per_sm >= 5) {
                    launch_chain(k_reduce_q5<T, A, VPL>, qctas, QUEUE_THREADS, queue_smem<T, A>(p.dpad), s, p);
                    q5 = true;
                }
            }
            if (!q5) launch_chain(k_reduce<T, A, VPL, OUT_QUEUE>, qctas, QUEUE_THREADS, queue_smem<T, A>(p.dpad), s, p);
        } else if (p.out_mode == OUT_RING) {
            if constexpr (sizeof(T) != 8) {
                // persistent: every CTA resident at once (one per SM at 16 warps)
                const uint32_t threads = 32 * (p.ring_pw + p.ring_cw);
                const size_t smem = ring_hdr_bytes() + (size_t)p.ring_slots * ring_slot_bytes<T>(p.dpad) +
                                    (size_t)p.ring_pw * list_bytes<A>();
                uint32_t per_sm = 65536u / (threads * 128u);
                const uint32_t by_smem = (uint32_t)((227u * 1024u) / (smem + 1024u));
                if (by_smem < per_sm) per_sm = by_smem;
                if (per_sm < 1) per_sm = 1;
                uint32_t rctas = (warps + p.ring_pw - 1) / p.ring_pw;
                if (rctas > 152 * per_sm) rctas = 152 * per_sm;
                launch_chain(k_reduce<T, A, VPL, OUT_RING>, rctas, threads, smem, s, p);
            }
        }
        else launch_chain(k_reduce<T, A, VPL, OUT_ADAM>, ctas, RED_THREADS, lists, s, p);
    } else {
        uint32_t ctas = std::min<uint32_t>((warps + FIX_THREADS / 32 - 1) / (FIX_THREADS / 32), 152 * 16);
        constexpr int LT = fixl_threads(VPL);
        const size_t lsmem = (size_t)(LT / 32) * p.dpad * sizeof(A);
        // which: 1 both kernels, 2 the short spans, 3 the long spans
        const bool shorts = which != 3, longs = which != 2;
        if (p.out_mode == OUT_DENSE) {
            if (shorts) launch_chain(k_fixup<T, A, VPL, OUT_DENSE>, ctas, FIX_THREADS, 0, s, p);
            if (longs) launch_chain(k_fixup_long<T, A, VPL, OUT_DENSE>, 152, LT, lsmem, s, p);
        } else {
            if (shorts) launch_chain(k_fixup<T, A, VPL, OUT_ADAM>, ctas, FIX_THREADS, 0, s, p);
            if (longs) launch_chain(k_fixup_long<T, A, VPL, OUT_ADAM>, 152, LT, lsmem, s, p);
        }
    }
}

template <typename T, typename A, int VPL>
static cudaError_t fixl_setup() {
    const int bytes = (fixl_threads(VPL) / 32) * VPL * 32 * (int)sizeof(A);
    cudaError_t e = cudaFuncSetAttribute(k_fixup_long<T, A, VPL, OUT_DENSE>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_fixup_long<T, A, VPL, OUT_ADAM>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_reduce<T, A, VPL, OUT_QUEUE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)queue_smem<T, A>(VPL * 32));
    if constexpr (VPL <= 8) {
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(k_reduce_q5<T, A, VPL>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)queue_smem<T, A>(VPL * 32));
    }
    if constexpr (sizeof(T) != 8) {
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(k_reduce<T, A, VPL, OUT_RING>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     227 * 1024);
    }
    return e;
}

bool ring_supported(int tt, uint32_t dpad, uint32_t pw, uint32_t cw, uint32_t slots) {
    if (tt == TT_F64 || pw < 1 || cw < 1 || pw + cw > RING_MAX_WARPS || slots < 2 || slots > RING_MAX_SLOTS)
        return false;
    if (slots % cw) return false;   // each Adam warp owns whole slots (exact parity waits)
    const uint32_t es = tt == TT_BF16 ? 2u : 4u;
    if ((dpad * 4u) % 16u || (dpad * es) % 16u) return false;   // bulk copies move 16-byte multiples
    return ring_smem_bytes(tt, dpad, pw, slots) <= 227u * 1024u;
}

size_t ring_smem_bytes(int tt, uint32_t dpad, uint32_t pw, uint32_t slots) {
    return ring_hdr_bytes() + (size_t)pw * list_bytes<float>() +
           (size_t)slots * (tt == TT_BF16 ? ring_slot_bytes<__nv_bfloat16>(dpad) : ring_slot_bytes<float>(dpad));
}

template <typename T, typename A>
static cudaError_t fixl_setup_all() {
    cudaError_t e = cudaSuccess;
    const cudaError_t r[5] = {fixl_setup<T, A, 1>(), fixl_setup<T, A, 2>(), fixl_setup<T, A, 4>(),
                              fixl_setup<T, A, 8>(), fixl_setup<T, A, 16>()};
    for (cudaError_t x : r)
        if (x != cudaSuccess) e = x;
    return e;
}

// Opts the long-span fixup kernels in to their dynamic shared memory (one row
// per warp, up to 64 KB); called at context creation, outside any capture.
// Once per device (the current one): later contexts on it skip the calls.
cudaError_t reduce_kernels_setup() {
    static std::mutex mu;
    static bool done[256] = {};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lk(mu);
    if (dev >= 0 && dev < 256 && done[dev]) return cudaSuccess;
    e = fixl_setup_all<float, float>();
    const cudaError_t b = fixl_setup_all<__nv_bfloat16, float>();
    const cudaError_t d = fixl_setup_all<double, double>();
    e = e != cudaSuccess ? e : (b != cudaSuccess ? b : d);
    if (e == cudaSuccess && dev >= 0 && dev < 256) done[dev] = true;
    return e;
}

template <typename T, typename A>
static void red_dispatch(int vpl, const ReduceParams& p, uint64_t cap, cudaStream_t s, int which) {
    switch (vpl) {
        case 1: red_launch<T, A, 1>(p, cap, s, which); break;
        case 2: red_launch<T, A, 2>(p, cap, s, which); break;
        case 4: red_launch<T, A, 4>(p, cap, s, which); break;
        case 8: red_launch<T, A, 8>(p, cap, s, which); break;
        default: red_launch<T, A, 16>(p, cap, s, which); break;
    }
}

static void reduce_or_fixup(int tt, int vpl, const ReduceParams& p, uint64_t cap, cudaStream_t s, int which) {
    if (tt == TT_F32) red_dispatch<float, float>(vpl, p, cap, s, which);
    else if (tt == TT_BF16) red_dispatch<__nv_bfloat16, float>(vpl, p, cap, s, which);
    else red_dispatch<double, double>(vpl, p, cap, s, which);
}

void launch_reduce(int tt, int vpl, const ReduceParams& p, uint64_t cap, cudaStream_t s) {
    reduce_or_fixup(tt, vpl, p, cap, s, 0);
}

void launch_fixup(int tt, int vpl, const ReduceParams& p, uint64_t cap, cudaStream_t s, int part) {
    reduce_or_fixup(tt, vpl, p, cap, s, part == 1 ? 2 : (part == 2 ? 3 : 1));
}

template <typename T>
static void adam_dispatch(int vpl, BatchState* st, T* table, float* m, float* v, const float* g,
                          const uint32_t* touched, const uint32_t* n_touched, uint32_t dpad, uint32_t max_rows,
                          uint64_t seed, cudaStream_t s) {
    uint32_t ctas = (max_rows + RED_THREADS / 32 - 1) / (RED_THREADS / 32);
    if (ctas > RED_MAX_CTAS) ctas = RED_MAX_CTAS;
    if (ctas == 0) ctas = 1;
    switch (vpl) {
        case 1: launch_chain(k_adam_dense<T, 1>, ctas, RED_THREADS, 0, s, st, table, m, v, g, touched, n_touched, dpad, seed); break;
        case 2: launch_chain(k_adam_dense<T, 2>, ctas, RED_THREADS, 0, s, st, table, m, v, g, touched, n_touched, dpad, seed); break;
        case 4: launch_chain(k_adam_dense<T, 4>, ctas, RED_THREADS, 0, s, st, table, m, v, g, touched, n_touched, dpad, seed); break;
        case 8: launch_chain(k_adam_dense<T, 8>, ctas, RED_THREADS, 0, s, st, table, m, v, g, touched, n_touched, dpad, seed); break;
        default: launch_chain(k_adam_dense<T, 16>, ctas, RED_THREADS, 0, s, st, table, m, v, g, touched, n_touched, dpad, seed); break;
    }
}

void launch_adam_dense(int tt, int vpl, BatchState* st, void* table, float* m, float* v, const float* g,
                       const uint32_t* touched, const uint32_t* n_touched, uint32_t dpad, uint32_t max_rows,
                       uint64_t seed, cudaStream_t s) {
    if (tt == TT_F32) adam_dispatch<float>(vpl, st, (float*)table, m, v, g, touched, n_touched, dpad, max_rows, seed, s);
    else if (tt == TT_BF16)
        adam_dispatch<__nv_bfloat16>(vpl, st, (__nv_bfloat16*)table, m, v, g, touched, n_touched, dpad, max_rows, seed, s);
}

// Packs touched rows of a padded dense buffer into out[r * dims] (scatter=0),
// or writes them back into a dense [n_feat x dims] buffer (scatter=1).
template <typename E>
__global__ void k_pack_rows(const E* dense, const uint32_t* rows, const uint32_t* n_rows, uint32_t dpad,
                            uint32_t dims, E* out, int scatter) {
    const uint32_t n = *n_rows;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < (uint64_t)n * dims;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t r = (uint32_t)(i / dims), k = (uint32_t)(i % dims);
        const uint32_t f = rows[r];
        if (scatter) out[(uint64_t)f * dims + k] = dense[(uint64_t)f * dpad + k];
        else out[i] = dense[(uint64_t)f * dpad + k];
    }
}

void launch_pack_rows(size_t es, const void* dense, const uint32_t* rows, const uint32_t* n_rows, uint32_t dpad,
                      uint32_t dims, void* out, int scatter, uint32_t max_rows, cudaStream_t s) {
    uint64_t total = (uint64_t)max_rows * dims;
    unsigned blocks = (unsigned)std::min<uint64_t>((total + 255) / 256, 152 * 16);
    if (!blocks) blocks = 1;
    if (es == 8) k_pack_rows<double><<<blocks, 256, 0, s>>>((const double*)dense, rows, n_rows, dpad, dims, (double*)out, scatter);
    else k_pack_rows<float><<<blocks, 256, 0, s>>>((const float*)dense, rows, n_rows, dpad, dims, (float*)out, scatter);
}

}  // namespace ep
