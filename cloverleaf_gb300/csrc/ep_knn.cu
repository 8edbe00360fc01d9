// ep_knn.cu -- node embeddings from feature embeddings and exact cosine
// top-k on the GPU (the evaluation side of the path).
//
//   ep_embed_features  NodeEmbedder.embed_feature_set (src/lib.rs:2092-2124)
//                      with AvgAggregator / WeightedAggregator
//                      (src/algos/aggregator.rs:17-120): warp per node.
//   ep_align           NeighborhoodAligner.align (src/algos/alignment.rs,
//                      src/lib.rs:3040-3110): warp per node.
//   ep_knn_cosine      NodeEmbeddings.nearest_neighbor for many queries at
//                      once (src/embeddings.rs:149-173, cosine distance):
//                      rows normalised to BF16, then a tcgen05 GEMM (FP32
//                      accumulation in tensor memory) fused with a per-query
//                      top-k that never leaves registers.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/ep_gb300.h"
#include "ep_device.cuh"

namespace ep {
namespace {

thread_local std::string g_knn_err;
thread_local float g_knn_ms = 0.f;     // CUDA-event time of the last top-k or alignment kernel

int knn_fail(int code, const char* msg) {
    g_knn_err = msg;
    return code;
}
int knn_cuda_fail(cudaError_t e, const char* what) {
    cudaGetLastError();
    g_knn_err = std::string(what) + ": " + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? EP_ERR_OOM : EP_ERR_CUDA;
}

#define KCK(call, what)                                 \
    do {                                                \
        cudaError_t e_ = (call);                        \
        if (e_ != cudaSuccess) return knn_cuda_fail(e_, what); \
    } while (0)

struct DevMem {
    void* p = nullptr;
    ~DevMem() { if (p) cudaFree(p); }
    cudaError_t alloc(size_t n) { return cudaMalloc(&p, n ? n : 16); }
};

// ---------------------------------------------------------------------------
// Node embeddings: out[v] = sum_f w_f E[f] / sum_f w_f over v's features in
// CSR order, f32 as the reference (w_f * e rounded, then added; the weights
// summed in f32); nodes without features stay zero.  Up to 16 elements per
// lane (dims <= 512).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_embed(uint64_t n, const uint64_t* __restrict__ fptr,
                                               const uint32_t* __restrict__ fids, const float* __restrict__ fw,
                                               uint32_t d, const float* __restrict__ table, float* __restrict__ out) {
    const int lane = threadIdx.x & 31;
    const uint64_t v = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (v >= n) return;
    float acc[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) acc[i] = 0.f;
    float wsum = 0.f;
    const uint64_t b = fptr[v], e = fptr[v + 1];
    for (uint64_t j = b; j < e; ++j) {
        const uint32_t f = fids[j];
        const float w = fw ? fw[f] : 1.f;
        wsum += w;
        const float* row = table + (uint64_t)f * d;
#pragma unroll
        for (int i = 0; i < 16; ++i) {
            const uint32_t k = (uint32_t)lane + 32u * i;
            if (k < d) acc[i] = __fadd_rn(acc[i], fw ? __fmul_rn(w, row[k]) : row[k]);
        }
    }
#pragma unroll
    for (int i = 0; i < 16; ++i) {
        const uint32_t k = (uint32_t)lane + 32u * i;
        if (k < d) out[v * d + k] = e > b ? acc[i] / wsum : 0.f;
    }
}

// ---------------------------------------------------------------------------
// Neighbourhood alignment (NeighborhoodAligner.align, src/algos/alignment.rs:
// 25-75): out[v] = (1 - a) * sum_j p_j E[u_j] + a * E[v] over the first
// min(deg, kmax) edges in CSR order, p_j the edge probability recovered from
// the CDF weights (w_0, w_j - w_{j-1}), a = alpha, or min(1, 1 / ln(deg + 1))
// when alpha < 0.  f32 as the reference: every product rounded, then added,
// per element in edge order.  Warp per node, up to 16 elements per lane.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_align(uint64_t n, const uint64_t* __restrict__ rp,
                                               const uint32_t* __restrict__ cols, const float* __restrict__ cdf,
                                               uint32_t d, const float* __restrict__ E, float alpha, uint64_t kmax,
                                               float* __restrict__ out) {
    const int lane = threadIdx.x & 31;
    const uint64_t v = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (v >= n) return;
    float acc[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) acc[i] = 0.f;
    const uint64_t b = rp[v], deg = rp[v + 1] - b;
    const uint64_t m = deg < kmax ? deg : kmax;
    for (uint64_t j = 0; j < m; ++j) {
        const float p = j ? __fsub_rn(cdf[b + j], cdf[b + j - 1]) : cdf[b];
        const float* row = E + (uint64_t)cols[b + j] * d;
#pragma unroll
        for (int i = 0; i < 16; ++i) {
            const uint32_t k = (uint32_t)lane + 32u * i;
            if (k < d) acc[i] = __fadd_rn(acc[i], __fmul_rn(p, row[k]));
        }
    }
    const float a = alpha >= 0.f ? alpha : fminf(__fdiv_rn(1.f, logf(__fadd_rn((float)deg, 1.f))), 1.f);
    const float c = __fsub_rn(1.f, a);
    const float* own = E + v * d;
#pragma unroll
    for (int i = 0; i < 16; ++i) {
        const uint32_t k = (uint32_t)lane + 32u * i;
        if (k < d) out[v * d + k] = __fadd_rn(__fmul_rn(acc[i], c), __fmul_rn(own[k], a));
    }
}

// Rows scaled to unit L2 norm (zero rows stay zero), rounded to BF16 and
// written straight into the tile image the tensor core reads (see below):
// tiles of 2^tlog rows; per tile, per 64-element K block, 8-row atoms of
// 1024 B in which the 16-byte chunk c of row r sits at chunk c ^ (r % 8).
// Rows from n up to the tile boundary are written as zeros.
__device__ __forceinline__ uint64_t swz_offset(uint64_t row, uint32_t k, uint32_t nkb, uint32_t tlog) {
    const uint64_t tile = row >> tlog;
    const uint32_t r = (uint32_t)row & ((1u << tlog) - 1u), kb = k >> 6, c = (k & 63u) >> 3, e = k & 7u;
    const uint64_t kb_bytes = (uint64_t)128u << tlog;
    return tile * nkb * kb_bytes + kb * kb_bytes + (r >> 3) * 1024u + (r & 7u) * 128u + ((c ^ (r & 7u)) << 4) + e * 2u;
}

__global__ void __launch_bounds__(256) k_norm_swz(uint64_t n, uint64_t n_tiled, uint32_t d, uint32_t dpad,
                                                  uint32_t tlog, const float* __restrict__ x,
                                                  unsigned char* __restrict__ y) {
    const int lane = threadIdx.x & 31;
    const uint64_t r = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (r >= n_tiled) return;
    const bool in = r < n;
    float ss = 0.f;
    if (in)
        for (uint32_t k = lane; k < d; k += 32) {
            const float t = x[r * d + k];
            ss += t * t;
        }
    ss = warp_sum<float>(ss);
    const float inv = ss > 0.f ? 1.f / sqrtf(ss) : 0.f;
    const uint32_t nkb = dpad / 64;
    for (uint32_t k = lane; k < dpad; k += 32) {
        const float v = (in && k < d) ? x[r * d + k] * inv : 0.f;
        *reinterpret_cast<__nv_bfloat16*>(y + swz_offset(r, k, nkb, tlog)) = __float2bfloat16_rn(v);
    }
}

// ---------------------------------------------------------------------------
// Cosine top-k: one CTA per 128 queries, warp-specialised.
//
// Copy warp: copies the query tile (M = 128 rows, all of K) once, then
// streams the database through KNN_STAGES shared-memory stages, one stage
// per 64-element K block of a 256-row tile, with cp.async.bulk from the tile
// images (completion counted in bytes on mbarriers).  A stage is refilled
// once the MMAs that read it have completed.
// MMA warp: per database tile, once its accumulator is free, lane 0 issues
// 4 MMAs per K block (M = 128, N = 256, K = 16; BF16 x BF16 -> FP32) into one
// of two 256-column accumulators in tensor memory, frees each stage through
// a commit, and signals the finished tile through another.  Both loops run
// warp-uniform; the MMA descriptors are built once and advanced by adds.
// Epilogue warps: warp w reads TMEM lane quarter w % 4 (lane = query row)
// and the column slice w / 4 of each tile, 32 columns per load, then
// releases the accumulator.  Each thread keeps a sorted top-KMAX of its
// columns in registers and admits a value only above its k-th best so far,
// skipping blocks of 16 or 32 values whose maximum cannot enter; the slices'
// lists are merged per query at the end.  Operands sit in shared memory as K-major,
// 128-byte-swizzled tiles.
// All waits are bounded; a timeout sets an abort flag that ends every role's
// loop, the copies and MMAs still in flight are waited for, and the error
// word is set.
// ---------------------------------------------------------------------------
constexpr int KNN_BM = 128, KNN_BN = 256, KNN_STAGES = 4, KNN_ACC = 2;
constexpr uint32_t KNN_A_KB = KNN_BM * 128u, KNN_B_KB = KNN_BN * 128u;   // bytes per 64-element K block
constexpr uint32_t KNN_TMEM_COLS = KNN_BN * KNN_ACC;                     // 512: all of tensor memory
constexpr uint32_t KNN_WAIT_LIMIT = 1u << 22;    // mbarrier polls (32 ns sleeps) before giving up
enum : uint32_t { KNN_ERR_TIMEOUT = 1u };

// This warp's TMEM lane quarter, columns taddr .. taddr + N - 1 (one 32-bit
// value per column) into r, and the largest of the thread's N values in mx:
// the reducing TMEM load of sm_103a, so that a block's skip test costs no
// instructions.  The caller waits for the load.
__device__ __forceinline__ void tmem_ld_max(uint32_t taddr, uint32_t (&r)[32], float& mx) {
    asm volatile(
        "tcgen05.ld.red.sync.aligned.32x32b.x32.max.f32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, %32, [%33];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]),
          "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]),
          "=r"(r[30]), "=r"(r[31]), "=f"(mx)
        : "r"(taddr)
        : "memory");
}
__device__ __forceinline__ void tmem_ld_max(uint32_t taddr, uint32_t (&r)[16], float& mx) {
    asm volatile(
        "tcgen05.ld.red.sync.aligned.32x32b.x16.max.f32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
        "%16, [%17];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=f"(mx)
        : "r"(taddr)
        : "memory");
}

// Epilogue shape per list length, within the register file: 16 warps (4
// column slices of 64, loaded 16 columns at a time) for KMAX <= 16; 8 warps
// (2 slices of 128, 32 at a time) for KMAX 32.
template <int KMAX>
struct KnnRoles {
    static constexpr int EPI = KMAX <= 16 ? 16 : 8;
    static constexpr int BW = KMAX <= 16 ? 16 : 32;    // columns per TMEM load and per skip test
    static constexpr int SLICES = EPI / 4, CW = KNN_BN / SLICES, BLOCKS = CW / BW;
    static constexpr int COPY = EPI, MMA = EPI + 1, THREADS = 32 * (EPI + 2);
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// K-major, 128-byte swizzle, version 1; SBO = 1024 B between 8-row atoms.
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3fffu);          // start address
    d |= (uint64_t)1u << 16;                           // leading byte offset (unused when swizzled)
    d |= (uint64_t)(1024u >> 4) << 32;                 // stride byte offset
    d |= (uint64_t)1u << 46;                           // descriptor version
    d |= (uint64_t)2u << 61;                           // 128-byte swizzle
    return d;
}

// kind::f16 instruction descriptor: BF16 A and B (K-major), FP32 D, M x N.
__host__ __device__ constexpr uint32_t umma_idesc(uint32_t M, uint32_t N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((N >> 3) << 17) | ((M >> 4) << 24);
}

__device__ __forceinline__ void mbar_init(uint64_t* m, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(m)), "r"(count) : "memory");
}

// Polls the mbarrier for the completion of the phase with the given parity:
// at most KNN_WAIT_LIMIT polls, 32 ns apart, and none once *abort is set.
// Returns 1 when the phase completed.
__device__ __forceinline__ uint32_t mbar_wait(uint64_t* mbar, uint32_t parity, volatile uint32_t* abort) {
    uint32_t done = 0;
    for (uint32_t it = 0; it < KNN_WAIT_LIMIT; ++it) {
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
            : "=r"(done)
            : "r"(smem_u32(mbar)), "r"(parity)
            : "memory");
        if (done || *abort) break;
        __nanosleep(32);
    }
    return done;
}

__device__ __forceinline__ void mbar_arrive(uint64_t* mbar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(mbar)) : "memory");
}

// One thread: `pieces` bulk copies of `bytes` each, from src + i * src_stride
// to dst + i * bytes, all counted on mbar.
__device__ __forceinline__ void bulk_load(unsigned char* dst, const unsigned char* src, uint32_t pieces,
                                          uint32_t bytes, uint64_t src_stride, uint64_t* mbar) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(mbar)), "r"(pieces * bytes)
                 : "memory");
    for (uint32_t i = 0; i < pieces; ++i)
        asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                         smem_u32(dst + i * bytes)),
                     "l"(src + i * src_stride), "r"(bytes), "r"(smem_u32(mbar))
                     : "memory");
}

// The 4 MMAs of one K block (K = 64) into the accumulator at tmem_d.  Every
// lane of the (converged) MMA warp runs this; the instructions are predicated
// on `leader`, so one thread issues them.  ad / bd: descriptors of the
// block; a K step of 16 elements moves the start address by 32 B.
__device__ __forceinline__ void issue_kblock_mma(uint64_t ad, uint64_t bd, uint32_t tmem_d, bool first,
                                                 uint32_t leader) {
    constexpr uint32_t idesc = umma_idesc(KNN_BM, KNN_BN);
#pragma unroll
    for (uint32_t s = 0; s < 4; ++s) {
        const uint32_t acc = (!first || s) ? 1u : 0u;
        asm volatile(
            "{\n .reg .pred p, l;\n setp.ne.b32 p, %4, 0;\n setp.ne.b32 l, %5, 0;\n"
            " @l tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(tmem_d),
            "l"(ad + s * 2u), "l"(bd + s * 2u), "r"(idesc), "r"(acc), "r"(leader)
            : "memory");
    }
}

// Arrives on mbar once every MMA this thread issued so far has completed.
__device__ __forceinline__ void mma_commit(uint64_t* mbar, uint32_t leader) {
    asm volatile(
        "{\n .reg .pred l;\n setp.ne.b32 l, %1, 0;\n"
        " @l tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n}" ::"r"(smem_u32(mbar)),
        "r"(leader)
        : "memory");
}

template <int KMAX>
__device__ __forceinline__ void topk_push(float (&vals)[KMAX], uint32_t (&ids)[KMAX], float v, uint32_t id) {
    vals[KMAX - 1] = v;
    ids[KMAX - 1] = id;
#pragma unroll
    for (int i = KMAX - 1; i >= 1; --i) {
        if (vals[i] > vals[i - 1]) {
            const float tv = vals[i];
            vals[i] = vals[i - 1];
            vals[i - 1] = tv;
            const uint32_t ti = ids[i];
            ids[i] = ids[i - 1];
            ids[i - 1] = ti;
        }
    }
}

// k-th largest of a list sorted in descending order (k in [1, KMAX]): the
// minimum of its first k entries, written so that the registers are never
// indexed at run time
template <int KMAX>
__device__ __forceinline__ float kth_value(const float (&vals)[KMAX], uint32_t k) {
    float t = vals[0];
#pragma unroll
    for (int i = 1; i < KMAX; ++i) t = fminf(t, (uint32_t)i < k ? vals[i] : INFINITY);
    return t;
}

template <int KMAX>
__global__ void __launch_bounds__(KnnRoles<KMAX>::THREADS, 1)
    k_cos_topk(const unsigned char* __restrict__ Q, uint64_t nq, const unsigned char* __restrict__ D, uint64_t ndb,
               uint32_t dpad, const uint64_t* __restrict__ qself, uint32_t k, uint32_t* __restrict__ idx_out,
               float* __restrict__ sim_out, uint32_t* __restrict__ err) {
    using R = KnnRoles<KMAX>;
    extern __shared__ unsigned char knn_smem_raw[];
    __shared__ uint64_t bar_a, bar_full[KNN_STAGES], bar_empty[KNN_STAGES], bar_acc_full[KNN_ACC],
        bar_acc_free[KNN_ACC];
    __shared__ uint64_t s_loaded, s_landed, s_issued;    // stages copied / seen landed / stages whose MMAs issued
    __shared__ uint32_t tmem_slot, s_a_landed;
    __shared__ volatile uint32_t abort_flag;
    unsigned char* smem = (unsigned char*)(((uintptr_t)knn_smem_raw + 1023) & ~(uintptr_t)1023);
    const uint32_t nkb = dpad / 64;
    const uint32_t a_bytes = nkb * KNN_A_KB;
    unsigned char* sA = smem;
    auto sB = [&](uint32_t st) { return smem + a_bytes + st * KNN_B_KB; };
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint64_t ntiles = (ndb + KNN_BN - 1) / KNN_BN, nstages = ntiles * nkb;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                     "r"(KNN_TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (threadIdx.x == 0) {
        abort_flag = 0;
        s_loaded = s_landed = s_issued = 0;
        s_a_landed = 0;
        mbar_init(&bar_a, 1);
        for (int i = 0; i < KNN_STAGES; ++i) {
            mbar_init(&bar_full[i], 1);
            mbar_init(&bar_empty[i], 1);
        }
        for (int i = 0; i < KNN_ACC; ++i) {
            mbar_init(&bar_acc_full[i], 1);
            mbar_init(&bar_acc_free[i], R::EPI);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_slot;

    // per-thread top-k (epilogue warps)
    float vals[KMAX];
    uint32_t ids[KMAX];
#pragma unroll
    for (int i = 0; i < KMAX; ++i) { vals[i] = -INFINITY; ids[i] = 0xffffffffu; }
    const int quarter = warp & 3, slice = warp >> 2;
    const uint32_t qrow = 32u * quarter + lane;                 // TMEM lane = accumulator row = query
    const uint64_t myq = (uint64_t)blockIdx.x * KNN_BM + qrow;
    // column ids fit 32 bits (the host keeps n_db below 2^32 - 1); ~0 = no row to skip
    const uint32_t self = (warp < R::EPI && qself && myq < nq && qself[myq] < ndb) ? (uint32_t)qself[myq] : ~0u;
    const uint32_t ndb32 = (uint32_t)ndb;

    if (warp == R::COPY) {
        // ---- copies ----
        uint64_t loaded = 0;
        if (ntiles) {
            if (lane == 0) bulk_load(sA, Q + (uint64_t)blockIdx.x * a_bytes, nkb, KNN_A_KB, KNN_A_KB, &bar_a);
            for (uint64_t sg = 0; sg < nstages; ++sg) {
                const uint32_t st = (uint32_t)(sg % KNN_STAGES), use = (uint32_t)(sg / KNN_STAGES);
                // the stage is free once the MMAs of its previous K block completed
                if (sg >= (uint64_t)KNN_STAGES &&
                    !__all_sync(0xffffffffu, mbar_wait(&bar_empty[st], (use - 1u) & 1u, &abort_flag))) {
                    abort_flag = 1;
                    break;
                }
                if (lane == 0) bulk_load(sB(st), D + sg * KNN_B_KB, 2, KNN_B_KB / 2, KNN_B_KB / 2, &bar_full[st]);
                loaded = sg + 1;
            }
        }
        if (lane == 0) s_loaded = loaded;
    } else if (warp == R::MMA) {
        // ---- MMA issue ----
        uint64_t landed = 0, issued = 0;
        uint32_t a_ok = 0;
        if (ntiles) {
            const uint64_t ad0 = umma_desc(smem_u32(sA)), bd0 = umma_desc(smem_u32(sB(0)));
            bool ok = a_ok = __all_sync(0xffffffffu, mbar_wait(&bar_a, 0, &abort_flag));
            uint64_t sg = 0;
            for (uint64_t j = 0; ok && j < ntiles; ++j) {
                const uint32_t acc = (uint32_t)(j % KNN_ACC), ause = (uint32_t)(j / KNN_ACC);
                if (j >= (uint64_t)KNN_ACC &&
                    !__all_sync(0xffffffffu, mbar_wait(&bar_acc_free[acc], (ause - 1u) & 1u, &abort_flag))) {
                    ok = false;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                for (uint32_t kb = 0; kb < nkb; ++kb, ++sg) {
                    const uint32_t st = (uint32_t)(sg % KNN_STAGES), use = (uint32_t)(sg / KNN_STAGES);
                    if (!__all_sync(0xffffffffu, mbar_wait(&bar_full[st], use & 1u, &abort_flag))) {
                        ok = false;
                        break;
                    }
                    landed = sg + 1;
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                    issue_kblock_mma(ad0 + kb * (KNN_A_KB >> 4), bd0 + st * (KNN_B_KB >> 4), tmem + acc * KNN_BN,
                                     kb == 0, lane == 0);
                    mma_commit(&bar_empty[st], lane == 0);
                    issued = sg + 1;
                }
                if (!ok) break;
                mma_commit(&bar_acc_full[acc], lane == 0);
            }
            if (!ok) abort_flag = 1;
        }
        if (lane == 0) {
            s_landed = landed;
            s_issued = issued;
            s_a_landed = a_ok;
        }
    } else {
        // ---- epilogue ----
        float thr = -INFINITY;                     // k-th best so far
        for (uint64_t j = 0; j < ntiles; ++j) {
            const uint32_t acc = (uint32_t)(j % KNN_ACC), ause = (uint32_t)(j / KNN_ACC);
            // warp-uniform decision: the loads below are .sync.aligned
            if (!__all_sync(0xffffffffu, mbar_wait(&bar_acc_full[acc], ause & 1u, &abort_flag))) {
                abort_flag = 1;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            // Blocks are software-pipelined where registers allow (16-column
            // blocks): block bl+1's TMEM load is in flight while block bl is
            // scanned, with two register sets alternating.  32-column blocks
            // (k > 16) load and wait one block at a time.
            constexpr int NB = R::BW <= 16 ? 2 : 1;
            uint32_t r[NB][R::BW];
            float bmax[NB];
            const uint32_t tl = tmem + acc * KNN_BN + (uint32_t)(slice * R::CW) + ((uint32_t)(32 * quarter) << 16);
            if constexpr (NB == 2) {
                __syncwarp();
                tmem_ld_max(tl, r[0], bmax[0]);
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            }
            // (unrolled only when pipelined: four copies of the 32-entry
            // insertion path would not fit the instruction cache)
            constexpr int UNR = NB == 2 ? R::BLOCKS : 1;
#pragma unroll UNR
            for (int bl = 0; bl < R::BLOCKS; ++bl) {
                const int cb = NB == 2 ? (bl & 1) : 0;
                __syncwarp();
                if constexpr (NB == 1) {
                    tmem_ld_max(tl + (uint32_t)(bl * R::BW), r[0], bmax[0]);
                    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                }
                if (NB == 2 && bl + 1 < R::BLOCKS) {
                    tmem_ld_max(tl + (uint32_t)((bl + 1) * R::BW), r[(cb ^ 1) % NB], bmax[(cb ^ 1) % NB]);
                } else if (bl + 1 == R::BLOCKS) {
                    // release the accumulator: this warp's values are all in registers
                    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
                    __syncwarp();
                    if (lane == 0) mbar_arrive(&bar_acc_free[acc]);
                }
                // the block's largest similarity first: most blocks cannot enter
                if (bmax[cb] > thr) {
                    unsigned cand = 0;
#pragma unroll
                    for (int t = 0; t < R::BW; ++t) cand |= (__uint_as_float(r[cb][t]) > thr ? 1u : 0u) << t;
                    const uint32_t col0 = (uint32_t)j * KNN_BN + (uint32_t)(slice * R::CW + bl * R::BW);
                    while (cand) {
                        const int t = __ffs(cand) - 1;
                        cand &= cand - 1;
                        float v = __uint_as_float(r[cb][0]);
#pragma unroll
                        for (int u = 1; u < R::BW; ++u) v = t == u ? __uint_as_float(r[cb][u]) : v;
                        const uint32_t col = col0 + (uint32_t)t;
                        if (v > thr && col < ndb32 && col != self) {
                            topk_push<KMAX>(vals, ids, v, col);
                            thr = kth_value<KMAX>(vals, k);
                        }
                    }
                }
                if (NB == 2 && bl + 1 < R::BLOCKS) {
                    __syncwarp();
                    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                }
            }
        }
    }
    __syncthreads();
    const bool aborted = abort_flag != 0;
    if (aborted) {
        if (threadIdx.x == 0) atomicOr(err, KNN_ERR_TIMEOUT);
        if (warp == R::MMA && lane == 0 && ntiles) {
            // last bounded waits for the copies and MMAs that may still be in flight
            volatile uint32_t never = 0;
            if (!s_a_landed) mbar_wait(&bar_a, 0, &never);
            for (uint64_t sg = s_landed; sg < s_loaded; ++sg)
                mbar_wait(&bar_full[sg % KNN_STAGES], (uint32_t)((sg / KNN_STAGES) & 1), &never);
            if (s_issued) {     // a commit covers every earlier MMA
                const uint64_t sg = s_issued - 1;
                mbar_wait(&bar_empty[sg % KNN_STAGES], (uint32_t)((sg / KNN_STAGES) & 1), &never);
            }
        }
    } else {
        // merge the slices' sorted lists per query (the stages are free now)
        float* pv = reinterpret_cast<float*>(smem);                         // [SLICES][128][KMAX]
        uint32_t* pi = reinterpret_cast<uint32_t*>(smem + (size_t)R::SLICES * KNN_BM * KMAX * 4);
        if (warp < R::EPI) {
            const size_t base = ((size_t)slice * KNN_BM + qrow) * KMAX;
#pragma unroll
            for (int i = 0; i < KMAX; ++i) { pv[base + i] = vals[i]; pi[base + i] = ids[i]; }
        }
        __syncthreads();
        if (warp < 4 && myq < nq) {
            float thr = kth_value<KMAX>(vals, k);
            for (int sl = 1; sl < R::SLICES; ++sl) {
                const size_t b2 = ((size_t)sl * KNN_BM + qrow) * KMAX;
                for (uint32_t i = 0; i < k; ++i) {
                    const float v = pv[b2 + i];
                    if (!(v > thr)) break;     // sorted: the rest cannot enter
                    topk_push<KMAX>(vals, ids, v, pi[b2 + i]);
                    thr = kth_value<KMAX>(vals, k);
                }
            }
#pragma unroll
            for (int i = 0; i < KMAX; ++i) {
                if ((uint32_t)i < k) {
                    idx_out[myq * k + i] = ids[i];
                    sim_out[myq * k + i] = vals[i];
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (warp == 0) {
        __syncwarp();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(KNN_TMEM_COLS)
                     : "memory");
    }
}

// compile-time selection by k
template <int KMAX>
int knn_run(const unsigned char* Q, uint64_t nq, const unsigned char* D, uint64_t ndb, uint32_t dpad,
            const uint64_t* qself, uint32_t k, uint32_t* idx, float* sim, uint32_t* err, cudaStream_t s) {
    // query tile + KNN_STAGES K-block stages (reused at the end for the slices' lists)
    const size_t tiles = (size_t)(dpad / 64) * KNN_A_KB + (size_t)KNN_STAGES * KNN_B_KB;
    const size_t lists = (size_t)KnnRoles<KMAX>::SLICES * KNN_BM * KMAX * 8;
    const size_t smem = std::max(tiles, lists) + 1024;
    KCK(cudaFuncSetAttribute(k_cos_topk<KMAX>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
        "knn shared memory");
    const unsigned grid = (unsigned)((nq + KNN_BM - 1) / KNN_BM);
    cudaEvent_t e0, e1;
    KCK(cudaEventCreate(&e0), "events");
    KCK(cudaEventCreate(&e1), "events");
    cudaEventRecord(e0, s);
    k_cos_topk<KMAX><<<grid, KnnRoles<KMAX>::THREADS, smem, s>>>(Q, nq, D, ndb, dpad, qself, k, idx, sim, err);
    cudaEventRecord(e1, s);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    if (e == cudaSuccess) cudaEventElapsedTime(&g_knn_ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    KCK(e, "knn launch");
    return EP_OK;
}

}  // namespace
}  // namespace ep

using namespace ep;

extern "C" int ep_embed_features(int device, uint64_t n_nodes, const uint64_t* fptr, const uint32_t* fids,
                                 const float* fweight, uint32_t n_feat, uint32_t dims, const float* table,
                                 float* out) {
    if (!fptr || !out || (n_nodes && !table && n_feat) || dims == 0 || dims > 512)
        return knn_fail(EP_ERR_INVALID_ARG, "invalid arguments (dims must be in [1, 512])");
    const uint64_t nf = fptr[n_nodes];
    for (uint64_t v = 0; v < n_nodes; ++v)
        if (fptr[v + 1] < fptr[v]) return knn_fail(EP_ERR_INVALID_ARG, "fptr is not monotone");
    for (uint64_t j = 0; j < nf; ++j)
        if (fids[j] >= n_feat) return knn_fail(EP_ERR_INVALID_ARG, "feature id out of range");
    KCK(cudaSetDevice(device), "select device");
    if (!n_nodes) return EP_OK;
    cudaStream_t s;
    KCK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "stream");
    struct SG { cudaStream_t s; ~SG() { cudaStreamDestroy(s); } } sg{s};
    DevMem dptr, dids, dw, dtab, dout;
    KCK(dptr.alloc((n_nodes + 1) * 8), "alloc");
    KCK(dids.alloc(nf * 4), "alloc");
    KCK(dtab.alloc((size_t)n_feat * dims * 4), "alloc");
    KCK(dout.alloc((size_t)n_nodes * dims * 4), "alloc");
    if (fweight) KCK(dw.alloc((size_t)n_feat * 4), "alloc");
    KCK(cudaMemcpyAsync(dptr.p, fptr, (n_nodes + 1) * 8, cudaMemcpyHostToDevice, s), "upload");
    if (nf) KCK(cudaMemcpyAsync(dids.p, fids, nf * 4, cudaMemcpyHostToDevice, s), "upload");
    if (n_feat) KCK(cudaMemcpyAsync(dtab.p, table, (size_t)n_feat * dims * 4, cudaMemcpyHostToDevice, s), "upload");
    if (fweight) KCK(cudaMemcpyAsync(dw.p, fweight, (size_t)n_feat * 4, cudaMemcpyHostToDevice, s), "upload");
    const uint64_t blocks = (n_nodes * 32 + 255) / 256;
    k_embed<<<(unsigned)blocks, 256, 0, s>>>(n_nodes, (const uint64_t*)dptr.p, (const uint32_t*)dids.p,
                                             fweight ? (const float*)dw.p : nullptr, dims, (const float*)dtab.p,
                                             (float*)dout.p);
    KCK(cudaGetLastError(), "embed launch");
    KCK(cudaMemcpyAsync(out, dout.p, (size_t)n_nodes * dims * 4, cudaMemcpyDeviceToHost, s), "download");
    KCK(cudaStreamSynchronize(s), "embed");
    return EP_OK;
}

extern "C" int ep_align(int device, uint64_t n_nodes, const uint64_t* row_ptr, const uint32_t* cols,
                        const float* w_cdf, uint32_t dims, const float* emb, float alpha, uint64_t max_neighbors,
                        float* out) {
    if (!row_ptr || (n_nodes && (!emb || !out)) || dims == 0 || dims > 512)
        return knn_fail(EP_ERR_INVALID_ARG, "invalid arguments (dims must be in [1, 512])");
    if (alpha > 1.f || alpha != alpha) return knn_fail(EP_ERR_INVALID_ARG, "alpha must be <= 1 (negative: adaptive)");
    const uint64_t ne = row_ptr[n_nodes];
    if (ne && (!cols || !w_cdf)) return knn_fail(EP_ERR_INVALID_ARG, "null edge arrays");
    for (uint64_t v = 0; v < n_nodes; ++v)
        if (row_ptr[v + 1] < row_ptr[v]) return knn_fail(EP_ERR_INVALID_ARG, "row_ptr is not monotone");
    for (uint64_t j = 0; j < ne; ++j)
        if (cols[j] >= n_nodes) return knn_fail(EP_ERR_INVALID_ARG, "column id out of range");
    KCK(cudaSetDevice(device), "select device");
    if (!n_nodes) return EP_OK;
    cudaStream_t s;
    KCK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "stream");
    struct SG { cudaStream_t s; ~SG() { cudaStreamDestroy(s); } } sg{s};
    DevMem drp, dcols, dcdf, demb, dout;
    KCK(drp.alloc((n_nodes + 1) * 8), "alloc");
    KCK(dcols.alloc(ne * 4), "alloc");
    KCK(dcdf.alloc(ne * 4), "alloc");
    KCK(demb.alloc((size_t)n_nodes * dims * 4), "alloc");
    KCK(dout.alloc((size_t)n_nodes * dims * 4), "alloc");
    KCK(cudaMemcpyAsync(drp.p, row_ptr, (n_nodes + 1) * 8, cudaMemcpyHostToDevice, s), "upload");
    if (ne) {
        KCK(cudaMemcpyAsync(dcols.p, cols, ne * 4, cudaMemcpyHostToDevice, s), "upload");
        KCK(cudaMemcpyAsync(dcdf.p, w_cdf, ne * 4, cudaMemcpyHostToDevice, s), "upload");
    }
    KCK(cudaMemcpyAsync(demb.p, emb, (size_t)n_nodes * dims * 4, cudaMemcpyHostToDevice, s), "upload");
    cudaEvent_t e0, e1;
    KCK(cudaEventCreate(&e0), "events");
    KCK(cudaEventCreate(&e1), "events");
    struct EG { cudaEvent_t a, b; ~EG() { cudaEventDestroy(a); cudaEventDestroy(b); } } eg{e0, e1};
    cudaEventRecord(e0, s);
    k_align<<<(unsigned)((n_nodes * 32 + 255) / 256), 256, 0, s>>>(
        n_nodes, (const uint64_t*)drp.p, (const uint32_t*)dcols.p, (const float*)dcdf.p, dims,
        (const float*)demb.p, alpha, max_neighbors ? max_neighbors : ~0ull, (float*)dout.p);
    cudaEventRecord(e1, s);
    KCK(cudaGetLastError(), "align launch");
    KCK(cudaMemcpyAsync(out, dout.p, (size_t)n_nodes * dims * 4, cudaMemcpyDeviceToHost, s), "download");
    KCK(cudaStreamSynchronize(s), "align");
    cudaEventElapsedTime(&g_knn_ms, e0, e1);
    return EP_OK;
}

extern "C" int ep_knn_cosine(int device, uint64_t n_db, uint32_t dims, const float* db, uint64_t n_q,
                             const float* q, const uint64_t* q_self, uint32_t k, uint32_t* idx_out, float* sim_out) {
    if (dims == 0 || dims > 256) return knn_fail(EP_ERR_INVALID_ARG, "dims must be in [1, 256]");
    if (k == 0 || k > 32) return knn_fail(EP_ERR_INVALID_ARG, "k must be in [1, 32]");
    if (n_db >= 0xffffffffull) return knn_fail(EP_ERR_INVALID_ARG, "n_db must be below 2^32 - 1");
    if ((n_db && !db) || (n_q && (!q || !idx_out || !sim_out)))
        return knn_fail(EP_ERR_INVALID_ARG, "null array");
    if (q_self)
        for (uint64_t i = 0; i < n_q; ++i)
            if (q_self[i] != ~0ull && q_self[i] >= n_db) return knn_fail(EP_ERR_INVALID_ARG, "q_self out of range");
    KCK(cudaSetDevice(device), "select device");
    if (!n_q) return EP_OK;
    const uint32_t dpad = (dims + 63) / 64 * 64;
    const uint64_t q_tile_bytes = (uint64_t)(dpad / 64) * 128 * KNN_BM, db_tile_bytes = (uint64_t)(dpad / 64) * 128 * KNN_BN;
    const uint64_t db_tiles = (n_db + KNN_BN - 1) / KNN_BN, q_tiles = (n_q + KNN_BM - 1) / KNN_BM;
    cudaStream_t s;
    KCK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "stream");
    struct SG { cudaStream_t s; ~SG() { cudaStreamDestroy(s); } } sg{s};
    DevMem draw, dq, dD, dQ, dself, didx, dsim, derr;
    const uint64_t nmax = std::max(n_db, n_q);
    KCK(draw.alloc(nmax * dims * 4), "alloc");
    KCK(dD.alloc(std::max<uint64_t>(db_tiles, 1) * db_tile_bytes), "alloc");
    KCK(dQ.alloc(q_tiles * q_tile_bytes), "alloc");
    KCK(didx.alloc(n_q * k * 4), "alloc");
    KCK(dsim.alloc(n_q * k * 4), "alloc");
    KCK(derr.alloc(4), "alloc");
    KCK(cudaMemsetAsync(derr.p, 0, 4, s), "clear");
    if (q_self) {
        KCK(dself.alloc(n_q * 8), "alloc");
        KCK(cudaMemcpyAsync(dself.p, q_self, n_q * 8, cudaMemcpyHostToDevice, s), "upload");
    }
    if (n_db) {
        KCK(cudaMemcpyAsync(draw.p, db, n_db * dims * 4, cudaMemcpyHostToDevice, s), "upload");
        k_norm_swz<<<(unsigned)((db_tiles * KNN_BN * 32 + 255) / 256), 256, 0, s>>>(
            n_db, db_tiles * KNN_BN, dims, dpad, 8, (const float*)draw.p, (unsigned char*)dD.p);
        KCK(cudaGetLastError(), "normalise");
    }
    KCK(cudaMemcpyAsync(draw.p, q, n_q * dims * 4, cudaMemcpyHostToDevice, s), "upload");
    k_norm_swz<<<(unsigned)((q_tiles * KNN_BM * 32 + 255) / 256), 256, 0, s>>>(n_q, q_tiles * KNN_BM, dims, dpad, 7,
                                                                              (const float*)draw.p,
                                                                              (unsigned char*)dQ.p);
    KCK(cudaGetLastError(), "normalise");
    const uint64_t* qs = q_self ? (const uint64_t*)dself.p : nullptr;
    // the shortest list that holds k: insertion and the k-th-value scan cost O(KMAX)
    const unsigned char *Qp = (const unsigned char*)dQ.p, *Dp = (const unsigned char*)dD.p;
    uint32_t *ip = (uint32_t*)didx.p, *ep = (uint32_t*)derr.p;
    float* sp = (float*)dsim.p;
    int rc = k <= 8    ? knn_run<8>(Qp, n_q, Dp, n_db, dpad, qs, k, ip, sp, ep, s)
             : k <= 12 ? knn_run<12>(Qp, n_q, Dp, n_db, dpad, qs, k, ip, sp, ep, s)
             : k <= 16 ? knn_run<16>(Qp, n_q, Dp, n_db, dpad, qs, k, ip, sp, ep, s)
                       : knn_run<32>(Qp, n_q, Dp, n_db, dpad, qs, k, ip, sp, ep, s);
    if (rc) return rc;
    uint32_t herr = 0;
    KCK(cudaMemcpyAsync(idx_out, didx.p, n_q * k * 4, cudaMemcpyDeviceToHost, s), "download");
    KCK(cudaMemcpyAsync(sim_out, dsim.p, n_q * k * 4, cudaMemcpyDeviceToHost, s), "download");
    KCK(cudaMemcpyAsync(&herr, derr.p, 4, cudaMemcpyDeviceToHost, s), "download");
    KCK(cudaStreamSynchronize(s), "knn");
    if (herr) return knn_fail(EP_ERR_DEVICE, "tensor-core wait timed out");
    return EP_OK;
}

extern "C" const char* ep_knn_last_error(void) { return g_knn_err.c_str(); }

extern "C" float ep_knn_last_kernel_ms(void) { return g_knn_ms; }
