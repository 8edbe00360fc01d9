// ep_knn.cu -- node embeddings from feature embeddings and exact cosine
// top-k on the GPU (the evaluation side of the path).
//
//   ep_embed_features  NodeEmbedder.embed_feature_set (src/lib.rs:2092-2124)
//                      with AvgAggregator / WeightedAggregator
//                      (src/algos/aggregator.rs:17-120): warp per node.
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

// Rows scaled to unit L2 norm (zero rows stay zero), as BF16 padded to dpad.
__global__ void __launch_bounds__(256) k_norm_bf16(uint64_t n, uint32_t d, uint32_t dpad, const float* __restrict__ x,
                                                   __nv_bfloat16* __restrict__ y) {
    const int lane = threadIdx.x & 31;
    const uint64_t r = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (r >= n) return;
    float ss = 0.f;
    for (uint32_t k = lane; k < d; k += 32) {
        const float t = x[r * d + k];
        ss += t * t;
    }
    ss = warp_sum<float>(ss);
    const float inv = ss > 0.f ? 1.f / sqrtf(ss) : 0.f;
    for (uint32_t k = lane; k < dpad; k += 32) y[r * dpad + k] = __float2bfloat16_rn(k < d ? x[r * d + k] * inv : 0.f);
}

// ---------------------------------------------------------------------------
// Cosine top-k: one CTA (4 warps) per 128 queries.
//
// Operand tiles live in shared memory in the K-major 128-byte-swizzled
// layout the tensor core reads: per 64-element K block, rows of 128 B in
// 8-row atoms of 1024 B; the 16-byte chunk c of row r sits at chunk position
// c ^ (r % 8).  A (queries, M = 128) is loaded once; B (database rows,
// N = 128) once per tile.  One thread issues the MMAs of a tile into a
// 128 x 128 FP32 accumulator in tensor memory and commits them to an
// mbarrier; then thread t of the CTA reads row t (its query) with tcgen05.ld
// and merges the 128 similarities into its sorted top-KMAX in registers.
// ---------------------------------------------------------------------------
constexpr int KNN_BM = 128, KNN_BN = 128, KNN_THREADS = 128;
constexpr uint32_t KNN_TMEM_COLS = 128;
constexpr uint32_t KNN_WAIT_LIMIT = 1u << 22;    // mbarrier polls (32 ns sleeps) before giving up
enum : uint32_t { KNN_ERR_TIMEOUT = 1u };

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

// Stages rows [row0, row0 + nrows) of a [n x dpad] BF16 matrix (rows >= n
// zero-filled) into the swizzled layout at s (1024-byte aligned).
__device__ __forceinline__ void stage_rows(unsigned char* s, const __nv_bfloat16* __restrict__ g, uint64_t n,
                                           uint64_t row0, int nrows, uint32_t dpad) {
    const uint32_t chunks = dpad / 8;                  // 16-byte chunks per row
    const uint32_t total = (uint32_t)nrows * chunks;
    for (uint32_t i = threadIdx.x; i < total; i += KNN_THREADS) {
        const uint32_t r = i / chunks, c = i % chunks;
        const uint32_t kb = c / 8, cc = c % 8;
        const uint32_t off = kb * (uint32_t)nrows * 128u + (r / 8) * 1024u + (r % 8) * 128u + ((cc ^ (r % 8)) * 16u);
        const uint64_t row = row0 + r;
        const bool in = row < n;
        const void* src = in ? (const void*)(g + row * dpad + (uint64_t)c * 8) : (const void*)g;
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(smem_u32(s + off)), "l"(src),
                     "r"(in ? 16 : 0)
                     : "memory");
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
}

// Polls the mbarrier for the completion of the phase with the given parity:
// at most KNN_WAIT_LIMIT polls, 32 ns apart.  Returns 1 when it completed.
__device__ __forceinline__ uint32_t mbar_wait(uint64_t* mbar, uint32_t parity) {
    uint32_t done = 0;
    for (uint32_t it = 0; it < KNN_WAIT_LIMIT; ++it) {
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
            : "=r"(done)
            : "r"(smem_u32(mbar)), "r"(parity)
            : "memory");
        if (done) break;
        __nanosleep(32);
    }
    return done;
}

template <int KMAX>
__device__ __forceinline__ void topk_push(float (&vals)[KMAX], uint32_t (&ids)[KMAX], float v, uint32_t id) {
    if (!(v > vals[KMAX - 1])) return;
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

template <int KMAX>
__global__ void __launch_bounds__(KNN_THREADS, 1)
    k_cos_topk(const __nv_bfloat16* __restrict__ Q, uint64_t nq, const __nv_bfloat16* __restrict__ D, uint64_t ndb,
               uint32_t dpad, const uint64_t* __restrict__ qself, uint32_t k, uint32_t* __restrict__ idx_out,
               float* __restrict__ sim_out, uint32_t* __restrict__ err) {
    extern __shared__ unsigned char knn_smem_raw[];
    __shared__ uint64_t mbar;
    __shared__ uint32_t tmem_slot;
    unsigned char* smem = (unsigned char*)(((uintptr_t)knn_smem_raw + 1023) & ~(uintptr_t)1023);
    unsigned char* sA = smem;
    unsigned char* sB = smem + (size_t)KNN_BM * dpad * 2;
    const int warp = threadIdx.x >> 5;
    const uint64_t q0 = (uint64_t)blockIdx.x * KNN_BM;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                     "r"(KNN_TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (threadIdx.x == 0) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar)) : "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_slot;

    stage_rows(sA, Q, nq, q0, KNN_BM, dpad);

    float vals[KMAX];
    uint32_t ids[KMAX];
#pragma unroll
    for (int i = 0; i < KMAX; ++i) { vals[i] = -INFINITY; ids[i] = 0xffffffffu; }
    const uint64_t myq = q0 + threadIdx.x;              // TMEM lane = accumulator row = query
    const uint64_t self = (qself && myq < nq) ? qself[myq] : ~0ull;
    const uint32_t idesc = umma_idesc(KNN_BM, KNN_BN);
    const uint32_t nkb = dpad / 64;
    bool timed_out = false;
    uint32_t phase = 0;

    for (uint64_t t0 = 0; t0 < ndb && !timed_out; t0 += KNN_BN) {
        stage_rows(sB, D, ndb, t0, KNN_BN, dpad);
        asm volatile("cp.async.wait_all;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");   // staged tiles -> tensor core
        __syncthreads();
        if (threadIdx.x == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            for (uint32_t kb = 0; kb < nkb; ++kb) {
#pragma unroll
                for (uint32_t s = 0; s < 4; ++s) {          // K = 16 per MMA: 32 bytes within the 128-byte row
                    const uint64_t ad = umma_desc(smem_u32(sA + kb * KNN_BM * 128u) + s * 32u);
                    const uint64_t bd = umma_desc(smem_u32(sB + kb * KNN_BN * 128u) + s * 32u);
                    const uint32_t acc = (kb | s) ? 1u : 0u;
                    asm volatile(
                        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(tmem),
                        "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
                        : "memory");
                }
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                             smem_u32(&mbar))
                         : "memory");
        }
        // wait for the tile's MMAs (bounded); the outcome is made CTA-wide
        uint32_t done = mbar_wait(&mbar, phase);
        if (__syncthreads_or(!done)) {
            timed_out = true;
            if (threadIdx.x == 0) atomicOr(err, KNN_ERR_TIMEOUT);
            // give the committed MMAs a second bounded wait before TMEM is freed
            if (!done) mbar_wait(&mbar, phase);
            done = 0;
        }
        phase ^= 1u;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        if (done) {
            for (uint32_t c0 = 0; c0 < (uint32_t)KNN_BN; c0 += 32) {
                uint32_t r[32];
                const uint32_t taddr = tmem + ((uint32_t)(32 * warp) << 16) + c0;
                asm volatile(
                    "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
                    "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
                    : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                      "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
                      "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]),
                      "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]),
                      "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
                    : "r"(taddr)
                    : "memory");
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
                for (int t = 0; t < 32; ++t) {
                    const uint64_t col = t0 + c0 + (uint32_t)t;
                    if (col < ndb && col != self) topk_push<KMAX>(vals, ids, __uint_as_float(r[t]), (uint32_t)col);
                }
            }
        }
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();       // TMEM and the B tile are free for the next tile
    }
    if (myq < nq && !timed_out) {
#pragma unroll
        for (int i = 0; i < KMAX; ++i) {
            if ((uint32_t)i < k) {
                idx_out[myq * k + i] = ids[i];
                sim_out[myq * k + i] = vals[i];
            }
        }
    }
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(KNN_TMEM_COLS)
                     : "memory");
}

// compile-time selection by k
template <int KMAX>
int knn_run(const __nv_bfloat16* Q, uint64_t nq, const __nv_bfloat16* D, uint64_t ndb, uint32_t dpad,
            const uint64_t* qself, uint32_t k, uint32_t* idx, float* sim, uint32_t* err, cudaStream_t s) {
    const size_t smem = (size_t)(KNN_BM + KNN_BN) * dpad * 2 + 1024;
    KCK(cudaFuncSetAttribute(k_cos_topk<KMAX>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
        "knn shared memory");
    const unsigned grid = (unsigned)((nq + KNN_BM - 1) / KNN_BM);
    k_cos_topk<KMAX><<<grid, KNN_THREADS, smem, s>>>(Q, nq, D, ndb, dpad, qself, k, idx, sim, err);
    KCK(cudaGetLastError(), "knn launch");
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

extern "C" int ep_knn_cosine(int device, uint64_t n_db, uint32_t dims, const float* db, uint64_t n_q,
                             const float* q, const uint64_t* q_self, uint32_t k, uint32_t* idx_out, float* sim_out) {
    if (dims == 0 || dims > 256) return knn_fail(EP_ERR_INVALID_ARG, "dims must be in [1, 256]");
    if (k == 0 || k > 32) return knn_fail(EP_ERR_INVALID_ARG, "k must be in [1, 32]");
    if ((n_db && !db) || (n_q && (!q || !idx_out || !sim_out)))
        return knn_fail(EP_ERR_INVALID_ARG, "null array");
    if (q_self)
        for (uint64_t i = 0; i < n_q; ++i)
            if (q_self[i] != ~0ull && q_self[i] >= n_db) return knn_fail(EP_ERR_INVALID_ARG, "q_self out of range");
    KCK(cudaSetDevice(device), "select device");
    if (!n_q) return EP_OK;
    const uint32_t dpad = (dims + 63) / 64 * 64;
    cudaStream_t s;
    KCK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "stream");
    struct SG { cudaStream_t s; ~SG() { cudaStreamDestroy(s); } } sg{s};
    DevMem draw, dq, dD, dQ, dself, didx, dsim, derr;
    const uint64_t nmax = std::max(n_db, n_q);
    KCK(draw.alloc(nmax * dims * 4), "alloc");
    KCK(dD.alloc(std::max<uint64_t>(n_db, 1) * dpad * 2), "alloc");
    KCK(dQ.alloc(n_q * dpad * 2), "alloc");
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
        k_norm_bf16<<<(unsigned)((n_db * 32 + 255) / 256), 256, 0, s>>>(n_db, dims, dpad, (const float*)draw.p,
                                                                       (__nv_bfloat16*)dD.p);
        KCK(cudaGetLastError(), "normalise");
    }
    KCK(cudaMemcpyAsync(draw.p, q, n_q * dims * 4, cudaMemcpyHostToDevice, s), "upload");
    k_norm_bf16<<<(unsigned)((n_q * 32 + 255) / 256), 256, 0, s>>>(n_q, dims, dpad, (const float*)draw.p,
                                                                   (__nv_bfloat16*)dQ.p);
    KCK(cudaGetLastError(), "normalise");
    const uint64_t* qs = q_self ? (const uint64_t*)dself.p : nullptr;
    int rc = k <= 16 ? knn_run<16>((const __nv_bfloat16*)dQ.p, n_q, (const __nv_bfloat16*)dD.p, n_db, dpad, qs, k,
                                   (uint32_t*)didx.p, (float*)dsim.p, (uint32_t*)derr.p, s)
                     : knn_run<32>((const __nv_bfloat16*)dQ.p, n_q, (const __nv_bfloat16*)dD.p, n_db, dpad, qs, k,
                                   (uint32_t*)didx.p, (float*)dsim.p, (uint32_t*)derr.p, s);
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
