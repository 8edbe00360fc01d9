// ep_sort.cu -- stable LSD radix sort of gradient items by feature id.
//
// The value carried with each key is the item's (role-src, count-weight bits)
// pair, so the reduction reads both with one coalesced load.
//
// Replaces the per-batch std::HashMap merge of src/algos/ep/mod.rs:223-233
// and the racy Hogwild row writes (src/hogwild.rs:15-60): after a stable sort
// by feature id the items of one feature are contiguous and keep their
// emission order (anchor, role, occurrence), so the reduction that follows is
// deterministic and can apply the reference's first-occurrence rule.
//
// One pass per 8-bit digit, three kernels per pass:
//   k_radix_hist     per-tile digit counts -> hist[digit * ntiles + tile]
//   k_radix_colscan  one warp per digit: exclusive scan of that digit's counts
//                    over the tiles (in place) and the digit total
//   k_radix_scatter  digit bases from the 256 totals (scanned per CTA), then
//                    per-tile stable ranks (warp match + per-warp counters)
// The item count lives in device memory (BatchState::n_items), so the same
// launches replay inside a CUDA graph for any batch.
#include <cuda_runtime.h>

#include "ep_device.cuh"
#include "ep_internal.h"
#include "ep_launch.cuh"

namespace ep {

constexpr int SORT_THREADS = 256;          // 8 warps
constexpr int SORT_ROUNDS = 8;             // rounds of 32 items per warp
constexpr int SORT_TILE = SORT_THREADS * SORT_ROUNDS;   // 2048 items
constexpr int SORT_MAX_GRID = 152 * 4;

size_t radix_hist_entries(uint64_t cap) {
    const uint64_t tiles = (cap + SORT_TILE - 1) / SORT_TILE;
    return (size_t)(256 * (tiles ? tiles : 1)) + 256;   // + digit totals
}

__global__ void __launch_bounds__(SORT_THREADS) k_radix_hist(const uint32_t* __restrict__ keys, const BatchState* st,
                                                             int shift, uint32_t* __restrict__ hist) {
    pdl_wait();
    pdl_trigger();
    __shared__ uint32_t h[256];
    const uint32_t n = st->n_items;
    const uint32_t ntiles = (n + SORT_TILE - 1) / SORT_TILE;
    for (uint32_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        h[threadIdx.x] = 0;
        __syncthreads();
        const uint32_t base = tile * SORT_TILE;
        const uint32_t end = min(base + SORT_TILE, n);
        for (uint32_t i = base + threadIdx.x; i < end; i += SORT_THREADS)
            atomicAdd(&h[(keys[i] >> shift) & 255u], 1u);
        __syncthreads();
        hist[threadIdx.x * ntiles + tile] = h[threadIdx.x];
        __syncthreads();
    }
}

// One warp per digit: exclusive scan of hist[d * ntiles .. + ntiles) and the
// digit's total in dtot[d].
__global__ void __launch_bounds__(256) k_radix_colscan(const BatchState* st, uint32_t* hist, uint32_t* dtot) {
    pdl_wait();
    pdl_trigger();
    const int lane = threadIdx.x & 31;
    const uint32_t d = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (d >= 256) return;
    const uint32_t n = st->n_items;
    const uint32_t ntiles = (n + SORT_TILE - 1) / SORT_TILE;
    uint32_t* col = hist + (size_t)d * ntiles;
    uint32_t carry = 0;
    for (uint32_t b = 0; b < ntiles; b += 32) {
        const uint32_t t = b + lane;
        const uint32_t x = t < ntiles ? col[t] : 0u;
        const uint32_t incl = warp_incl_scan(x, lane);
        if (t < ntiles) col[t] = carry + incl - x;
        carry += __shfl_sync(FULL, incl, 31);
    }
    if (lane == 0) dtot[d] = carry;
}

__global__ void __launch_bounds__(SORT_THREADS) k_radix_scatter(const uint32_t* __restrict__ keys_in,
                                                                const uint2* __restrict__ vals_in,
                                                                const uint32_t* __restrict__ item_src,
                                                                const float* __restrict__ item_c,
                                                                uint32_t* __restrict__ keys_out,
                                                                uint2* __restrict__ vals_out,
                                                                const BatchState* st, int shift,
                                                                const uint32_t* __restrict__ hist,
                                                                const uint32_t* __restrict__ dtot) {
    pdl_wait();
    pdl_trigger();
    __shared__ uint32_t wcount[SORT_THREADS / 32][256];
    __shared__ uint32_t dbase[256];
    __shared__ uint32_t wtot[SORT_THREADS / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const uint32_t n = st->n_items;
    const uint32_t ntiles = (n + SORT_TILE - 1) / SORT_TILE;
    if (blockIdx.x >= ntiles) return;
    {   // exclusive scan of the 256 digit totals -> first position of each digit
        const uint32_t x = dtot[threadIdx.x];
        const uint32_t incl = warp_incl_scan(x, lane);
        if (lane == 31) wtot[w] = incl;
        __syncthreads();
        uint32_t off = 0;
        for (int ww = 0; ww < w; ++ww) off += wtot[ww];
        dbase[threadIdx.x] = off + incl - x;
        __syncthreads();
    }
    for (uint32_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        for (int i = threadIdx.x; i < (SORT_THREADS / 32) * 256; i += SORT_THREADS) (&wcount[0][0])[i] = 0;
        __syncthreads();
        const uint32_t base = tile * SORT_TILE + w * (32 * SORT_ROUNDS);
        uint32_t key[SORT_ROUNDS], rank[SORT_ROUNDS];
        uint2 val[SORT_ROUNDS];
#pragma unroll
        for (int r = 0; r < SORT_ROUNDS; ++r) {
            const uint32_t i = base + r * 32 + lane;
            const bool ok = i < n;
            key[r] = ok ? keys_in[i] : 0u;
            val[r] = ok ? (vals_in ? vals_in[i] : make_uint2(item_src[i], __float_as_uint(item_c[i])))
                        : make_uint2(0u, 0u);
            const uint32_t dig = ok ? ((key[r] >> shift) & 255u) : 256u;
            const unsigned peers = __match_any_sync(FULL, dig);
            const uint32_t before = ok ? wcount[w][dig] : 0u;
            __syncwarp();
            const int leader = __ffs(peers) - 1;
            if (ok && lane == leader) wcount[w][dig] = before + __popc(peers);
            __syncwarp();
            rank[r] = before + __popc(peers & ((1u << lane) - 1u));
        }
        __syncthreads();
        // exclusive prefix over warps, per digit
        if (threadIdx.x < 256) {
            uint32_t s = 0;
#pragma unroll
            for (int ww = 0; ww < SORT_THREADS / 32; ++ww) {
                const uint32_t c = wcount[ww][threadIdx.x];
                wcount[ww][threadIdx.x] = s;
                s += c;
            }
        }
        __syncthreads();
#pragma unroll
        for (int r = 0; r < SORT_ROUNDS; ++r) {
            const uint32_t i = base + r * 32 + lane;
            if (i < n) {
                const uint32_t dig = (key[r] >> shift) & 255u;
                const uint32_t pos = dbase[dig] + hist[dig * ntiles + tile] + wcount[w][dig] + rank[r];
                keys_out[pos] = key[r];
                vals_out[pos] = val[r];
            }
        }
        __syncthreads();
    }
}

// Sorts keys[0, n_items) carrying (item_src, item_c) values.  Ping-pongs
// between (keys, keys_alt) and (vals, vals_alt); returns where the result is.
void launch_radix_sort(BatchState* st, uint32_t* keys, uint32_t* keys_alt, const uint32_t* item_src,
                       const float* item_c, uint2* vals, uint2* vals_alt, uint32_t* hist, uint64_t cap,
                       int key_bits, uint32_t** sorted_keys, uint2** sorted_vals, cudaStream_t s) {
    const uint64_t tiles = (cap + SORT_TILE - 1) / SORT_TILE;
    const unsigned grid = (unsigned)(tiles < SORT_MAX_GRID ? (tiles ? tiles : 1) : SORT_MAX_GRID);
    const int passes = key_bits <= 0 ? 1 : (key_bits + 7) / 8;
    // pass p reads K[p % 2] and writes K[(p + 1) % 2]; values start from the
    // item arrays (vals_in == nullptr) and then alternate between vals / vals_alt.
    uint32_t* K[2] = {keys, keys_alt};
    uint2* V[2] = {vals, vals_alt};
    uint32_t* kin = nullptr;
    uint2* vin = nullptr;
    uint32_t* dtot = hist + radix_hist_entries(cap) - 256;
    for (int p = 0; p < passes; ++p) {
        const int shift = 8 * p;
        kin = K[p & 1];
        uint32_t* kout = K[(p + 1) & 1];
        vin = p == 0 ? nullptr : V[(p - 1) & 1];
        uint2* vout = V[p & 1];
        launch_chain(k_radix_hist, grid, SORT_THREADS, 0, s, (const uint32_t*)kin, (const BatchState*)st, shift, hist);
        launch_chain(k_radix_colscan, 32, 256, 0, s, (const BatchState*)st, hist, dtot);
        launch_chain(k_radix_scatter, grid, SORT_THREADS, 0, s, (const uint32_t*)kin, (const uint2*)vin, item_src, item_c,
                     kout, vout, (const BatchState*)st, shift, (const uint32_t*)hist, (const uint32_t*)dtot);
        kin = kout;
        vin = vout;
    }
    *sorted_keys = kin;
    *sorted_vals = vin;
}

}  // namespace ep
