// ep_device.cuh -- device building blocks: counter-based Philox RNG, warp
// primitives, and vectorised access to one table row split across a warp.
//
// Row layout in HBM: a table of n_feat rows, each padded to `dpad` elements
// (dpad = VPL * ceil(dims / VPL), VPL = values per lane).  Lane l of a warp
// owns elements [l*VPL, l*VPL + VPL) of every row, so one row is read by one
// coalesced warp-wide access of VPL*sizeof(T) bytes per lane (16 B for BF16
// at d=256).  Padding elements are zero and stay zero under training.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

namespace ep {

constexpr unsigned FULL = 0xffffffffu;

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy
// as 1, 2, 3", SC 2011).  Counter-based: every draw is a pure function of
// (key, counter), so sampling is reproducible and needs no RNG state.
// ---------------------------------------------------------------------------
struct u32x4 { uint32_t x, y, z, w; };

__host__ __device__ __forceinline__ void mulhilo32(uint32_t a, uint32_t b, uint32_t& hi, uint32_t& lo) {
    uint64_t p = (uint64_t)a * (uint64_t)b;
    hi = (uint32_t)(p >> 32);
    lo = (uint32_t)p;
}

__host__ __device__ __forceinline__ u32x4 philox(u32x4 c, uint64_t key) {
    uint32_t k0 = (uint32_t)key, k1 = (uint32_t)(key >> 32);
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        uint32_t hi0, lo0, hi1, lo1;
        mulhilo32(0xD2511F53u, c.x, hi0, lo0);
        mulhilo32(0xCD9E8D57u, c.z, hi1, lo1);
        c = u32x4{hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    return c;
}

// Stream ids (third counter word, top byte).
enum : uint32_t { ST_NBR = 1u, ST_NEG = 2u, ST_NSEL = 3u, ST_ROUND = 4u, ST_INIT = 5u, ST_NOISE = 6u, ST_FSEL = 7u, ST_HARD = 8u, ST_WRES = 9u, ST_PPR = 10u };

__host__ __device__ __forceinline__ uint32_t rand_u32(uint64_t seed, uint32_t a, uint32_t b,
                                                      uint32_t stream, uint32_t i) {
    u32x4 r = philox(u32x4{a, b, (stream << 24) | (i >> 2), 0x5bd1e995u}, seed);
    switch (i & 3u) { case 0: return r.x; case 1: return r.y; case 2: return r.z; default: return r.w; }
}

// 32-bit finalizer of MurmurHash3 (Appleby): a bijective avalanche mix.
__host__ __device__ __forceinline__ uint32_t mix32(uint32_t x) {
    x ^= x >> 16;
    x *= 0x85ebca6bu;
    x ^= x >> 13;
    x *= 0xc2b2ae35u;
    x ^= x >> 16;
    return x;
}

// Uniform integer in [0, n) by multiply-high (bias < n / 2^32).
__host__ __device__ __forceinline__ uint32_t below(uint32_t r, uint32_t n) {
    return (uint32_t)(((uint64_t)r * (uint64_t)n) >> 32);
}
__host__ __device__ __forceinline__ float unit_f32(uint32_t r) {   // [0, 1)
    return (float)(r >> 8) * (1.0f / 16777216.0f);
}

// ---------------------------------------------------------------------------
// Warp primitives
// ---------------------------------------------------------------------------
template <typename A>
__device__ __forceinline__ A warp_sum(A v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
    return v;
}

__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t v, int lane) {
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t t = __shfl_up_sync(FULL, v, o);
        if (lane >= o) v += t;
    }
    return v;
}

template <typename A> __device__ __forceinline__ bool is_finite(A x) { return isfinite(x); }

// ---------------------------------------------------------------------------
// Row I/O.  RowIO<T, VPL>::load reads this lane's VPL elements of a row as A.
// ---------------------------------------------------------------------------
template <int BYTES> struct VecT;
template <> struct VecT<2> { using type = unsigned short; };
template <> struct VecT<4> { using type = unsigned int; };
template <> struct VecT<8> { using type = uint2; };
template <> struct VecT<16> { using type = uint4; };

template <typename T> __device__ __forceinline__ float to_f(T x);
template <> __device__ __forceinline__ float to_f<float>(float x) { return x; }
template <> __device__ __forceinline__ float to_f<__nv_bfloat16>(__nv_bfloat16 x) { return __bfloat162float(x); }

template <typename A, typename T> __device__ __forceinline__ A cvt_in(T x) { return (A)to_f<T>(x); }
template <> __device__ __forceinline__ double cvt_in<double, double>(double x) { return x; }
template <> __device__ __forceinline__ float cvt_in<float, double>(double x) { return (float)x; }

// acc[k] += c * x[k] over a lane's slice.  FP32 pairs go through the packed
// FMA of sm_100+ (__ffma2_rn: two independent fused multiply-adds, each
// rounded once, so results equal the scalar loop's bit for bit).
template <typename A, int VPL>
__device__ __forceinline__ void axpy_slice(A (&acc)[VPL], A c, const A (&x)[VPL]) {
    if constexpr (std::is_same<A, float>::value && VPL >= 2 && (VPL % 2) == 0) {
        const float2 cc = make_float2(c, c);
#pragma unroll
        for (int k = 0; k < VPL; k += 2) {
            const float2 r = __ffma2_rn(cc, make_float2(x[k], x[k + 1]), make_float2(acc[k], acc[k + 1]));
            acc[k] = r.x;
            acc[k + 1] = r.y;
        }
    } else {
#pragma unroll
        for (int k = 0; k < VPL; ++k) acc[k] += c * x[k];
    }
}

template <typename T, int VPL>
struct RowIO {
    static constexpr int BYTES = VPL * (int)sizeof(T);
    static constexpr int VB = BYTES >= 16 ? 16 : BYTES;
    static constexpr int NV = BYTES / VB;
    using V = typename VecT<VB>::type;

    // Read-only path (ld.global.nc): valid while no kernel writes the row
    // concurrently, which holds for the table inside one forward kernel.
    template <typename A>
    static __device__ __forceinline__ void load(const T* __restrict__ row, int lane, A (&out)[VPL]) {
        union { V v[NV]; T t[VPL]; } u;
        const V* src = reinterpret_cast<const V*>(row + lane * VPL);
#pragma unroll
        for (int i = 0; i < NV; ++i) u.v[i] = __ldg(src + i);
#pragma unroll
        for (int k = 0; k < VPL; ++k) out[k] = cvt_in<A, T>(u.t[k]);
    }
    // Coherent load (rows written earlier in the same kernel).
    template <typename A>
    static __device__ __forceinline__ void load_cg(const T* row, int lane, A (&out)[VPL]) {
        union { V v[NV]; T t[VPL]; } u;
        const V* src = reinterpret_cast<const V*>(row + lane * VPL);
#pragma unroll
        for (int i = 0; i < NV; ++i) u.v[i] = __ldcg(src + i);
#pragma unroll
        for (int k = 0; k < VPL; ++k) out[k] = cvt_in<A, T>(u.t[k]);
    }
    // Plain load through a generic pointer (shared or global memory).
    template <typename A>
    static __device__ __forceinline__ void load_generic(const T* row, int lane, A (&out)[VPL]) {
        union { V v[NV]; T t[VPL]; } u;
        const V* src = reinterpret_cast<const V*>(row + lane * VPL);
#pragma unroll
        for (int i = 0; i < NV; ++i) u.v[i] = src[i];
#pragma unroll
        for (int k = 0; k < VPL; ++k) out[k] = cvt_in<A, T>(u.t[k]);
    }
    // Raw row slice kept in its storage type while loads are in flight.
    struct Raw { V v[NV]; };
    // number of raw slices that fit in about 32 registers
    static constexpr int INFLIGHT = (BYTES >= 128) ? 1 : (128 / BYTES > 8 ? 8 : 128 / BYTES);
    static __device__ __forceinline__ Raw load_raw(const T* __restrict__ row, int lane) {
        Raw r;
        const V* src = reinterpret_cast<const V*>(row + lane * VPL);
#pragma unroll
        for (int i = 0; i < NV; ++i) r.v[i] = __ldg(src + i);
        return r;
    }
    template <typename A>
    static __device__ __forceinline__ void fma(A (&acc)[VPL], A c, const Raw& r) {
        union { V v[NV]; T t[VPL]; } u;
#pragma unroll
        for (int i = 0; i < NV; ++i) u.v[i] = r.v[i];
        A x[VPL];
#pragma unroll
        for (int k = 0; k < VPL; ++k) x[k] = cvt_in<A, T>(u.t[k]);
        axpy_slice<A, VPL>(acc, c, x);
    }
    static __device__ __forceinline__ void store_raw(T* row, int lane, const T (&in)[VPL]) {
        union { V v[NV]; T t[VPL]; } u;
#pragma unroll
        for (int k = 0; k < VPL; ++k) u.t[k] = in[k];
        V* dst = reinterpret_cast<V*>(row + lane * VPL);
#pragma unroll
        for (int i = 0; i < NV; ++i) dst[i] = u.v[i];
    }
};

template <typename T> struct FromA;
template <> struct FromA<float> {
    template <typename A> static __device__ __forceinline__ float cvt(A x) { return (float)x; }
};
template <> struct FromA<__nv_bfloat16> {
    template <typename A> static __device__ __forceinline__ __nv_bfloat16 cvt(A x) {
        return __float2bfloat16_rn((float)x);
    }
};
template <> struct FromA<double> {
    template <typename A> static __device__ __forceinline__ double cvt(A x) { return (double)x; }
};

// Stores VPL accumulator values into a row of T (float/double: exact cast).
template <typename T, int VPL, typename A>
__device__ __forceinline__ void store_row(T* row, int lane, const A (&in)[VPL]) {
    T t[VPL];
#pragma unroll
    for (int k = 0; k < VPL; ++k) t[k] = FromA<T>::cvt(in[k]);
    RowIO<T, VPL>::store_raw(row, lane, t);
}

// Storage type of the per-role gradient directions: BF16 next to a BF16
// table (accumulated in FP32 by the reducer), else the accumulation type.
template <typename T, typename A> struct DirOf { using type = A; };
template <> struct DirOf<__nv_bfloat16, float> { using type = __nv_bfloat16; };

// FP32 -> BF16 with stochastic rounding: adds uniform 16-bit noise below the
// BF16 mantissa before truncation, so E[bf16(x)] = x and small Adam updates
// are not lost to round-to-nearest.  NaN/Inf pass through unchanged.
__device__ __forceinline__ __nv_bfloat16 bf16_stochastic(float x, uint32_t r16) {
    uint32_t b = __float_as_uint(x);
    if ((b & 0x7f800000u) == 0x7f800000u) return __float2bfloat16_rn(x);
    b += (r16 & 0xffffu);
    b &= 0xffff0000u;
    return __ushort_as_bfloat16((unsigned short)(b >> 16));
}

// The same rounding of an element pair in one instruction: sm_100-family
// stochastic-rounding conversion (PTX cvt.rs.bf16x2.f32).  Returns the pair
// packed as stored (lo in the low half); lo takes rbits[15:0] and hi
// rbits[31:16] as its 16 random bits, so the result equals
// {bf16_stochastic(hi, rbits >> 16), bf16_stochastic(lo, rbits & 0xffff)}
// bit for bit, NaN, infinities and subnormals included
// (ep_selftest_stochastic_rounding checks this on the device).
__device__ __forceinline__ uint32_t bf16x2_stochastic(float lo, float hi, uint32_t rbits) {
    uint32_t d;
    asm("cvt.rs.bf16x2.f32 %0, %1, %2, %3;" : "=r"(d) : "f"(hi), "f"(lo), "r"(rbits));
    return d;
}

}  // namespace ep
