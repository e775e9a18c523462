// common.cuh -- value traits, order-preserving keys and small block primitives shared by
// the sm_103a kernels of the MWU differential-expression backend.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace hpdex {

// Reference enum values (AI4Cell/hpdex src/cpp/include/mannwhitneyu.hpp:24-31).
enum ZeroHandling : int { ZH_NONE = 0, ZH_MIN = 1, ZH_MAX = 2, ZH_MIX = 3 };
enum Alternative : int { ALT_LESS = 0, ALT_GREATER = 1, ALT_TWO_SIDED = 2 };

// ---------------------------------------------------------------------------------------
// Order-preserving keys. The reference compares every value after casting it to double
// (src/cpp/mannwhitneyu.cpp:920); two values tie iff their doubles compare equal. The key
// maps that order onto unsigned integers: floats flip the sign bit (negatives: all bits),
// -0.0 is first canonicalised to +0.0 so that it ties with 0.0, signed integers flip the
// top bit. 64-bit integers go through double so that values above 2^53 collapse exactly
// the way the reference's cast does.
// ---------------------------------------------------------------------------------------
__device__ __forceinline__ uint32_t key_of_f32(float v) {
    uint32_t u = __float_as_uint(v);
    if ((u << 1) == 0u) u = 0u;
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ unsigned long long key_of_f64(double v) {
    uint64_t u = (uint64_t)__double_as_longlong(v);
    if ((u << 1) == 0ull) u = 0ull;
    return (u >> 63) ? ~u : (u | 0x8000000000000000ull);
}

template <class V>
struct Val;

#define HPDEX_SIGNED_SMALL(T)                                                            \
    template <>                                                                          \
    struct Val<T> {                                                                      \
        using Key = uint32_t;                                                            \
        static __device__ __forceinline__ bool finite(T) { return true; }                \
        static __device__ __forceinline__ bool zero(T x) { return x == 0; }              \
        static __device__ __forceinline__ bool neg(T x) { return x < 0; }                \
        static __device__ __forceinline__ Key key(T x) {                                 \
            return (uint32_t)(int32_t)x ^ 0x80000000u;                                   \
        }                                                                                \
        static __device__ __forceinline__ double to_double(T x) { return (double)x; }   \
    };
#define HPDEX_UNSIGNED_SMALL(T)                                                          \
    template <>                                                                          \
    struct Val<T> {                                                                      \
        using Key = uint32_t;                                                            \
        static __device__ __forceinline__ bool finite(T) { return true; }                \
        static __device__ __forceinline__ bool zero(T x) { return x == 0; }              \
        static __device__ __forceinline__ bool neg(T) { return false; }                  \
        static __device__ __forceinline__ Key key(T x) { return (uint32_t)x; }           \
        static __device__ __forceinline__ double to_double(T x) { return (double)x; }   \
    };
HPDEX_SIGNED_SMALL(int8_t)
HPDEX_SIGNED_SMALL(int16_t)
HPDEX_SIGNED_SMALL(int32_t)
HPDEX_UNSIGNED_SMALL(uint8_t)
HPDEX_UNSIGNED_SMALL(uint16_t)
HPDEX_UNSIGNED_SMALL(uint32_t)
#undef HPDEX_SIGNED_SMALL
#undef HPDEX_UNSIGNED_SMALL

template <>
struct Val<float> {
    using Key = uint32_t;
    static __device__ __forceinline__ bool finite(float x) {
        return (__float_as_uint(x) & 0x7f800000u) != 0x7f800000u;
    }
    static __device__ __forceinline__ bool zero(float x) { return x == 0.0f; }
    static __device__ __forceinline__ bool neg(float x) { return x < 0.0f; }
    static __device__ __forceinline__ Key key(float x) { return key_of_f32(x); }
    static __device__ __forceinline__ double to_double(float x) { return (double)x; }
};
template <>
struct Val<double> {
    using Key = unsigned long long;
    static __device__ __forceinline__ bool finite(double x) {
        return ((uint64_t)__double_as_longlong(x) & 0x7ff0000000000000ull) != 0x7ff0000000000000ull;
    }
    static __device__ __forceinline__ bool zero(double x) { return x == 0.0; }
    static __device__ __forceinline__ bool neg(double x) { return x < 0.0; }
    static __device__ __forceinline__ Key key(double x) { return key_of_f64(x); }
    static __device__ __forceinline__ double to_double(double x) { return x; }
};
template <>
struct Val<int64_t> {
    using Key = unsigned long long;
    static __device__ __forceinline__ bool finite(int64_t) { return true; }
    static __device__ __forceinline__ bool zero(int64_t x) { return x == 0; }
    static __device__ __forceinline__ bool neg(int64_t x) { return x < 0; }
    static __device__ __forceinline__ Key key(int64_t x) { return key_of_f64((double)x); }
    static __device__ __forceinline__ double to_double(int64_t x) { return (double)x; }
};
template <>
struct Val<uint64_t> {
    using Key = unsigned long long;
    static __device__ __forceinline__ bool finite(uint64_t) { return true; }
    static __device__ __forceinline__ bool zero(uint64_t x) { return x == 0; }
    static __device__ __forceinline__ bool neg(uint64_t) { return false; }
    static __device__ __forceinline__ Key key(uint64_t x) { return key_of_f64((double)x); }
    static __device__ __forceinline__ double to_double(uint64_t x) { return (double)x; }
};

__device__ __forceinline__ int bit_length(uint32_t x) { return 32 - __clz(x); }
__device__ __forceinline__ int bit_length(unsigned long long x) { return 64 - __clzll((long long)x); }

template <class K>
__device__ __forceinline__ K shfl_xor_key(K v, int m) {
    return __shfl_xor_sync(0xffffffffu, v, m);
}

template <class K>
__device__ __forceinline__ K warp_min(K v) {
#pragma unroll
    for (int m = 16; m > 0; m >>= 1) {
        K o = __shfl_xor_sync(0xffffffffu, v, m);
        v = o < v ? o : v;
    }
    return v;
}
template <class K>
__device__ __forceinline__ K warp_max(K v) {
#pragma unroll
    for (int m = 16; m > 0; m >>= 1) {
        K o = __shfl_xor_sync(0xffffffffu, v, m);
        v = o > v ? o : v;
    }
    return v;
}
__device__ __forceinline__ unsigned long long warp_sum_u64(unsigned long long v) {
#pragma unroll
    for (int m = 16; m > 0; m >>= 1) v += __shfl_xor_sync(0xffffffffu, v, m);
    return v;
}
__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        uint32_t o = __shfl_up_sync(0xffffffffu, v, d);
        if (lane >= d) v += o;
    }
    return v;
}

}  // namespace hpdex
