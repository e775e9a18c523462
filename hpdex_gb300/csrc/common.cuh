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

// inverses of the two float keys (the value of the double, -0.0 read back as +0.0)
__device__ __forceinline__ float f32_of_key(uint32_t k) {
    return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}
__device__ __forceinline__ double f64_of_key(unsigned long long k) {
    return __longlong_as_double((long long)((k >> 63) ? (k & 0x7fffffffffffffffull) : ~k));
}

// Value traits: finite / zero / negative as the reference tests them, the order key, the
// double the reference compares, small_int (an integer of magnitude below 2^31: such values
// can be counted in integer bins) and the value back from a key.
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
        static __device__ __forceinline__ bool small_int(T) { return true; }             \
        static __device__ __forceinline__ double from_key(Key k) {                       \
            return (double)(int32_t)(k ^ 0x80000000u);                                   \
        }                                                                                \
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
        static __device__ __forceinline__ bool small_int(T x) { return x < 0x80000000u; } \
        static __device__ __forceinline__ double from_key(Key k) { return (double)k; }   \
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
    static __device__ __forceinline__ bool small_int(float x) {
        return fabsf(x) < 2147483648.0f && x == truncf(x);
    }
    static __device__ __forceinline__ double from_key(Key k) { return (double)f32_of_key(k); }
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
    static __device__ __forceinline__ bool small_int(double x) {
        return fabs(x) < 2147483648.0 && x == trunc(x);
    }
    static __device__ __forceinline__ double from_key(Key k) { return f64_of_key(k); }
};
template <>
struct Val<int64_t> {
    using Key = unsigned long long;
    static __device__ __forceinline__ bool finite(int64_t) { return true; }
    static __device__ __forceinline__ bool zero(int64_t x) { return x == 0; }
    static __device__ __forceinline__ bool neg(int64_t x) { return x < 0; }
    static __device__ __forceinline__ Key key(int64_t x) { return key_of_f64((double)x); }
    static __device__ __forceinline__ double to_double(int64_t x) { return (double)x; }
    static __device__ __forceinline__ bool small_int(int64_t x) {
        return x > -2147483648ll && x < 2147483648ll;
    }
    static __device__ __forceinline__ double from_key(Key k) { return f64_of_key(k); }
};
template <>
struct Val<uint64_t> {
    using Key = unsigned long long;
    static __device__ __forceinline__ bool finite(uint64_t) { return true; }
    static __device__ __forceinline__ bool zero(uint64_t x) { return x == 0; }
    static __device__ __forceinline__ bool neg(uint64_t) { return false; }
    static __device__ __forceinline__ Key key(uint64_t x) { return key_of_f64((double)x); }
    static __device__ __forceinline__ double to_double(uint64_t x) { return (double)x; }
    static __device__ __forceinline__ bool small_int(uint64_t x) { return x < 2147483648ull; }
    static __device__ __forceinline__ double from_key(Key k) { return f64_of_key(k); }
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
