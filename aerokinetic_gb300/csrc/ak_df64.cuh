// ak_df64.cuh -- double-float ("df64") arithmetic for the collision.
//
// A value is hi + lo with two FP32 numbers, |lo| <= ulp(hi) / 2: a 48-bit
// significand evaluated on the FP32 pipe, which GB300 issues 64 times as fast
// as FP64.  The operations are the classical error-free transformations:
// TwoSum (Knuth), FastTwoSum (Dekker) and the FMA-based TwoProd, combined as
// in Joldes, Muller and Popescu, "Tight and rigorous error bounds for basic
// building blocks of double-word arithmetic" (ACM TOMS 44, 2017): the addition
// is the "sloppy" double-word sum, whose error is bounded relative to the
// operands (~2^-47 of the larger), which is what a population update needs;
// products and quotients keep ~2^-46 relative accuracy.  Exponent range is
// FP32's: adequate for populations, densities and velocities of a lattice.
#pragma once
#include <cmath>

namespace ak {

struct df64 {
    float hi, lo;
    df64() = default;
    __host__ __device__ constexpr df64(float h, float l) : hi(h), lo(l) {}
    __host__ __device__ constexpr df64(double d) : hi((float)d), lo((float)(d - (double)(float)d)) {}
    __host__ __device__ constexpr df64(int i) : df64((double)i) {}
    __host__ __device__ explicit operator double() const { return (double)hi + (double)lo; }
};

// storage of a df64 population: one 8-byte word
struct alignas(8) df2 {
    float hi, lo;
};

__host__ __device__ __forceinline__ float df_fma(float a, float b, float c) {
#ifdef __CUDA_ARCH__
    return __fmaf_rn(a, b, c);
#else
    return std::fma(a, b, c);
#endif
}

__host__ __device__ __forceinline__ df64 fast_two_sum(float a, float b) {  // |a| >= |b| or a == 0
    const float s = a + b;
    return df64(s, b - (s - a));
}

__host__ __device__ __forceinline__ df64 two_sum(float a, float b) {
    const float s = a + b, bb = s - a;
    return df64(s, (a - (s - bb)) + (b - bb));
}

__host__ __device__ __forceinline__ df64 operator+(df64 a, df64 b) {
    const df64 s = two_sum(a.hi, b.hi);
    return fast_two_sum(s.hi, s.lo + (a.lo + b.lo));
}
__host__ __device__ __forceinline__ df64 operator-(df64 a) { return df64(-a.hi, -a.lo); }
__host__ __device__ __forceinline__ df64 operator-(df64 a, df64 b) { return a + (-b); }
__host__ __device__ __forceinline__ df64 operator*(df64 a, df64 b) {
    const float p = a.hi * b.hi;
    float e = df_fma(a.hi, b.hi, -p);
    e = df_fma(a.hi, b.lo, df_fma(a.lo, b.hi, e));
    return fast_two_sum(p, e);
}
__host__ __device__ __forceinline__ df64 operator/(df64 a, df64 b) {
    const float q1 = a.hi / b.hi;
    const df64 r = a - b * df64(q1, 0.0f);
    const float q2 = r.hi / b.hi;
    const df64 r2 = r - b * df64(q2, 0.0f);
    return fast_two_sum(q1, q2) + df64(r2.hi / b.hi, 0.0f);
}
__host__ __device__ __forceinline__ df64 &operator+=(df64 &a, df64 b) { return a = a + b; }
__host__ __device__ __forceinline__ df64 &operator-=(df64 &a, df64 b) { return a = a - b; }
__host__ __device__ __forceinline__ df64 &operator*=(df64 &a, df64 b) { return a = a * b; }

}  // namespace ak
