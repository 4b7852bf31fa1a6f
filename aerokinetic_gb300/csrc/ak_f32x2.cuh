// ak_f32x2.cuh -- two lattice cells per thread in Blackwell's packed FP32x2
// arithmetic.
//
// sm_100-family GPUs execute FP32 additions, multiplications and fused
// multiply-adds on a pair of values in one instruction (__fadd2_rn,
// __fmul2_rn, __ffma2_rn).  The FP32-compute stream-collide is bound by
// instruction issue, not by bytes, so evaluating the collision of two
// x-adjacent cells as one stream of packed instructions halves its
// arithmetic issue slots.  F2 is the collision templates' number type for
// that: each lane is one cell, and every operation rounds exactly as the
// scalar FP32 operation on that lane would.  A product stays unevaluated
// (P2) until it is added, so a * b + c compiles to one fused multiply-add,
// as the scalar code's contraction does; a product used any other way is
// rounded first.
#pragma once
#include <cuda_runtime.h>

namespace ak {

// the packed instructions exist from sm_100 on; a translation unit compiled
// for an older device (a host-side test program) gets per-lane operations
// with the same rounding
#if !defined(__CUDA_ARCH__) || __CUDA_ARCH__ >= 1000
__device__ __forceinline__ float2 f2_fma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 f2_add(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 f2_mul(float2 a, float2 b) { return __fmul2_rn(a, b); }
// a - b as one packed subtraction (PTX sub.rn.f32x2): the same rounding as
// a + (-b), without negating b first
__device__ __forceinline__ float2 f2_sub(float2 a, float2 b) {
    float2 d;
    asm("{\n\t.reg .b64 ra, rb, rd;\n\t"
        "mov.b64 ra, {%2, %3};\n\t"
        "mov.b64 rb, {%4, %5};\n\t"
        "sub.rn.f32x2 rd, ra, rb;\n\t"
        "mov.b64 {%0, %1}, rd;\n\t}"
        : "=f"(d.x), "=f"(d.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return d;
}
#else
__device__ __forceinline__ float2 f2_fma(float2 a, float2 b, float2 c) {
    return make_float2(__fmaf_rn(a.x, b.x, c.x), __fmaf_rn(a.y, b.y, c.y));
}
__device__ __forceinline__ float2 f2_add(float2 a, float2 b) { return make_float2(__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y)); }
__device__ __forceinline__ float2 f2_mul(float2 a, float2 b) { return make_float2(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)); }
__device__ __forceinline__ float2 f2_sub(float2 a, float2 b) { return make_float2(__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y)); }
#endif

struct F2 {
    float2 v;
    F2() = default;
    __host__ __device__ __forceinline__ F2(float2 x) : v(x) {}
    __host__ __device__ __forceinline__ explicit F2(float s) : v(make_float2(s, s)) {}
    __host__ __device__ __forceinline__ explicit F2(double s) : v(make_float2((float)s, (float)s)) {}
    __host__ __device__ __forceinline__ explicit F2(int s) : v(make_float2((float)s, (float)s)) {}
};

__device__ __forceinline__ float2 neg2(float2 a) { return make_float2(-a.x, -a.y); }

// an unevaluated product a * b
struct P2 {
    float2 a, b;
    __device__ __forceinline__ operator F2() const { return F2(f2_mul(a, b)); }
};

__device__ __forceinline__ P2 operator*(F2 a, F2 b) { return P2{a.v, b.v}; }
__device__ __forceinline__ P2 operator*(P2 a, F2 b) { return P2{F2(a).v, b.v}; }
__device__ __forceinline__ P2 operator*(F2 a, P2 b) { return P2{a.v, F2(b).v}; }
__device__ __forceinline__ P2 operator*(P2 a, P2 b) { return P2{F2(a).v, F2(b).v}; }

__device__ __forceinline__ F2 operator+(F2 a, F2 b) { return F2(f2_add(a.v, b.v)); }
__device__ __forceinline__ F2 operator-(F2 a, F2 b) { return F2(f2_sub(a.v, b.v)); }
__device__ __forceinline__ F2 operator-(F2 a) { return F2(neg2(a.v)); }
__device__ __forceinline__ P2 operator-(P2 p) { return P2{neg2(p.a), p.b}; }

__device__ __forceinline__ F2 operator+(P2 p, F2 c) { return F2(f2_fma(p.a, p.b, c.v)); }
__device__ __forceinline__ F2 operator+(F2 c, P2 p) { return F2(f2_fma(p.a, p.b, c.v)); }
__device__ __forceinline__ F2 operator-(P2 p, F2 c) { return F2(f2_fma(p.a, p.b, neg2(c.v))); }
__device__ __forceinline__ F2 operator-(F2 c, P2 p) { return F2(f2_fma(neg2(p.a), p.b, c.v)); }
__device__ __forceinline__ F2 operator+(P2 p, P2 q) { return F2(f2_fma(p.a, p.b, F2(q).v)); }
__device__ __forceinline__ F2 operator-(P2 p, P2 q) { return F2(f2_fma(p.a, p.b, neg2(F2(q).v))); }

__device__ __forceinline__ F2 operator/(F2 a, F2 b) { return F2(make_float2(a.v.x / b.v.x, a.v.y / b.v.y)); }
__device__ __forceinline__ F2 operator/(P2 a, F2 b) { return F2(a) / b; }

__device__ __forceinline__ F2 &operator+=(F2 &a, F2 b) { return a = a + b; }
__device__ __forceinline__ F2 &operator+=(F2 &a, P2 b) { return a = a + b; }
__device__ __forceinline__ F2 &operator-=(F2 &a, F2 b) { return a = a - b; }
__device__ __forceinline__ F2 &operator*=(F2 &a, F2 b) { return a = F2(a * b); }

}  // namespace ak
