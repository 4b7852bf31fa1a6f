// ak_peaks.cuh -- arithmetic ceilings of the engine's kernels on the device
// they run on.
//
// GB300 issues FP64 at a small fraction of its FP32 rate, so the plain FP64
// stream-collide is bound by the FP64 pipe, not by HBM.  Two measurements
// state that bound:
//   * k_fma_peak: dependent fused multiply-add chains (eight per thread, so
//     the pipe, not the latency, limits them) over a grid of every SM's
//     worth of blocks, timed with CUDA events: the device's FMA throughput
//     in FP64 or FP32 (two FLOPs per FMA);
//   * the collision's algorithmic FLOPs per cell: the same __host__ __device__
//     collision templates instantiated on a host number type that counts its
//     additions, multiplications and divisions (a fused multiply-add in the
//     compiled kernel is one multiplication and one addition here).
#pragma once
#include <cmath>

#include "ak_lattice.cuh"

namespace ak {

template <typename T>
__global__ void __launch_bounds__(256) k_fma_peak(T *__restrict__ out, int iters, T a, T b) {
    T x[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = T(threadIdx.x + k) * T(1e-3);
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 8; ++k) x[k] = fma(x[k], a, b);
    }
    T s = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) s += x[k];
    // never true (the chains converge to b / (1 - a) = 1): keeps the work
    if (s == T(-1)) out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// the same chains in packed FP32x2 fused multiply-adds (two FMAs per
// instruction and lane): eight float2 chains per thread
__global__ void __launch_bounds__(256) k_fma2_peak(float *__restrict__ out, int iters, float a, float b) {
    float2 x[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = make_float2((threadIdx.x + k) * 1e-3f, (threadIdx.x + 2 * k) * 1e-3f);
    const float2 a2 = make_float2(a, a), b2 = make_float2(b, b);
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 8; ++k) x[k] = f2_fma(x[k], a2, b2);
    }
    float s = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) s += x[k].x + x[k].y;
    if (s == -1.0f) out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// Host number type that counts the arithmetic applied to it.
struct Counted {
    double v = 0;
    Counted() = default;
    Counted(double x) : v(x) {}  // NOLINT: literals and weights convert implicitly
    static long long adds, muls, divs, sqrts;
    static void reset() { adds = muls = divs = sqrts = 0; }
};
inline long long Counted::adds = 0, Counted::muls = 0, Counted::divs = 0, Counted::sqrts = 0;
inline Counted operator+(Counted a, Counted b) { ++Counted::adds; return Counted(a.v + b.v); }
inline Counted operator-(Counted a, Counted b) { ++Counted::adds; return Counted(a.v - b.v); }
inline Counted operator*(Counted a, Counted b) { ++Counted::muls; return Counted(a.v * b.v); }
inline Counted operator/(Counted a, Counted b) { ++Counted::divs; return Counted(a.v / b.v); }
inline Counted operator-(Counted a) { return Counted(-a.v); }  // a sign flip, folded into its consumer
inline Counted &operator+=(Counted &a, Counted b) { return a = a + b; }
inline Counted &operator-=(Counted &a, Counted b) { return a = a - b; }
inline Counted &operator*=(Counted &a, Counted b) { return a = a * b; }
inline bool operator>(Counted a, Counted b) { return a.v > b.v; }
inline bool operator<(Counted a, Counted b) { return a.v < b.v; }
inline Counted sqrt(Counted a) { ++Counted::sqrts; return Counted(std::sqrt(a.v)); }

}  // namespace ak
