// ak_lattice.cuh -- D3Q27 stencil, population storage and the cumulant
// collision used by every sm_103a kernel of the engine.
//
// Directions follow lbmpy's D3Q27 order (the reference's pdf[..., d] index).
// The collision is the compressible cumulant operator the reference configures
// (src/aerokinetic/solver.py:75-77, interface.py:124-128): the five deviatoric
// second-order cumulants relax with omega_shear, their trace with omega_bulk,
// and every cumulant of order >= 3 with rate 1 to its zero equilibrium
// (Geier et al. 2015, doi:10.1016/j.camwa.2015.05.001).
//
// With all higher cumulants at zero, the post-collision state is determined by
// rho, u and the relaxed covariance S (= second-order central moments / rho):
// its central moments are Gaussian pairings of S.  Applying the per-axis
// central-moment -> population map (the three-point transform of Geier's
// chimera scheme) to that pairing sum gives eleven separable terms,
//
//   f*(cx,cy,cz)/rho = A(cx,cy) phi_z(cz) + B(cx,cy) psi_z(cz) + C(cx,cy) chi(cz)
//   A = phi_x phi_y + s_xy psi_x psi_y + 2 s_xy^2 chi chi
//   B = s_xz psi_x phi_y + s_yz phi_x psi_y + 2 s_xy (s_xz chi psi_y + s_yz psi_x chi)
//   C = 2 s_xz^2 chi phi_y + 2 s_yz^2 phi_x chi + 2 s_xz s_yz psi_x psi_y + 8 s_xy s_xz s_yz chi chi
//
// with phi_a(c) the 1-D population of mean u_a and variance s_aa, psi_a(c) =
// (u-1/2, -2u, u+1/2) and chi = (1/2, -1, 1/2).  Everything is evaluated as a
// deviation from the rest weights (g = f - w, rho = 1 + drho, s_aa = 1/3 +
// sigma_a), so single precision keeps its relative accuracy on the small
// quantities it stores.
#pragma once
#include <cuda_fp16.h>
#include <stdint.h>

#include "ak_df64.cuh"
#include "ak_f32x2.cuh"

namespace ak {

constexpr int Q = 27;

// lbmpy D3Q27 order.  The tables are packed into 64-bit words at compile
// time (2 bits per velocity component, 5 bits per direction index, 12
// entries per word), so a direction known only at run time (a link's
// direction, a loop that is not unrolled) costs a shift and a mask; a plain
// constexpr array indexed at run time is materialised in local memory.
struct Packed27 {
    uint64_t w[3] = {0, 0, 0};
    int bits = 0;
    __host__ __device__ constexpr int get(int i) const {
        const uint64_t word = i < 12 ? w[0] : (i < 24 ? w[1] : w[2]);
        return (int)((word >> (bits * (i % 12))) & ((1ull << bits) - 1));
    }
};
__host__ __device__ constexpr Packed27 pack27(const int8_t (&t)[27], int offset, int bits) {
    Packed27 p;
    p.bits = bits;
    for (int i = 0; i < 27; ++i) p.w[i / 12] |= (uint64_t)(t[i] + offset) << (bits * (i % 12));
    return p;
}
__host__ __device__ constexpr int cx(int q) {
    constexpr int8_t t[Q] = {0, 0, 0, -1, 1, 0, 0, -1, 1, -1, 1, 0, 0, -1, 1, 0, 0, -1, 1, 1, -1, 1, -1, 1, -1, 1, -1};
    constexpr Packed27 p = pack27(t, 1, 2);
    return p.get(q) - 1;
}
__host__ __device__ constexpr int cy(int q) {
    constexpr int8_t t[Q] = {0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, -1, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1};
    constexpr Packed27 p = pack27(t, 1, 2);
    return p.get(q) - 1;
}
__host__ __device__ constexpr int cz(int q) {
    constexpr int8_t t[Q] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, 1, 1, -1, -1, -1, -1, 1, 1, 1, 1, -1, -1, -1, -1};
    constexpr Packed27 p = pack27(t, 1, 2);
    return p.get(q) - 1;
}
// direction index of (cx, cy, cz) given as (ix, iy, iz) = c + 1
__host__ __device__ constexpr int qof(int ix, int iy, int iz) {
    constexpr int8_t t[27] = {26, 9, 22, 17, 3, 13, 24, 7, 20,   // cx = -1
                              16, 2, 12, 6, 0, 5, 15, 1, 11,     // cx = 0
                              25, 10, 21, 18, 4, 14, 23, 8, 19}; // cx = +1
    constexpr Packed27 p = pack27(t, 0, 5);
    return p.get((ix * 3 + iy) * 3 + iz);
}
__host__ __device__ constexpr int inv(int q) {
    constexpr int8_t t[Q] = {0, 2, 1, 4, 3, 6, 5, 10, 9, 8, 7, 16, 15, 18, 17, 12, 11, 14, 13, 26, 25, 24, 23, 22, 21, 20, 19};
    constexpr Packed27 p = pack27(t, 0, 5);
    return p.get(q);
}
__host__ __device__ constexpr double w1(int i) { return i == 1 ? 2.0 / 3.0 : 1.0 / 6.0; }  // i = c + 1
__host__ __device__ constexpr double weight(int q) {
    return w1(cx(q) + 1) * w1(cy(q) + 1) * w1(cz(q) + 1);
}

// ---------------------------------------------------------------- storage
// Populations are stored shifted, as g = f - w (zero-centred, the reference's
// own representation).  The FP16 form stores (g - a_q) / w_q, where a_q is
// the zero-centred equilibrium of the freestream: a per-direction constant
// shift that makes the stored numbers small deviations from the farfield
// state (so the format's 11-bit significand is spent on the flow's
// departures from it) and scaled by 1/w_q into the same range for every
// direction.  With a zero freestream a_q = 0 and the shift is plain f - w.
template <typename S> struct Store;
// T: the collision's arithmetic; A: the arithmetic of the boundaries and
// the refinement transfers.
template <> struct Store<double> {
    using T = double;
    using A = double;
    static constexpr int MIN_BLOCKS = 4;
    __device__ static __forceinline__ double load(const double *p, int, float) { return __ldg(p); }
    __device__ static __forceinline__ void store(double *p, int, double v, float) { *p = v; }
};
template <> struct Store<float> {
    using T = float;
    using A = float;
    static constexpr int MIN_BLOCKS = 8;
    __device__ static __forceinline__ float load(const float *p, int, float) { return __ldg(p); }
    __device__ static __forceinline__ void store(float *p, int, float v, float) { *p = v; }
};
template <> struct Store<__half> {
    using T = float;
    using A = float;
    static constexpr int MIN_BLOCKS = 8;
    __device__ static __forceinline__ float load(const __half *p, int q, float shift) {
        return fmaf(__half2float(__ldg(p)), (float)weight(q), shift);
    }
    __device__ static __forceinline__ void store(__half *p, int q, float v, float shift) {
        const float inv = (float)(1.0 / weight(q));
        *p = __float2half_rn(fmaf(v, inv, -shift * inv));
    }
};
// df64 form: FP64-sized storage as (hi, lo) float pairs, the collision in
// double-float arithmetic on the FP32 pipe, boundaries and transfers in FP64
template <> struct Store<df2> {
    using T = df64;
    using A = double;
    static constexpr int MIN_BLOCKS = 4;
    __device__ static __forceinline__ df64 load(const df2 *p, int, float) {
        const float2 v = __ldg(reinterpret_cast<const float2 *>(p));
        return df64(v.x, v.y);
    }
    __device__ static __forceinline__ void store(df2 *p, int, df64 v, float) {
        *reinterpret_cast<float2 *>(p) = make_float2(v.hi, v.lo);
    }
};
// the FP16 shift by value, for kernels that index it with compile-time q
struct Shift27 {
    float v[27];
};

// ---------------------------------------------------------------- collision
// a * s for a power of two s (0.5, 2, -2, 4, -1): exact in every form, so the
// double-float form scales both of its words instead of a full product
template <typename T>
__host__ __device__ __forceinline__ T mul_pow2(T a, double s) {
    return a * T(s);
}
template <>
__host__ __device__ __forceinline__ df64 mul_pow2<df64>(df64 a, double s) {
    return df64(a.hi * (float)s, a.lo * (float)s);
}
// FP64 on the device: GB300 issues FP64 at 1/64 of its FP32 rate, and the
// plain collision is bound by that pipe, so the exact scalings run on the
// integer pipe instead: s = +-2^k adds k to the exponent field of the high
// word (and flips the sign for s < 0).  Identical to a * s for every normal
// a with a normal product and for +-0; a subnormal a (|a| < 2^-1022) is
// returned unscaled.  s is a compile-time constant at every call site, so
// the selection below folds away.
template <>
__host__ __device__ __forceinline__ double mul_pow2<double>(double a, double s) {
#ifdef __CUDA_ARCH__
    if (s == -1.0) return -a;  // a sign modifier on the consumer
    const int k = (s == 0.5 || s == -0.5) ? -1 : ((s == 2.0 || s == -2.0) ? 1 : ((s == 4.0 || s == -4.0) ? 2 : 0));
    if (k == 0) return a * s;
    int hi = __double2hiint(a);
    const int lo = __double2loint(a);
    if (hi & 0x7ff00000) hi += k * (1 << 20);  // a normal a: scale; +-0 and subnormals keep their exponent
    if (s < 0) hi ^= (int)0x80000000;
    return __hiloint2double(hi, lo);
#else
    return a * s;
#endif
}

// Smagorinsky subgrid model (sgs="smagorinsky", solver.py:74-77; Hou,
// Sterling, Chen & Doolen 1996 in lattice units): with the non-equilibrium
// second moments Pi_ab = K_ab - rho/3 delta_ab (K the central moments) and
// |Pi| = sqrt(2 Pi:Pi) / rho, the cell's shear rate is
// 2 / (tau0 + sqrt(tau0^2 + 18 C^2 |Pi|)), tau0 = 1/omega the molecular
// relaxation time.  c18 = 18 C^2; c18 = 0 keeps the molecular rate.  The
// double-float form evaluates the rate in FP64 (a few operations per cell).
template <typename T> struct SgsReal { using type = T; };
template <> struct SgsReal<df64> { using type = double; };
template <> struct SgsReal<F2> { using type = float; };
template <typename T>
struct Sgs {
    typename SgsReal<T>::type tau0 = 0, c18 = 0;
};
template <typename T>
__host__ __device__ __forceinline__ T smagorinsky_rate(const Sgs<T> &m, T rinv, T pxx, T pyy, T pzz, T pxy, T pxz,
                                                      T pyz) {
    using R = typename SgsReal<T>::type;
    const R a = R(pxx), b = R(pyy), c = R(pzz), d = R(pxy), e = R(pxz), f = R(pyz);
    const R ss = (a * a + b * b + c * c) + R(2) * (d * d + e * e + f * f);
    const R norm = sqrt(R(2) * ss) * R(rinv);
    return T(R(2) / (m.tau0 + sqrt(m.c18 * norm + m.tau0 * m.tau0)));
}

// mac (optional): the cell's (drho, jx, jy, jz), which the collision
// conserves; a null mac compiles away.
// the subgrid rate of a pair of cells, lane by lane in FP32
__device__ __forceinline__ F2 smagorinsky_rate(const Sgs<F2> &m, F2 rinv, F2 pxx, F2 pyy, F2 pzz, F2 pxy, F2 pxz,
                                               F2 pyz) {
    const Sgs<float> s{m.tau0, m.c18};
    return F2(make_float2(smagorinsky_rate<float>(s, rinv.v.x, pxx.v.x, pyy.v.x, pzz.v.x, pxy.v.x, pxz.v.x, pyz.v.x),
                          smagorinsky_rate<float>(s, rinv.v.y, pxx.v.y, pyy.v.y, pzz.v.y, pxy.v.y, pxz.v.y, pyz.v.y)));
}

template <typename T>
__host__ __device__ __forceinline__ void collide(T g[Q], T omega_s, T omega_b, const Sgs<T> &sgs = Sgs<T>{},
                                                 T *mac = nullptr) {
    // raw moments of g up to second order through partial line sums
    T Z0[3][3], Z1[3][3], Z2[3][3];
#pragma unroll
    for (int ix = 0; ix < 3; ++ix)
#pragma unroll
        for (int iy = 0; iy < 3; ++iy) {
            const T a = g[qof(ix, iy, 0)], b = g[qof(ix, iy, 1)], c = g[qof(ix, iy, 2)];
            Z1[ix][iy] = c - a;
            Z2[ix][iy] = c + a;
            Z0[ix][iy] = Z2[ix][iy] + b;
        }
    T Y00[3], Y01[3], Y02[3], Y10[3], Y11[3], Y20[3];
#pragma unroll
    for (int ix = 0; ix < 3; ++ix) {
        Y01[ix] = Z0[ix][2] - Z0[ix][0];
        Y02[ix] = Z0[ix][2] + Z0[ix][0];
        Y00[ix] = Y02[ix] + Z0[ix][1];
        Y11[ix] = Z1[ix][2] - Z1[ix][0];
        Y10[ix] = Z1[ix][0] + Z1[ix][1] + Z1[ix][2];
        Y20[ix] = Z2[ix][0] + Z2[ix][1] + Z2[ix][2];
    }
    const T M200 = Y00[2] + Y00[0];
    const T drho = M200 + Y00[1];
    const T jx = Y00[2] - Y00[0];
    const T jy = Y01[0] + Y01[1] + Y01[2];
    const T M110 = Y01[2] - Y01[0];
    const T M020 = Y02[0] + Y02[1] + Y02[2];
    const T jz = Y10[0] + Y10[1] + Y10[2];
    const T M101 = Y10[2] - Y10[0];
    const T M011 = Y11[0] + Y11[1] + Y11[2];
    const T M002 = Y20[0] + Y20[1] + Y20[2];

    const T rho = T(1) + drho;
    const T rinv = T(1) / rho;
    const T ux = jx * rinv, uy = jy * rinv, uz = jz * rinv;
    if (mac) {
        mac[0] = drho;
        mac[1] = jx;
        mac[2] = jy;
        mac[3] = jz;
    }
    // second-order central moments minus their rest value 1/3
    const T kdx = M200 - jx * ux, kdy = M020 - jy * uy, kdz = M002 - jz * uz;
    const T kxy = M110 - jx * uy, kxz = M101 - jx * uz, kyz = M011 - jy * uz;
    const T third = T(1) / T(3);
    const T d3 = drho * third;
    const T om1 = T(1) - (sgs.c18 > 0 ? smagorinsky_rate(sgs, rinv, kdx - d3, kdy - d3, kdz - d3, kxy, kxz, kyz)
                                      : omega_s);
    const T P1 = om1 * (kdx - kdy), P2 = om1 * (kdx - kdz);
    const T S = kdx + kdy + kdz;
    const T tr = S + omega_b * (drho - S);
    const T kx = (P1 + P2 + tr) * third;
    const T ky = kx - P1, kz = kx - P2;
    const T sig[3] = {(kx - d3) * rinv, (ky - d3) * rinv, (kz - d3) * rinv};
    const T sxy = om1 * kxy * rinv, sxz = om1 * kxz * rinv, syz = om1 * kyz * rinv;
    const T u[3] = {ux, uy, uz};

    T dphi[3][3], phi[3][3], psi[3][3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const T t = u[a] * u[a] + sig[a];
        const T h = T(0.5) * t, hu = T(0.5) * u[a];
        dphi[a][0] = h - hu;
        dphi[a][1] = -t;
        dphi[a][2] = h + hu;
        phi[a][0] = T(1.0 / 6.0) + dphi[a][0];
        phi[a][1] = T(2.0 / 3.0) + dphi[a][1];
        phi[a][2] = T(1.0 / 6.0) + dphi[a][2];
        psi[a][0] = u[a] - T(0.5);
        psi[a][1] = T(-2) * u[a];
        psi[a][2] = u[a] + T(0.5);
    }
    const T chi[3] = {T(0.5), T(-1), T(0.5)};
    const T sxy2 = T(2) * sxy * sxy, sxz2 = T(2) * sxz * sxz, syz2 = T(2) * syz * syz;
    const T bxz = T(2) * sxy * sxz, byz = T(2) * sxy * syz, cxz = T(2) * sxz * syz;
    const T c8 = T(4) * bxz * syz;  // 8 s_xy s_xz s_yz
#pragma unroll
    for (int ix = 0; ix < 3; ++ix)
#pragma unroll
        for (int iy = 0; iy < 3; ++iy) {
            const T A0 = T(w1(ix) * w1(iy));
            const T dA = dphi[0][ix] * phi[1][iy] + T(w1(ix)) * dphi[1][iy] + sxy * psi[0][ix] * psi[1][iy] +
                         sxy2 * (chi[ix] * chi[iy]);
            const T B = sxz * psi[0][ix] * phi[1][iy] + syz * phi[0][ix] * psi[1][iy] +
                        bxz * chi[ix] * psi[1][iy] + byz * psi[0][ix] * chi[iy];
            const T C = sxz2 * chi[ix] * phi[1][iy] + syz2 * phi[0][ix] * chi[iy] + cxz * psi[0][ix] * psi[1][iy] +
                        c8 * (chi[ix] * chi[iy]);
            const T rA = rho * dA, rB = rho * B, rC = rho * C, rA0 = rho * A0, dA0 = drho * A0;
#pragma unroll
            for (int iz = 0; iz < 3; ++iz)
                g[qof(ix, iy, iz)] = dA0 * T(w1(iz)) + rA0 * dphi[2][iz] + rA * phi[2][iz] + rB * psi[2][iz] +
                                     rC * chi[iz];
        }
}

// The ten moments the collision needs, m = (drho, jx, jy, jz, M200, M020,
// M002, M110, M101, M011), from 27 values by the chimera sums along z, then
// y, then x (66 additions).
template <typename V>
__host__ __device__ __forceinline__ void chimera_sums(const V f[Q], V m[10]) {
    V Z0[3][3], Z1[3][3], Z2[3][3];
#pragma unroll
    for (int ix = 0; ix < 3; ++ix)
#pragma unroll
        for (int iy = 0; iy < 3; ++iy) {
            const V a = f[qof(ix, iy, 0)], b = f[qof(ix, iy, 1)], c = f[qof(ix, iy, 2)];
            Z1[ix][iy] = c - a;
            Z2[ix][iy] = c + a;
            Z0[ix][iy] = Z2[ix][iy] + b;
        }
    V Y00[3], Y01[3], Y02[3], Y10[3], Y11[3], Y20[3];
#pragma unroll
    for (int ix = 0; ix < 3; ++ix) {
        Y01[ix] = Z0[ix][2] - Z0[ix][0];
        Y02[ix] = Z0[ix][2] + Z0[ix][0];
        Y00[ix] = Y02[ix] + Z0[ix][1];
        Y11[ix] = Z1[ix][2] - Z1[ix][0];
        Y10[ix] = Z1[ix][0] + Z1[ix][1] + Z1[ix][2];
        Y20[ix] = Z2[ix][0] + Z2[ix][1] + Z2[ix][2];
    }
    m[4] = Y00[2] + Y00[0];
    m[0] = m[4] + Y00[1];
    m[1] = Y00[2] - Y00[0];
    m[2] = Y01[0] + Y01[1] + Y01[2];
    m[7] = Y01[2] - Y01[0];
    m[5] = Y02[0] + Y02[1] + Y02[2];
    m[3] = Y10[0] + Y10[1] + Y10[2];
    m[8] = Y10[2] - Y10[0];
    m[9] = Y11[0] + Y11[1] + Y11[2];
    m[6] = Y20[0] + Y20[1] + Y20[2];
}

// The plain FP64 form's forward sums on the integer pipe.  GB300 issues
// FP64 at 1/64 of its FP32 rate and the plain collision is bound by that
// pipe, while its integer pipe idles; the 66 additions are exact on
// integers, so each zero-centred population becomes round(g 2^52) (integer
// instructions on its bit pattern), the sums run on 64-bit integers, and
// each of the ten moments is rounded back to double once (integer
// instructions again).  Each population is rounded to a multiple of 2^-52
// (half a unit in the last place of a value near 1) instead of every partial
// sum being rounded.  |g| < 64 keeps every sum inside 63 bits; a population
// of magnitude 64 or more, or a non-finite one, belongs to a state that has
// diverged (the density alone would be 64 times the reference) and makes
// the moments NaN, as a non-finite population does in FP64 sums.
namespace fixsum {
constexpr int BITS = 52;
__device__ __forceinline__ long long from_double(double v, bool &ok) {
    const long long b = __double_as_longlong(v);
    const int e = (int)((b >> 52) & 0x7ff);  // v = m 2^(e - 1075)
    ok &= e <= 1028;                          // |v| < 2^6
    long long r = 0;
    if (e != 0) {
        const long long m = (b & 0x000fffffffffffffLL) | 0x0010000000000000LL;
        const int sh = e - 1075 + BITS;
        if (sh >= 0)
            r = m << (sh < 5 ? sh : 5);
        else if (sh > -54)
            r = (m + (1LL << (-sh - 1))) >> -sh;  // magnitude rounded half up
    }
    return b < 0 ? -r : r;
}
// v 2^-52 as the nearest double (ties away from zero)
__device__ __forceinline__ double to_double(long long v) {
    if (v == 0) return 0.0;
    const unsigned long long a = v < 0 ? 0ULL - (unsigned long long)v : (unsigned long long)v;
    int top = 63 - __clzll((long long)a);  // a in [2^top, 2^(top + 1))
    unsigned long long mant;
    if (top <= 52) {
        mant = a << (52 - top);
    } else {
        const int d = top - 52;
        mant = (a >> d) + ((a >> (d - 1)) & 1ULL);
        if (mant >> 53) {
            mant >>= 1;
            ++top;
        }
    }
    // a 2^-52 = (mant 2^-52) 2^(top - 52): biased exponent top - 52 + 1023
    const unsigned long long bits = ((unsigned long long)(top + 971) << 52) | (mant & 0x000fffffffffffffULL) |
                                    (v < 0 ? 0x8000000000000000ULL : 0ULL);
    return __longlong_as_double((long long)bits);
}
}  // namespace fixsum

template <typename T>
__host__ __device__ __forceinline__ void forward_moments(const T g[Q], T m[10]) {
    chimera_sums<T>(g, m);
}
template <>
__host__ __device__ __forceinline__ void forward_moments<double>(const double g[Q], double m[10]) {
#ifdef __CUDA_ARCH__
    long long f[Q], s[10];
    bool ok = true;
#pragma unroll
    for (int q = 0; q < Q; ++q) f[q] = fixsum::from_double(g[q], ok);
    chimera_sums<long long>(f, s);
#pragma unroll
    for (int k = 0; k < 10; ++k) m[k] = ok ? fixsum::to_double(s[k]) : __longlong_as_double(0x7ff8000000000000LL);
#else
    chimera_sums<double>(g, m);
#endif
}

// Plain FP64 form.  The same operator with the fewest double-precision
// operations (the FP64 pipe bounds this kernel on GB300): populations f = g + w
// are formed directly, and the three per-axis expansions are factored as
// chimera passes that share their coefficients,
//   X(+-) = E_X +- D_X,  X(0) = (1 - t) X_phi - 2u X_psi - X_chi,
// first along x for A, B, C of every c_y, then along z with rho folded into
// the z-functions.  The forward sums (66 of the 450 operations) run on the
// integer pipe on the device (forward_moments<double>): ncu counted 277 FP64
// instructions per cell with FP64 sums (156 FMA, 87 add, 34 multiply), and
// the two-level coarse pass went from 0.776 to 0.586 ms with integer sums.
template <typename T>
__host__ __device__ __forceinline__ void collide_full(T g[Q], T om1, T omega_b, const Sgs<T> &sgs = Sgs<T>{},
                                                      T *mac = nullptr) {
    T mom[10];
    forward_moments(g, mom);
    const T drho = mom[0], jx = mom[1], jy = mom[2], jz = mom[3];
    const T M200 = mom[4], M020 = mom[5], M002 = mom[6], M110 = mom[7], M101 = mom[8], M011 = mom[9];

    const T rho = T(1) + drho;
    const T rinv = T(1) / rho;
    const T ux = jx * rinv, uy = jy * rinv, uz = jz * rinv;
    if (mac) {
        mac[0] = drho;
        mac[1] = jx;
        mac[2] = jy;
        mac[3] = jz;
    }
    // second-order central moments minus 1/3, relaxed
    const T kdx = M200 - jx * ux, kdy = M020 - jy * uy, kdz = M002 - jz * uz;
    const T third = T(1.0 / 3.0);
    if (sgs.c18 > 0) {
        const T d3 = drho * third;
        om1 = T(1) - smagorinsky_rate(sgs, rinv, kdx - d3, kdy - d3, kdz - d3, M110 - jx * uy, M101 - jx * uz,
                                      M011 - jy * uz);
    }
    const T P1 = om1 * (kdx - kdy), P2 = om1 * (kdx - kdz);
    const T S = kdx + kdy + kdz;
    const T kx = (P1 + P2 + (S + omega_b * (drho - S))) * third;
    // normalised covariance: s_aa = (1/3 + k_a) / rho; t_a = u_a^2 + s_aa
    const T r3 = third * rinv;
    const T tx = ux * ux + (r3 + kx * rinv);
    const T ty = uy * uy + (r3 + (kx - P1) * rinv);
    const T tz = uz * uz + (r3 + (kx - P2) * rinv);
    const T omr = om1 * rinv;
    const T sxy = (M110 - jx * uy) * omr, sxz = (M101 - jx * uz) * omr, syz = (M011 - jy * uz) * omr;
    // coefficient products
    const T s2xy = mul_pow2(sxy, 2.0), s2xz = mul_pow2(sxz, 2.0), s2yz = mul_pow2(syz, 2.0);
    const T kAchi = s2xy * sxy;        // 2 sxy^2
    const T kBpsi = s2xy * syz;        // 2 sxy syz
    const T kBchi = s2xy * sxz;        // 2 sxy sxz
    const T kCphi = s2yz * syz;        // 2 syz^2
    const T kCpsi = s2xz * syz;        // 2 sxz syz
    const T kCchi = s2xz * sxz;        // 2 sxz^2
    const T k8 = mul_pow2(kBchi, 4.0) * syz;   // 8 sxy sxz syz
    // y-functions
    const T phy[3] = {mul_pow2(ty - uy, 0.5), T(1) - ty, mul_pow2(ty + uy, 0.5)};
    const T psy[3] = {uy - T(0.5), mul_pow2(uy, -2.0), uy + T(0.5)};
    constexpr double chy[3] = {0.5, -1.0, 0.5};
    // x-functions: phi_x(+-1) = (t_x +- u_x) / 2, psi_x(+-1) = u_x +- 1/2
    const T htx = mul_pow2(tx, 0.5), hux = mul_pow2(ux, 0.5), omtx = T(1) - tx, m2ux = mul_pow2(ux, -2.0);
    const T px2 = htx + hux, px0 = htx - hux, sx2 = ux + T(0.5), sx0 = ux - T(0.5);
    // rho-scaled z-functions, the c_z = +1 and -1 rows as sums and differences
    const T rh = mul_pow2(rho, 0.5), rhtz = rh * tz, rhuz = rh * uz;
    const T r0z = rho * (T(1) - tz), rm2uz = mul_pow2(rho, -2.0) * uz, ruz = rho * uz;
    const T pz2 = rhtz + rhuz, pz0 = rhtz - rhuz, qz2 = ruz + rh, qz0 = ruz - rh;
#pragma unroll
    for (int iy = 0; iy < 3; ++iy) {
        // coefficients of phi_x, psi_x, chi_x in A, B, C for this c_y
        const T Ap = phy[iy], As = sxy * psy[iy], Ac = mul_pow2(kAchi, chy[iy]);
        const T Bp = syz * psy[iy], Bs = sxz * phy[iy] + mul_pow2(kBpsi, chy[iy]), Bc = kBchi * psy[iy];
        const T Cp = mul_pow2(kCphi, chy[iy]), Cs = kCpsi * psy[iy], Cc = kCchi * phy[iy] + mul_pow2(k8, chy[iy]);
        T A[3], B[3], C[3];
        {
            const T hc = mul_pow2(Ac, 0.5);
            A[2] = px2 * Ap + (sx2 * As + hc); A[0] = px0 * Ap + (sx0 * As + hc); A[1] = omtx * Ap + (m2ux * As - Ac);
        }
        {
            const T hc = mul_pow2(Bc, 0.5);
            B[2] = px2 * Bp + (sx2 * Bs + hc); B[0] = px0 * Bp + (sx0 * Bs + hc); B[1] = omtx * Bp + (m2ux * Bs - Bc);
        }
        {
            const T hc = mul_pow2(Cc, 0.5);
            C[2] = px2 * Cp + (sx2 * Cs + hc); C[0] = px0 * Cp + (sx0 * Cs + hc); C[1] = omtx * Cp + (m2ux * Cs - Cc);
        }
        // the rest weights (equal for c_z = -1 and +1) enter the fused
        // multiply-add chains as their first addend
#pragma unroll
        for (int ix = 0; ix < 3; ++ix) {
            const T w_pm = T(weight(qof(ix, iy, 2))), w_0 = T(weight(qof(ix, iy, 1)));
            const T cw = C[ix] * rh - w_pm;
            g[qof(ix, iy, 2)] = A[ix] * pz2 + (B[ix] * qz2 + cw);
            g[qof(ix, iy, 0)] = A[ix] * pz0 + (B[ix] * qz0 + cw);
            g[qof(ix, iy, 1)] = A[ix] * r0z + (B[ix] * rm2uz - (C[ix] * rho + w_0));
        }
    }
}

// The collision form of a storage type: the chimera form (fewest operations)
// for FP64 and for FP16 storage, whose quantisation (~1e-5 of a population)
// dominates the FP32 rounding of populations near their rest weight; the
// deviation form for FP32 storage, which keeps FP32's relative accuracy on
// the small deviations it stores.
template <typename S>
__host__ __device__ __forceinline__ void collide_stored(typename Store<S>::T g[Q], typename Store<S>::T omega_s,
                                                        typename Store<S>::T omega_b,
                                                        const Sgs<typename Store<S>::T> &sgs = {},
                                                        typename Store<S>::T *mac = nullptr) {
    using T = typename Store<S>::T;
    if constexpr (sizeof(S) == sizeof(float))
        collide<T>(g, omega_s, omega_b, sgs, mac);
    else
        collide_full<T>(g, T(1) - omega_s, omega_b, sgs, mac);
}

}  // namespace ak
